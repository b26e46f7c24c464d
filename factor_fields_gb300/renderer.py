"""Renderer surface: render_ray (renderer.py:8-27), the colour heads, the occupancy mask and
FactorFields.forward (models/FactorFields.py:843-898) for bounded scenes."""
import torch

from .config import Cfg


class SHRender(torch.nn.Module):
    """Degree-2 spherical-harmonics colour head: rgb = sigmoid(eval_sh(2, feat.view(-1, 3, 9), dirs))
    (models/sh.py:34-64 composed as the reference's renderModule). No parameters."""

    def __init__(self, in_channels=27):
        super().__init__()
        # A field fitted without rendering (e.g. an SDF with out_dim = 1) still owns a head, as
        # in the reference; the channel count is checked when rays are rendered.
        self.in_channels = in_channels


class AlphaGridMask(torch.nn.Module):
    """models/FactorFields.py:91-110: a 0/1 occupancy volume over an aabb."""

    def __init__(self, device, aabb, alpha_volume):
        super().__init__()
        self.device = device
        self.aabb = aabb.to(device)
        self.aabbSize = self.aabb[1] - self.aabb[0]
        self.invgridSize = 1.0 / self.aabbSize * 2
        self.alpha_volume = alpha_volume.view(1, 1, *alpha_volume.shape[-3:])
        self.gridSize = torch.tensor([alpha_volume.shape[-1], alpha_volume.shape[-2], alpha_volume.shape[-3]],
                                     dtype=torch.long, device=device)


def make_render_module(cfg, in_channels):
    shading = (cfg.renderer or Cfg()).get("shadingMode", "SH")
    if shading == "SH":
        return SHRender(in_channels)
    raise NotImplementedError(f"renderer.shadingMode {shading!r} is not implemented (use 'SH')")


def render_forward(model, rays_chunk, white_bg=True, is_train=False, ndc_ray=False, N_samples=-1):
    raise NotImplementedError("ray rendering is not built yet")
