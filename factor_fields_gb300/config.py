"""Configuration objects and the derivation of a field's sizes from its config.

Key names follow the reference's OmegaConf configs (configs/defaults.yaml:12-33,
configs/nerf.yaml:73-92); Cfg is a dict with attribute access so a reference config (or an
OmegaConf object converted with to_container) can be passed straight in.
"""
import copy

import numpy as np
import torch


class Cfg(dict):
    """dict with attribute access; missing keys read as None (like the reference's usage)."""

    def __getattr__(self, k):
        return self.get(k)

    def __setattr__(self, k, v):
        self[k] = v

    def __deepcopy__(self, memo):
        return Cfg({k: copy.deepcopy(v, memo) for k, v in self.items()})


def make_cfg(d):
    if isinstance(d, Cfg):
        return d
    if isinstance(d, dict):
        return Cfg({k: make_cfg(v) for k, v in d.items()})
    return d


DEFAULTS = {
    "defaults": {"mode": "reconstruction"},
    "model": {"coeff_type": "grid", "basis_type": "grid", "basis_mapping": "sawtooth",
              "basis_dims": [4, 4, 4, 2, 2, 2], "basis_resos": [32, 51, 70, 89, 108, 128],
              "freq_bands": [2.0, 3.2, 4.4, 5.6, 6.8, 8.0], "coeff_reso": 32, "total_params": 5308416,
              "T_basis": 0, "T_coeff": 0, "coef_init": 1.0, "coef_mode": "bilinear", "basis_mode": "bilinear",
              "num_layers": 2, "hidden_dim": 64, "out_dim": 32, "with_dropout": False},
    "dataset": {"aabb": [[-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]], "scene_reso": 768, "is_unbound": False,
                "dataset_name": "blender"},
    "training": {"volume_resoInit": 128, "volume_resoFinal": 300, "linear_mat": True, "coeff": True,
                 "basis": True, "renderModule": True},
    "renderer": {"shadingMode": "MLP_Fea", "num_layers": 3, "hidden_dim": 128, "fea2denseAct": "softplus",
                 "density_shift": -10.0, "distance_scale": 25.0, "view_pe": 6, "fea_pe": 2, "step_ratio": 0.5,
                 "rayMarch_weight_thres": 1e-3, "alphaMask_thres": 0.02},
}


def merged_cfg(overrides):
    """DEFAULTS updated (recursively) with overrides -> Cfg."""
    def merge(a, b):
        out = copy.deepcopy(a)
        for k, v in (b or {}).items():
            out[k] = merge(out.get(k, {}), v) if isinstance(v, dict) and isinstance(out.get(k), dict) else v
        return out
    return make_cfg(merge(DEFAULTS, overrides))


def n_to_reso(n_voxels, bbox):
    """utils.py:53-57: per-axis resolution giving about n_voxels cells over bbox (float32 ops)."""
    lo, hi = bbox[0], bbox[1]
    dim = len(lo)
    voxel = ((hi - lo).prod() / n_voxels).pow(1 / dim)
    return torch.round((hi - lo) / voxel).long().tolist()


class FieldGeometry:
    """Sizes of a grid/grid factor field derived from its config, as the reference's
    FactorFields.setup_params does (models/FactorFields.py:262-309). All tensors on the CPU."""

    def __init__(self, cfg):
        mode = cfg.defaults.mode
        aabb_list = cfg.dataset.aabb
        m = cfg.model
        if m.coeff_type != "grid" or m.basis_type != "grid":
            raise NotImplementedError("only basis_type='grid' with coeff_type='grid' is implemented "
                                      f"(got basis_type={m.basis_type!r}, coeff_type={m.coeff_type!r})")
        self.mode = mode
        self.in_dim = len(aabb_list[0]) - 1 if mode in ("images", "reconstructions") else len(aabb_list[0])
        self.aabb = torch.tensor(aabb_list, dtype=torch.float32)[:, :self.in_dim]
        self.basis_dims = list(m.basis_dims)
        n_feat = sum(self.basis_dims)
        self.n_scene = 1
        if "reconstruction" not in mode:
            if "image" in mode:
                self.basis_reso = list(m.basis_resos)
            else:
                self.basis_reso = np.round(np.array(m.basis_resos) * (min(aabb_list[1][:self.in_dim]) + 1)
                                           / 1024.0).astype("int").tolist()
            t_basis = m.T_basis if (m.T_basis or 0) > 0 else int(
                sum(np.power(np.array(self.basis_reso), self.in_dim) * np.array(self.basis_dims)))
            t_coeff = m.T_coeff if (m.T_coeff or 0) > 0 else (m.total_params or 0) - t_basis
            t_coeff = t_coeff if t_coeff > 0 else 8 ** self.in_dim * n_feat
            self.T_basis, self.T_coeff = t_basis, t_coeff
            if mode == "image":
                self.freq_bands = max(aabb_list[1][:self.in_dim]) / torch.tensor(self.basis_reso, dtype=torch.float32)
            else:
                self.freq_bands = torch.tensor(m.freq_bands, dtype=torch.float32)
            self.coeff_reso = n_to_reso(t_coeff // n_feat, self.aabb[:, :self.in_dim])[::-1]
            if mode == "sdf":
                self.freq_bands = self.freq_bands * 0.5
            elif mode == "images":
                self.coeff_reso = [int(aabb_list[1][-1])] + self.coeff_reso
                self.aabb = torch.tensor(aabb_list, dtype=torch.float32)
        else:
            self.coeff_reso = n_to_reso(m.coeff_reso ** self.in_dim, self.aabb[:, :self.in_dim])[::-1]
            self.T_coeff = n_feat * int(np.prod(self.coeff_reso))
            self.T_basis = m.total_params - self.T_coeff
            scale = self.T_basis / sum(np.power(np.array(m.basis_resos), self.in_dim) * np.array(self.basis_dims))
            scale = np.power(scale, 1.0 / self.in_dim)
            self.basis_reso = np.round(np.array(m.basis_resos) * scale).astype("int").tolist()
            freq = torch.tensor(m.freq_bands, dtype=torch.float32)
            if mode == "reconstructions":
                self.freq_bands = freq
                self.n_scene = int(aabb_list[1][-1])
            else:
                self.freq_bands = freq * (cfg.dataset.scene_reso / float(max(self.basis_reso)) / max(m.freq_bands))
        self.coeff_reso = [int(r) for r in self.coeff_reso]
        self.basis_reso = [int(r) for r in self.basis_reso]
        self.n_feat = n_feat

    @property
    def coord_dim(self):
        """Dims of the input points (and of the coefficient grid)."""
        return self.aabb.shape[1]


def render_step(aabb, grid_size, step_ratio):
    """update_renderParams (models/FactorFields.py:693-699): (stepSize tensor, nSamples)."""
    aabb_size = aabb[1] - aabb[0]
    units = aabb_size / (torch.tensor(grid_size, dtype=torch.long) - 1)
    step = torch.mean(units) * step_ratio
    diag = torch.sqrt(torch.sum(torch.square(aabb_size)))
    return step, int((diag / step).item()) + 1
