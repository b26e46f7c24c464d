"""The five benchmark workloads: config recipes and seeded synthetic inputs.

The reference measures on real datasets (images, meshes, NeRF scenes) that are not available
here; these seeded generators stand in for them with the same shapes, sizes and value ranges:

  cfg0  2-D field fit: 512x512x3 procedural image (64 anisotropic Gaussians + band-limited
        sinusoid noise, clipped to [0, 1]); 65,536 pixel coordinates per step, MSE.
  cfg1  3-D SDF fit: analytic SDF of a union of 16 spheres (r ~ U[0.1, 0.3]) and 8
        axis-aligned boxes in [-1, 1]^3; 262,144 points per step (half uniform, half surface
        points + N(0, 0.01^2)), L1.
  cfg2  radiance field, plain sampler: 32 Gaussian density blobs in [-1.5, 1.5]^3.
  cfg3  the same scene with the proposal sampler.
  cfg4  image set: 256 procedural 256x256x3 images (the cfg0 generator, seeds 1..256);
        262,144 coordinates per step spread over all images (z = image index + 0.5).

Targets are evaluated analytically at the sampled coordinates (no image is rasterised).
"""
import numpy as np
import torch

from .config import merged_cfg

FREQ6 = [2.0, 3.2, 4.4, 5.6, 6.8, 8.0]
RESOS6 = [32, 51, 70, 89, 108, 128]
DIMS6 = [4, 4, 4, 2, 2, 2]
N_BASIS_3D = int(sum(np.power(np.array(RESOS6), 3) * np.array(DIMS6)))  # 10,157,342


def field_cfg(key, small=False):
    """Reference-style config of one benchmark configuration (FactorFields(cfg) input).

    cfg0 uses mode 'image', whose constructor derives freq_bands = 512 / basis_resos; the
    benchmark's freq_bands (FREQ6) are set on the model after construction."""
    if key == "cfg0":
        return merged_cfg({"defaults": {"mode": "image"},
                           "model": {"total_params": 1426063, "out_dim": 3, "basis_mapping": "sawtooth"},
                           "dataset": {"aabb": [[0, 0], [512, 512]]}})
    if key == "cfg1":
        return merged_cfg({"defaults": {"mode": "reconstruction"},
                           "model": {"coeff_reso": 32, "total_params": 18 * 32 ** 3 + N_BASIS_3D, "out_dim": 1,
                                     "basis_mapping": "sawtooth"},
                           "dataset": {"aabb": [[-1, -1, -1], [1, 1, 1]], "scene_reso": 1024}})
    if key in ("cfg2", "cfg3"):
        return merged_cfg({"defaults": {"mode": "reconstruction"},
                           "model": {"coeff_reso": 64, "total_params": 18 * 64 ** 3 + N_BASIS_3D, "out_dim": 28,
                                     "basis_mapping": "triangle"},
                           "dataset": {"aabb": [[-1.5] * 3, [1.5] * 3], "scene_reso": 1024},
                           "renderer": {"shadingMode": "SH"}})
    if key == "cfg4":
        hi = [64, 64, 16] if small else [256, 256, 256]
        side = 8 if small else 32
        return merged_cfg({"defaults": {"mode": "images"},
                           "model": {"T_coeff": side * side * 18, "out_dim": 3, "basis_mapping": "sawtooth"},
                           "dataset": {"aabb": [[0, 0, 0], hi]}})
    raise KeyError(key)


# ---------------------------------------------------------------------------------------
# procedural images (cfg0, cfg4)
# ---------------------------------------------------------------------------------------

class ProceduralImage:
    """64 random anisotropic Gaussians + band-limited sinusoid noise on a W x H canvas."""

    def __init__(self, seed, width=512, height=512, n_gauss=64, n_waves=8):
        rng = np.random.default_rng(seed)
        self.w, self.h = width, height
        s = max(width, height)
        self.centers = rng.uniform(0, 1, (n_gauss, 2)) * [width, height]
        theta = rng.uniform(0, np.pi, n_gauss)
        sig = rng.uniform(s / 64, s / 8, (n_gauss, 2))
        rot = np.stack([np.stack([np.cos(theta), -np.sin(theta)], -1),
                        np.stack([np.sin(theta), np.cos(theta)], -1)], -2)  # [G,2,2]
        cov = rot @ (np.eye(2)[None] * (sig ** 2)[:, None, :]) @ np.transpose(rot, (0, 2, 1))
        self.prec = np.linalg.inv(cov)
        self.amp = rng.uniform(-0.6, 1.0, (n_gauss, 3))
        self.base = rng.uniform(0.2, 0.6, 3)
        self.freq = rng.integers(-16, 17, (n_waves, 2)) / np.array([width, height])
        self.phase = rng.uniform(0, 2 * np.pi, (n_waves, 3))
        self.wamp = rng.uniform(0.01, 0.05, (n_waves, 3))

    def __call__(self, xy):
        """xy [N, 2] pixel-space coordinates -> rgb [N, 3] float32 in [0, 1]."""
        xy = np.asarray(xy, np.float64)
        out = np.tile(self.base, (xy.shape[0], 1))
        for g in range(self.centers.shape[0]):
            d = xy - self.centers[g]
            q = np.einsum("ni,ij,nj->n", d, self.prec[g], d)
            out += np.exp(-0.5 * q)[:, None] * self.amp[g]
        arg = 2 * np.pi * (xy @ self.freq.T)  # [N, waves]
        for w in range(self.freq.shape[0]):
            out += np.sin(arg[:, w:w + 1] + self.phase[w]) * self.wamp[w]
        return np.clip(out, 0, 1).astype(np.float32)


def image_batch(seed, n, width=512, height=512, img=None):
    """n random pixel centres (x + 0.5, y + 0.5) and their colours."""
    rng = np.random.default_rng(seed)
    img = img or ProceduralImage(0, width, height)
    px = rng.integers(0, [width, height], (n, 2))
    xy = (px + 0.5).astype(np.float32)
    return xy, img(xy)


def image_set_batch(seed, n, n_images=256, side=256):
    """n coordinates (x + 0.5, y + 0.5, image + 0.5) over n_images procedural images (seeds
    1..n_images) and their colours."""
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, n_images, n)
    px = rng.integers(0, side, (n, 2))
    xyz = np.concatenate([px + 0.5, idx[:, None] + 0.5], 1).astype(np.float32)
    rgb = np.zeros((n, 3), np.float32)
    for i in np.unique(idx):
        sel = idx == i
        rgb[sel] = ProceduralImage(int(i) + 1, side, side)(xyz[sel, :2])
    return xyz, rgb


# ---------------------------------------------------------------------------------------
# analytic SDF (cfg1)
# ---------------------------------------------------------------------------------------

class SDFScene:
    """Union of 16 spheres (radius U[0.1, 0.3]) and 8 axis-aligned boxes in [-1, 1]^3."""

    def __init__(self, seed=0):
        rng = np.random.default_rng(seed)
        self.sc = rng.uniform(-0.7, 0.7, (16, 3))
        self.sr = rng.uniform(0.1, 0.3, 16)
        self.bc = rng.uniform(-0.7, 0.7, (8, 3))
        self.bh = rng.uniform(0.05, 0.25, (8, 3))

    def sdf(self, p):
        p = np.asarray(p, np.float64)
        ds = np.linalg.norm(p[:, None, :] - self.sc[None], axis=-1) - self.sr[None]
        q = np.abs(p[:, None, :] - self.bc[None]) - self.bh[None]
        db = np.linalg.norm(np.maximum(q, 0), axis=-1) + np.minimum(q.max(-1), 0)
        return np.minimum(ds.min(1), db.min(1))

    def surface_points(self, rng, n):
        k = rng.integers(0, 24, n)
        out = np.zeros((n, 3))
        sph = k < 16
        d = rng.standard_normal((int(sph.sum()), 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out[sph] = self.sc[k[sph]] + d * self.sr[k[sph], None]
        bi = k[~sph] - 16
        m = bi.shape[0]
        face = rng.integers(0, 3, m)
        sign = rng.choice([-1.0, 1.0], m)
        u = rng.uniform(-1, 1, (m, 3))
        u[np.arange(m), face] = sign
        out[~sph] = self.bc[bi] + u * self.bh[bi]
        return out


def sdf_batch(seed, n, scene=None):
    """n points (half uniform in [-1,1]^3, half near-surface) and their SDF values [n, 1]."""
    scene = scene or SDFScene(0)
    rng = np.random.default_rng(seed)
    h = n // 2
    uni = rng.uniform(-1, 1, (h, 3))
    surf = scene.surface_points(rng, n - h) + rng.normal(0, 0.01, (n - h, 3))
    p = np.clip(np.concatenate([uni, surf], 0), -1, 1).astype(np.float32)
    return p, scene.sdf(p).astype(np.float32)[:, None]


def to_device(arrs, device):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in arrs]
