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


# ---------------------------------------------------------------------------------------
# radiance-field scene (cfg2, cfg3)
# ---------------------------------------------------------------------------------------

class BlobScene:
    """32 Gaussian density blobs in [-1.5, 1.5]^3: sigma(x) = sum_b p_b exp(-|x - c_b|^2 / (2 s_b^2))
    with peaks p_b ~ U[5, 50], widths s_b ~ U[0.05, 0.3]; the colour at x is the density-weighted
    mean of the blobs' RGB albedos (view independent). Ground truth is rendered by FP64
    quadrature (render_gt) against a white background."""

    def __init__(self, seed=0, n_blobs=32):
        rng = np.random.default_rng(seed)
        self.centers = rng.uniform(-1.0, 1.0, (n_blobs, 3))
        self.peaks = rng.uniform(5.0, 50.0, n_blobs)
        self.widths = rng.uniform(0.05, 0.3, n_blobs)
        self.albedo = rng.uniform(0.05, 0.95, (n_blobs, 3))
        self.aabb = np.array([[-1.5] * 3, [1.5] * 3])

    def cameras(self, n_views=100, radius=4.0, seed=1):
        """c2w [n, 3, 4] (OpenCV axes: x right, y down, z forward) on the upper hemisphere,
        looking at the origin."""
        rng = np.random.default_rng(seed)
        th = rng.uniform(0, 2 * np.pi, n_views)
        ph = np.arccos(rng.uniform(0.1, 0.95, n_views))
        eye = np.stack([np.sin(ph) * np.cos(th), np.sin(ph) * np.sin(th), np.cos(ph)], 1) * radius
        out = np.zeros((n_views, 3, 4))
        for i, e in enumerate(eye):
            fwd = -e / np.linalg.norm(e)
            right = np.cross(fwd, np.array([0.0, 0.0, 1.0]))
            right /= np.linalg.norm(right)
            down = np.cross(fwd, right)
            out[i, :, 0], out[i, :, 1], out[i, :, 2], out[i, :, 3] = right, down, fwd, e
        return out

    @staticmethod
    def pixel_rays(c2w, px, py, width=400, height=400, focal=555.0):
        """Rays through pixel centres (get_ray_directions + get_rays, dataLoader/ray_utils.py:27-90,
        directions normalised as dataLoader/blender.py:55): [n, 6] float64."""
        d = np.stack([(px + 0.5 - width / 2) / focal, (py + 0.5 - height / 2) / focal, np.ones_like(px, float)], -1)
        d /= np.linalg.norm(d, axis=-1, keepdims=True)
        rd = np.einsum("nij,nj->ni", c2w[:, :3, :3], d)
        return np.concatenate([c2w[:, :3, 3], rd], -1)

    def ray_pool(self, n, seed, views=None, n_views=100, width=400, height=400):
        """n random camera rays (random view and pixel) from the scene's views."""
        rng = np.random.default_rng(seed)
        cams = self.cameras(n_views)
        v = rng.integers(0, n_views, n) if views is None else rng.choice(views, n)
        px, py = rng.integers(0, width, n), rng.integers(0, height, n)
        return self.pixel_rays(cams[v], px, py, width, height)

    def test_dataset(self, views, width=400, height=400, n_views=100, n_steps=512, device="cuda"):
        """Full test images of the given views in the layout the reference's evaluation reads
        (renderer.py:30-98): an object with img_wh, all_rays [V, H*W, 6] and all_rgbs
        [V, H*W, 3] (float32 CPU tensors; the colours are the FP64 ground truth)."""
        import types
        cams = self.cameras(n_views)
        py, px = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
        px, py = px.reshape(-1), py.reshape(-1)
        rays, rgbs = [], []
        for v in views:
            r = self.pixel_rays(np.repeat(cams[v][None], px.size, 0), px, py, width, height)
            rays.append(torch.from_numpy(r).float())
            rgbs.append(self.render_gt(r, n_steps=n_steps, device=device).float().cpu())
        return types.SimpleNamespace(img_wh=(width, height), all_rays=torch.stack(rays), all_rgbs=torch.stack(rgbs))

    def render_gt(self, rays, n_steps=1024, chunk=2048, device="cuda", with_depth=False):
        """FP64 quadrature of the emission-absorption integral along each ray through the box,
        white background: rgb [n, 3] float32 (midpoint rule, n_steps steps between box entry
        and exit; alpha_i = 1 - exp(-sigma_i dt)); with_depth also returns the expected depth
        sum_i w_i t_i [n] (the quantity depth_map is, models/FactorFields.py:895-896)."""
        dev = torch.device(device)
        c = torch.tensor(self.centers, dtype=torch.float64, device=dev)
        p = torch.tensor(self.peaks, dtype=torch.float64, device=dev)
        inv2s2 = torch.tensor(1.0 / (2 * self.widths ** 2), dtype=torch.float64, device=dev)
        alb = torch.tensor(self.albedo, dtype=torch.float64, device=dev)
        lo = torch.tensor(self.aabb[0], dtype=torch.float64, device=dev)
        hi = torch.tensor(self.aabb[1], dtype=torch.float64, device=dev)
        out, depths = [], []
        rays_t = torch.as_tensor(rays, dtype=torch.float64)
        for s in range(0, rays_t.shape[0], chunk):
            r = rays_t[s:s + chunk].to(dev)
            o, d = r[:, :3], r[:, 3:6]
            dd = torch.where(d == 0, torch.full_like(d, 1e-12), d)
            ta, tb = (lo - o) / dd, (hi - o) / dd
            t0 = torch.minimum(ta, tb).amax(-1).clamp(min=0.0)
            t1 = torch.maximum(ta, tb).amin(-1)
            t1 = torch.maximum(t1, t0)
            dt = (t1 - t0) / n_steps
            rgb = torch.zeros(r.shape[0], 3, dtype=torch.float64, device=dev)
            depth = torch.zeros(r.shape[0], dtype=torch.float64, device=dev)
            trans = torch.ones(r.shape[0], dtype=torch.float64, device=dev)
            blk = 128
            for b0 in range(0, n_steps, blk):
                steps = torch.arange(b0, min(b0 + blk, n_steps), dtype=torch.float64, device=dev) + 0.5
                ts = t0[:, None] + steps[None] * dt[:, None]                       # [n, blk]
                x = o[:, None, :] + d[:, None, :] * ts[..., None]                   # [n, blk, 3]
                g = torch.exp(-((x[:, :, None, :] - c) ** 2).sum(-1) * inv2s2) * p  # [n, blk, blobs]
                sig = g.sum(-1)
                col = (g @ alb) / sig.clamp(min=1e-300)[..., None]
                keep = torch.exp(-sig * dt[:, None])                                # 1 - alpha
                incl = torch.cumprod(keep, dim=1)
                excl = torch.cat([torch.ones_like(incl[:, :1]), incl[:, :-1]], 1)
                w = trans[:, None] * excl * (1.0 - keep)
                rgb += (w[..., None] * col).sum(1)
                depth += (w * ts).sum(1)
                trans = trans * incl[:, -1]
            rgb += trans[:, None]  # white background
            out.append(rgb.float())
            depths.append(depth.float())
        if with_depth:
            return torch.cat(out).cpu(), torch.cat(depths).cpu()
        return torch.cat(out).cpu()


def to_device(arrs, device):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in arrs]
