"""CPU baseline: the reference's own PyTorch op sequence for the field path, on the host cores.

TEST INFRASTRUCTURE ONLY: used by bench.py (--impl reference, and the cpu_baseline leg) and
by tests; never by the product path. The reference checkout is not available where the
benchmarks run, so this module restates, with the same PyTorch CPU kernels the reference calls, its field path:

  grid_mapping           models/FactorFields.py:11-22   (remainder / floor_divide / where)
  get_basis (grid)       models/FactorFields.py:479-490 (one F.grid_sample per level)
  get_coeff (grid)       models/FactorFields.py:432-434 (F.grid_sample, border, align=False)
  get_coding             models/FactorFields.py:523-527
  MLPMixer               models/FactorFields.py:113-159
and autograd's grid_sampler backward, and its render path for bounded scenes:

  sample_point           models/FactorFields.py:586-602
  AlphaGridMask          models/FactorFields.py:91-110, applied at :864-867
  basis2density          models/FactorFields.py:639-643
  raw2alpha              models/FactorFields.py:82-88
  FactorFields.forward   models/FactorFields.py:843-898 (the compositing, white background, clamp, depth)
with the configuration-2 colour head: eval_sh at degree 2 (models/sh.py:34-64, the published
real-SH table in the reference's op order) composed with a sigmoid.
tests/test_oracle_golden.py pins it to the golden outputs produced by the reference itself.
"""
import torch
import torch.nn.functional as F


def grid_mapping(positions, freq_bands, aabb, mode):
    size = max(aabb[1] - aabb[0])
    scale = size[..., None] / freq_bands
    if mode == "triangle":
        loc = (positions - aabb[0]).unsqueeze(-1) % scale
        odd = ((positions - aabb[0]).unsqueeze(-1) // scale) % 2
        loc = loc / (scale / 2) - 1
        return torch.where(odd == 1, -loc, loc)
    loc = (positions - aabb[0])[..., None] % scale
    return (loc / (scale / 2) - 1).clamp(-1.0, 1.0)


class RefField(torch.nn.Module):
    """Reference-layout parameters ([1, C, R..] grids, nn.Linear MLP) and the reference's ops."""

    def __init__(self, mode, aabb, basis_levels, coeff_grid, mlp_weights, mlp_biases, freq_bands, mapping,
                 basis_mode="bilinear", coef_mode="bilinear"):
        super().__init__()
        self.mode = mode
        aabb = torch.as_tensor(aabb, dtype=torch.float32)
        full = aabb.shape[1]
        self.in_dim = full - 1 if mode in ("images", "reconstructions") else full
        self.aabb = aabb if mode == "images" else aabb[:, :self.in_dim]
        self.basises = torch.nn.ParameterList([torch.nn.Parameter(torch.as_tensor(b).clone()) for b in basis_levels])
        self.coeff = torch.nn.Parameter(torch.as_tensor(coeff_grid).clone())
        self.weights = torch.nn.ParameterList([torch.nn.Parameter(torch.as_tensor(w).clone()) for w in mlp_weights])
        self.biases = [None if b is None else torch.nn.Parameter(torch.as_tensor(b).clone()) for b in mlp_biases]
        for i, b in enumerate(self.biases):
            if b is not None:
                self.register_parameter(f"bias{i}", b)
        self.freq_bands = torch.as_tensor(freq_bands, dtype=torch.float32)
        self.mapping, self.basis_mode, self.coef_mode = mapping, basis_mode, coef_mode

    def get_coeff(self, x):
        n, dim = x.shape
        inv = 2.0 / (self.aabb[1] - self.aabb[0])
        pts = ((x - self.aabb[0]) * inv - 1).view([1, -1] + [1] * (dim - 1) + [dim])
        return F.grid_sample(self.coeff, pts, mode=self.coef_mode, align_corners=False,
                             padding_mode="border").view(-1, n).t()

    def get_basis(self, x):
        n = x.shape[0]
        if self.mode == "images":
            x = x[..., :-1]
        L = len(self.freq_bands)
        xyz = grid_mapping(x, self.freq_bands, self.aabb[:, :self.in_dim], self.mapping)
        xyz = xyz.view(1, *([1] * (self.in_dim - 1)), -1, self.in_dim, L)
        outs = [F.grid_sample(self.basises[i], xyz[..., i], mode=self.basis_mode, align_corners=True).view(-1, n).T
                for i in range(L)]
        return torch.cat(outs, dim=-1)

    def get_coding(self, x):
        coeff = self.get_coeff(x)
        return self.get_basis(x) * coeff, coeff

    def mlp(self, h):
        for i, w in enumerate(self.weights):
            h = F.linear(h, w, self.biases[i])
            if i != len(self.weights) - 1:
                h = F.relu(h)
        return h

    def fit_step(self, x, target, loss="l1"):
        """One fwd+bwd regression step (the notebooks' loop without the optimizer)."""
        self.zero_grad(set_to_none=True)
        feats, _ = self.get_coding(x)
        pred = self.mlp(feats)
        err = pred - target
        lv = err.abs().mean() if loss == "l1" else (err * err).mean()
        lv.backward()
        return float(lv.detach())


def from_model(m):
    """RefField holding a CPU copy of a factor_fields_gb300.FactorFields' parameters."""
    ws, bs = m.linear_mat.weights()
    return RefField(m.cfg.defaults.mode, m.cfg.dataset.aabb, [b.detach().cpu() for b in m.basises],
                    m.coeffs[m.scene_idx].detach().cpu(), [w.detach().cpu() for w in ws],
                    [None if b is None else b.detach().cpu() for b in bs], m.freq_bands.cpu(),
                    m.cfg.model.basis_mapping, m.cfg.model.basis_mode, m.cfg.model.coef_mode)


SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396)


def eval_sh2(sh, dirs):
    """models/sh.py:34-64 at degree 2: sh [..., C, 9], dirs [..., 3] -> [..., C]."""
    result = SH_C0 * sh[..., 0]
    x, y, z = dirs[..., 0:1], dirs[..., 1:2], dirs[..., 2:3]
    result = result - SH_C1 * y * sh[..., 1] + SH_C1 * z * sh[..., 2] - SH_C1 * x * sh[..., 3]
    xx, yy, zz = x * x, y * y, z * z
    xy, yz, xz = x * y, y * z, x * z
    return (result + SH_C2[0] * xy * sh[..., 4] + SH_C2[1] * yz * sh[..., 5] + SH_C2[2] * (2.0 * zz - xx - yy) * sh[..., 6]
            + SH_C2[3] * xz * sh[..., 7] + SH_C2[4] * (xx - yy) * sh[..., 8])


def raw2alpha(sigma, dist):
    alpha = 1. - torch.exp(-sigma * dist)
    T = torch.cumprod(torch.cat([torch.ones_like(alpha[..., :1]), 1. - alpha + 1e-10], -1), -1)
    return alpha, alpha * T[..., :-1]


class RefRender:
    """FactorFields.forward for bounded scenes on a RefField (the reference's op sequence), with the
    degree-2 SH colour head. alpha_volume: the occupancy volume [D, H, W] (AlphaGridMask over
    aabb) or None."""

    def __init__(self, field, step, n_samples, alpha_volume=None, density_shift=-10.0, distance_scale=25.0,
                 weight_thres=1e-3, act="softplus"):
        self.f, self.step, self.n_samples = field, float(step), int(n_samples)
        self.aabb = field.aabb[:, :3]
        self.alpha = None if alpha_volume is None else torch.as_tensor(alpha_volume).view(1, 1, *alpha_volume.shape[-3:])
        self.inv = 1.0 / (self.aabb[1] - self.aabb[0]) * 2
        self.shift, self.dscale, self.thres, self.act = density_shift, distance_scale, weight_thres, act

    def sample_point(self, rays_o, rays_d, jitter=None):
        vec = torch.where(rays_d == 0, torch.full_like(rays_d, 1e-6), rays_d)
        rate_a = (self.aabb[1] - rays_o) / vec
        rate_b = (self.aabb[0] - rays_o) / vec
        t_min = torch.minimum(rate_a, rate_b).amax(-1).clamp(min=0.05, max=1e3)
        rng = torch.arange(self.n_samples)[None].float()
        if jitter is not None:
            rng = rng.repeat(rays_d.shape[-2], 1)
            rng += jitter
        interpx = t_min[..., None] + self.step * rng
        pts = rays_o[..., None, :] + rays_d[..., None, :] * interpx[..., None]
        outside = ((self.aabb[0] > pts) | (pts > self.aabb[1])).any(dim=-1)
        return pts, interpx, ~outside

    def forward(self, rays, white_bg=True, jitter=None):
        """(rgb [R, 3], depth [R]); jitter [R, 1] (training jitter u) or None."""
        viewdirs = rays[:, 3:6]
        xyz, z_vals, inner = self.sample_point(rays[:, :3], viewdirs, jitter)
        dists = torch.cat((z_vals[:, 1:] - z_vals[:, :-1], torch.zeros_like(z_vals[:, :1])), dim=-1)
        viewdirs = viewdirs.view(-1, 1, 3).expand(xyz.shape)
        valid = inner
        if self.alpha is not None:
            pts = (xyz[inner] - self.aabb[0]) * self.inv - 1
            a = F.grid_sample(self.alpha, pts.view(1, -1, 1, 1, 3), align_corners=True).view(-1)
            valid[inner.clone()] = a > 0.5
        sigma = torch.zeros(xyz.shape[:-1])
        rgb = torch.zeros((*xyz.shape[:2], 3))
        feat = None
        if valid.any():
            feats, _ = self.f.get_coding(xyz[valid])
            feat = self.f.mlp(feats)
            x = feat[..., 0] + self.shift
            sigma[valid] = F.softplus(x) if self.act == "softplus" else F.relu(x)
        alpha, weight = raw2alpha(sigma, dists * self.dscale)
        app = weight > self.thres
        valid_new = torch.logical_and(valid, app)
        app = valid_new[valid]
        if app.any():
            rgb[valid_new] = torch.sigmoid(eval_sh2(feat[app, 1:].view(-1, 3, 9), viewdirs[valid_new]))
        acc = torch.sum(weight, -1)
        rgb_map = torch.sum(weight[..., None] * rgb, -2)
        if white_bg:
            rgb_map = rgb_map + (1. - acc[..., None])
        rgb_map = rgb_map.clamp(0, 1)
        with torch.no_grad():
            depth = torch.sum(weight * z_vals, -1)
        return rgb_map, depth

    def train_step(self, rays, rgb_gt, jitter=None):
        """One fwd+bwd render step with the MSE loss (train_per_scene.py:150-160 without the
        optimizer); returns the loss."""
        self.f.zero_grad(set_to_none=True)
        rgb, _ = self.forward(rays, white_bg=True, jitter=jitter)
        loss = torch.mean((rgb - rgb_gt) ** 2)
        loss.backward()
        return float(loss.detach())
