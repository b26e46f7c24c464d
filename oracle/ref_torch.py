"""CPU baseline: the reference's own PyTorch op sequence for the field path, on the host cores.

TEST INFRASTRUCTURE ONLY: used by bench.py (--impl reference, and the cpu_baseline leg) and
by tests; never by the product path. The reference checkout is not available where the
benchmarks run, so this module restates, with the same PyTorch CPU kernels the reference calls, its field path:

  grid_mapping           models/FactorFields.py:11-22   (remainder / floor_divide / where)
  get_basis (grid)       models/FactorFields.py:479-490 (one F.grid_sample per level)
  get_coeff (grid)       models/FactorFields.py:432-434 (F.grid_sample, border, align=False)
  get_coding             models/FactorFields.py:523-527
  MLPMixer               models/FactorFields.py:113-159
and autograd's grid_sampler backward. tests/test_oracle_golden.py pins it to the golden
outputs produced by the reference itself.
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
