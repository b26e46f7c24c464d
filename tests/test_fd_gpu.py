"""The hand-written backward kernels against FP64 central finite differences of the FP64 oracle's
forward (models/FactorFields.py:425-527 field, :113-159 MLP, :82-88 / :876-896 compositing).

The finite differences are taken of the oracle's FP64 forward, independently of its analytic
backward; each checked gradient entry is compared with the GPU's. Tolerances are relative to the
largest gradient entry: float32 drop-in kernels 1e-4, BF16 fused kernels 3e-2 (against the
forward of the BF16-stored model: grids and MLP weights rounded to BF16). The field is linear in
every grid value, so its differences are exact for any step; MLP weights and compositing inputs
use small steps (1e-6 relative) away from the ReLU kinks and weight thresholds."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import need_gpu
from oracle import ff_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


def _small_model(precision="fp32", out_dim=28, mapping="triangle", seed=0):
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300.config import merged_cfg
    cfg = merged_cfg({"defaults": {"mode": "reconstruction"},
                      "model": {"basis_resos": [5, 6, 7, 8, 9, 10], "coeff_reso": 6, "total_params": 11106,
                                "out_dim": out_dim, "basis_mapping": mapping},
                      "dataset": {"aabb": [[-1.5] * 3, [1.5] * 3], "scene_reso": 1024},
                      "renderer": {"shadingMode": "SH"}})
    torch.manual_seed(seed)
    m = FactorFields(cfg, device="cuda", precision=precision)
    g = torch.Generator().manual_seed(seed + 1)
    with torch.no_grad():
        m.coeff_flat.copy_((torch.rand(m.coeff_flat.shape, generator=g) * 2 - 1).cuda())
        m.basis_flat.add_((torch.rand(m.basis_flat.shape, generator=g) * 0.4 - 0.2).cuda())
        if precision == "bf16":  # the stored model: BF16 values
            m.basis_flat.copy_(m.basis_flat.to(torch.bfloat16).float())
            m.coeff_flat.copy_(m.coeff_flat.to(torch.bfloat16).float())
    return m


def _spec(m):
    return O.FieldSpec(m.cfg.defaults.mode, m.cfg.dataset.aabb, m.basis_dims, m.basis_reso, m.freq_bands.cpu().numpy(),
                       m.coeff_reso, m.cfg.model.basis_mapping, m.cfg.model.basis_mode, m.cfg.model.coef_mode)


def _grids(m):
    return [b[0].detach().cpu().double().numpy().copy() for b in m.basises], \
        m.coeffs[0][0].detach().cpu().double().numpy().copy()


def _pick(grad, k, rng):
    """k entries: the largest |grad| half and a random half of the nonzero ones."""
    flat = np.abs(grad).reshape(-1)
    top = np.argsort(flat)[-(k // 2):]
    nz = np.flatnonzero(flat > 0)
    rest = rng.choice(nz, size=min(k - len(top), len(nz)), replace=False)
    return np.unique(np.concatenate([top, rest]))


def _fd_check(loss_fn, params, grads_gpu, k, rng, eps_rel, tol, what):
    """Central differences of loss_fn(params) (FP64) at k entries of each parameter array against
    the GPU gradients; error relative to max |gpu gradient| of that array."""
    for name, arr in params.items():
        g_gpu = np.asarray(grads_gpu[name], np.float64).reshape(arr.shape)
        scale = np.abs(g_gpu).max()
        assert scale > 0, name
        for flat in _pick(g_gpu, k, rng):
            idx = np.unravel_index(flat, arr.shape)
            orig = arr[idx]
            eps = eps_rel * max(1.0, abs(orig))
            arr[idx] = orig + eps
            lp = loss_fn()
            arr[idx] = orig - eps
            lm = loss_fn()
            arr[idx] = orig
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g_gpu[idx]) <= tol * scale, f"{what} {name}{idx}: fd {fd:.6g} gpu {g_gpu[idx]:.6g}"


def test_field_scatter_fd_dropin():
    """ff_field_backward (the drop-in grid_sample backward scatter) for L = sum g * feats + sum h *
    coeff over 3,000 points, basis levels and the coefficient grid, float32: 1e-4."""
    m = _small_model()
    rng = np.random.default_rng(0)
    x = rng.uniform(-1.5, 1.5, (3000, 3)).astype(np.float32)
    gfe = rng.standard_normal((3000, 18))
    gco = rng.standard_normal((3000, 18))
    feats, coeff = m.get_coding(torch.from_numpy(x).cuda())
    ((feats * torch.from_numpy(gfe).float().cuda()).sum() + (coeff * torch.from_numpy(gco).float().cuda()).sum()).backward()
    spec = _spec(m)
    bg, cg = _grids(m)
    params = {f"basis{l}": bg[l] for l in range(6)}
    params["coeff"] = cg
    grads = {f"basis{l}": m.layout.basis_view(m.basis_flat.grad, l)[0].cpu().numpy() for l in range(6)}
    grads["coeff"] = m.layout.coeff_view(m.coeff_flat.grad, 0)[0].cpu().numpy()

    def loss():
        f, c = O.get_coding(spec, bg, cg, x)
        return float((f * gfe).sum() + (c * gco).sum())

    _fd_check(loss, params, grads, 12, rng, 1e-3, 1e-4, "drop-in scatter")


def test_mlp_backward_fd_dropin():
    """ff_mlp_backward (MLPMixer 18 -> 64 -> 28, float32): weight, bias and input gradients."""
    m = _small_model()
    rng = np.random.default_rng(1)
    xin = rng.standard_normal((2000, 18)).astype(np.float32)
    g = rng.standard_normal((2000, 28))
    xt = torch.from_numpy(xin).cuda().requires_grad_(True)
    out = m.linear_mat(xt)
    (out * torch.from_numpy(g).float().cuda()).sum().backward()
    ws, bs = m.linear_mat.weights()
    wn = [w.detach().cpu().double().numpy().copy() for w in ws]
    bn = [None if b is None else b.detach().cpu().double().numpy().copy() for b in bs]
    xd = xin.astype(np.float64)
    params = {"w0": wn[0], "b0": bn[0], "w1": wn[1], "x": xd}
    grads = {"w0": ws[0].grad.cpu().numpy(), "b0": bs[0].grad.cpu().numpy(), "w1": ws[1].grad.cpu().numpy(),
             "x": xt.grad.cpu().numpy()}

    def loss():
        o, _ = O.mlp_fwd(wn, bn, xd)
        return float((o * g).sum())

    _fd_check(loss, params, grads, 16, rng, 1e-6, 1e-4, "drop-in MLP")


@pytest.mark.parametrize("mode", ["bwd", "fit"])
def test_fused_field_mlp_fd_bf16(mode):
    """The fused BF16 kernels' backward (ff_field_mlp_backward, MODE kBwd) and whole regression
    step (ff_field_fit_step, MODE kFit, L1 loss) on the BF16-stored model: grid and MLP gradients
    against central differences of the FP64 forward of that model, 3e-2."""
    from factor_fields_gb300.train import FieldFitRunner
    m = _small_model("bf16", out_dim=1 if mode == "fit" else 28, mapping="sawtooth", seed=3)
    ws, bs = m.linear_mat.weights()
    with torch.no_grad():  # the MLP weights the kernel multiplies by are their BF16 values
        for w in ws:
            w.copy_(w.to(torch.bfloat16).float())
    rng = np.random.default_rng(2)
    n = 4096
    x = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    if mode == "bwd":
        g = rng.standard_normal((n, 28))
        out = m.field_mlp(xt)
        (out * torch.from_numpy(g).float().cuda()).sum().backward()
    else:
        t = rng.standard_normal((n, 1)).astype(np.float32)
        FieldFitRunner(m, loss="l1", binned=False).step(xt, torch.from_numpy(t).cuda())
    spec = _spec(m)
    bg, cg = _grids(m)
    wn = [w.detach().cpu().double().numpy().copy() for w in ws]
    bn = [None if b is None else b.detach().cpu().double().numpy().copy() for b in bs]
    params = {"basis0": bg[0], "basis3": bg[3], "basis5": bg[5], "coeff": cg, "w0": wn[0], "w1": wn[1]}
    grads = {"basis0": m.layout.basis_view(m.basis_flat.grad, 0)[0].cpu().numpy(),
             "basis3": m.layout.basis_view(m.basis_flat.grad, 3)[0].cpu().numpy(),
             "basis5": m.layout.basis_view(m.basis_flat.grad, 5)[0].cpu().numpy(),
             "coeff": m.layout.coeff_view(m.coeff_flat.grad, 0)[0].cpu().numpy(),
             "w0": ws[0].grad.cpu().numpy(), "w1": ws[1].grad.cpu().numpy()}

    def loss():
        f, _ = O.get_coding(spec, bg, cg, x)
        o, _ = O.mlp_fwd(wn, bn, f)
        if mode == "bwd":
            return float((o * g).sum())
        return float(np.abs(o - t).mean())

    _fd_check(loss, params, grads, 10, rng, 1e-4, 3e-2, f"fused {mode}")


def _marched_batch(model_seed=0):
    """A small cfg2-style model with an occupancy mask, marched: (m, rays, jitter, rdesc, offsets,
    xyz, sidx, z [M], dist [M])."""
    from factor_fields_gb300.renderer import AlphaGridMask, march, render_desc
    from factor_fields_gb300 import workloads as W
    m = _small_model(seed=model_seed)
    m.update_renderParams([64, 64, 64])
    scene = W.BlobScene(0)
    rays = torch.from_numpy(scene.ray_pool(48, 9)).float().cuda()
    jitter = torch.rand(48, generator=torch.Generator().manual_seed(4)).cuda()
    axis = torch.linspace(-1.5, 1.5, 32, dtype=torch.float64)
    zz, yy, xx = torch.meshgrid(axis, axis, axis, indexing="ij")
    pts = torch.stack([xx, yy, zz], -1).reshape(-1, 3).numpy()
    dens = (np.exp(-((pts[:, None, :] - scene.centers) ** 2).sum(-1) / (2 * scene.widths ** 2)) * scene.peaks).sum(-1)
    m.alphaMask = AlphaGridMask(m.device, m.aabb, torch.from_numpy((dens > 1.0).reshape(32, 32, 32)).float().cuda())
    rdesc = render_desc(m, 256, True)
    offsets, xyz, sidx = march(m, rays, jitter, rdesc)
    # z and dist of each live sample as the kernels compute them (sample_point, :586-602, :861)
    _, zs, _ = O.sample_point(rays.cpu().numpy()[:, :3], rays.cpu().numpy()[:, 3:6], m.aabb.cpu().numpy(),
                              np.float32(m.stepSize.cpu()), 256, jitter.cpu().numpy()[:, None])
    dist = np.concatenate([(zs[:, 1:] - zs[:, :-1]).astype(np.float32), np.zeros((48, 1), np.float32)], 1)
    off = offsets.cpu().numpy()
    si = sidx.cpu().numpy()
    ray_of = np.repeat(np.arange(48), np.diff(off))
    return m, rays, jitter, rdesc, offsets, xyz, sidx, zs[ray_of, si], dist[ray_of, si]


def test_composite_backward_fd():
    """ff_composite_backward (the reverse transmittance scan + SH-2 head, float32) against central
    differences of the FP64 compositing (oracle composite_rows) w.r.t. the density feature and SH
    coefficients of the live samples: 1e-4."""
    from factor_fields_gb300 import _native as N
    m, rays, jitter, rdesc, offsets, xyz, sidx, z, dist = _marched_batch()
    M = xyz.shape[0]
    assert M > 500
    rng = np.random.default_rng(5)
    feat = rng.standard_normal((M, 28)).astype(np.float32)
    feat[:, 0] = rng.uniform(5, 14, M).astype(np.float32)  # softplus(f - 10): densities from ~0 to ~4
    ft = torch.from_numpy(feat).cuda()
    g_rgb = rng.standard_normal((48, 3))
    g_feat = torch.empty_like(ft)
    N.call("ff_composite_backward", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), 48, N.ptr(offsets), N.ptr(sidx),
           N.ptr(ft), 28, None, N.ptr(torch.from_numpy(g_rgb).float().cuda()), N.ptr(g_feat), N.stream_ptr())
    rspec = O.RenderSpec(m.aabb.cpu().numpy(), rdesc.step, 256, rdesc.density_shift, rdesc.distance_scale,
                         rdesc.weight_thres, True)
    off = offsets.cpu().numpy()
    dirs = rays.cpu().numpy()[:, 3:6]
    fd64 = feat.astype(np.float64)

    def loss():
        return float((O.composite_rows(rspec, fd64, z, dist, off, dirs) * g_rgb).sum())

    grads = g_feat.cpu().numpy()
    _fd_check(loss, {"feat": fd64}, {"feat": grads}, 60, rng, 1e-6, 1e-4, "composite")


def test_composite_rgb_backward_fd():
    """ff_composite_backward_rgb (per-sample colours from the MLP_Fea head): dL/dfeat0 and
    dL/dcolour against central differences of the FP64 compositing, 1e-4."""
    from factor_fields_gb300 import _native as N
    m, rays, jitter, rdesc, offsets, xyz, sidx, z, dist = _marched_batch(1)
    M = xyz.shape[0]
    rng = np.random.default_rng(6)
    feat = rng.standard_normal((M, 32)).astype(np.float32)
    feat[:, 0] = rng.uniform(5, 14, M).astype(np.float32)
    col = rng.uniform(0.05, 0.95, (M, 3)).astype(np.float32)
    ft, ct = torch.from_numpy(feat).cuda(), torch.from_numpy(col).cuda()
    g_rgb = rng.standard_normal((48, 3))
    g_feat = torch.empty_like(ft)
    g_col = torch.empty_like(ct)
    N.call("ff_composite_backward_rgb", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), 48, N.ptr(offsets),
           N.ptr(sidx), N.ptr(ft), 32, N.ptr(ct), None, N.ptr(torch.from_numpy(g_rgb).float().cuda()), N.ptr(g_feat),
           N.ptr(g_col), N.stream_ptr())
    gf = g_feat.cpu().numpy()
    assert np.all(gf[:, 1:] == 0)  # the head's channels are left for the head's backward
    rspec = O.RenderSpec(m.aabb.cpu().numpy(), rdesc.step, 256, rdesc.density_shift, rdesc.distance_scale,
                         rdesc.weight_thres, True)
    off = offsets.cpu().numpy()
    dirs = rays.cpu().numpy()[:, 3:6]
    fd64 = feat.astype(np.float64)
    c64 = col.astype(np.float64)

    def loss():
        return float((O.composite_rows(rspec, fd64, z, dist, off, dirs, rgb_rows=c64) * g_rgb).sum())

    _fd_check(loss, {"colour": c64}, {"colour": g_col.cpu().numpy()}, 40, rng, 1e-6, 1e-4, "composite colour")
    _fd_check(loss, {"feat": fd64}, {"feat": gf}, 40, rng, 1e-6, 1e-4, "composite density")
