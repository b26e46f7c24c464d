"""GPU parity of the proposal-sampler kernels against the oracle.

The proposal network has no reference implementation (parity unpinned for the network); the
pieces with reference semantics are pinned: resampling = sample_pdf (dataLoader/ray_utils.py:
132-174, itself pinned to golden vectors), compositing weights = raw2alpha (:82-88), the grid
lookup = trilinear grid_sample. The loss gradient is checked against FP64 central differences."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import need_gpu, rel_err
from oracle import ff_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


def make_sampler(reso=12, n_bins=64, n_fine=48, precision="fp32", learned=True):
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    torch.manual_seed(0)
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    return m, ProposalSampler(m, reso=reso, n_bins=n_bins, n_fine=n_fine, precision=precision, learned=learned)


def rays_np(n, seed=0):
    from factor_fields_gb300 import workloads as W
    return W.BlobScene(0).ray_pool(n, seed).astype(np.float32)


def test_encode_and_scatter_match_trilinear_grid_sample():
    from factor_fields_gb300 import _native as N
    m, s = make_sampler(reso=12)
    with torch.no_grad():
        s.grid.copy_(torch.randn(s.grid.shape, generator=torch.Generator().manual_seed(1)).cuda())
    rays = rays_np(64)
    rt = torch.from_numpy(rays).cuda()
    n, nb = rays.shape[0], s.n_bins
    feat = torch.empty(n * nb, 8, device="cuda")
    N.call("ff_proposal_encode", ctypes.byref(s.desc), N.ptr(s.grid), N.ptr(rt), n, N.ptr(feat), N.stream_ptr())
    # positions of the bin centres and the reference trilinear lookup (align_corners over the aabb)
    aabb = np.array([[-1.5] * 3, [1.5] * 3])
    t_in, t_out = O.proposal_segments(rays, aabb)
    seg = (t_out - t_in) / nb
    t = t_in[:, None] + (np.arange(nb)[None] + 0.5) * seg[:, None]
    x = rays[:, None, :3].astype(np.float64) + rays[:, None, 3:6] * t[..., None]
    coords = ((x - aabb[0]) / (aabb[1] - aabb[0]) * 2 - 1).reshape(-1, 3).astype(np.float32)
    grid = s.grid.detach().cpu().numpy().reshape(12, 12, 12, 8).transpose(3, 0, 1, 2)  # [C, D, H, W]
    ref = O.grid_sample_fwd(grid, coords, True, "zeros", "bilinear")
    assert rel_err(feat, ref) < 1e-4
    gfeat = torch.randn(n * nb, 8, generator=torch.Generator().manual_seed(2)).cuda()
    ggrid = torch.zeros_like(s.grid)
    N.call("ff_proposal_scatter", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(gfeat), N.ptr(ggrid), N.stream_ptr())
    refg = O.grid_sample_bwd(grid.shape, coords, gfeat.cpu().numpy(), True, "zeros", "bilinear")
    assert rel_err(ggrid.view(12, 12, 12, 8).permute(3, 0, 1, 2), refg) < 1e-4


@pytest.mark.parametrize("precision,n_rays,n_bins", [("bf16", 61, 64), ("fp32", 33, 96), ("bf16", 1, 32)])
def test_fused_head_matches_encode_mlp_scatter(precision, n_rays, n_bins):
    """ff_proposal_head_forward / _backward against the unfused composition: the grid lookup
    (ff_proposal_encode, pinned to trilinear grid_sample above), the MLP and its gradients in
    FP64, and the grid scatter of the FP64 feature gradient. Ragged sample counts (61 * 64,
    1 * 32 are not multiples of the 128-sample tile). BF16 tolerance: the first layer runs in
    split BF16 (hi + lo features and weights), dX takes BF16 W0, dW0 BF16 dH and features."""
    from factor_fields_gb300 import _native as N
    m, s = make_sampler(reso=12, n_bins=n_bins, precision=precision)
    gen = torch.Generator().manual_seed(7)
    with torch.no_grad():
        s.grid.copy_(torch.randn(s.grid.shape, generator=gen).cuda() * 0.5)
        l0, l1 = s.mlp.backbone
        l0.bias.copy_(torch.randn(64, generator=gen).cuda() * 0.2)
    st = N.stream_ptr()
    rt = torch.from_numpy(rays_np(n_rays, 9)).cuda()
    n, nb = n_rays, n_bins
    grid_r = s.grid_read()
    o = torch.empty(n * nb, 1, device="cuda")
    N.call("ff_proposal_head_forward", ctypes.byref(s.desc), N.ptr(grid_r), ctypes.byref(s.mlp_struct()), N.ptr(rt),
           n, N.ptr(o), st)
    feat = torch.empty(n * nb, 8, device="cuda")
    N.call("ff_proposal_encode", ctypes.byref(s.desc), N.ptr(grid_r), N.ptr(rt), n, N.ptr(feat), st)
    x = feat.double().cpu().requires_grad_(True)
    w0 = l0.weight.detach().double().cpu().requires_grad_(True)
    b0 = l0.bias.detach().double().cpu().requires_grad_(True)
    w1 = l1.weight.detach().double().cpu().requires_grad_(True)
    ref = torch.relu(x @ w0.T + b0) @ w1.T
    assert rel_err(o, ref.detach().numpy()) < 1e-3
    # samples with a hidden pre-activation within 1e-4 of 0 get no gradient: there the ReLU mask
    # of any float32 evaluation may differ from FP64's (a discrete jump, not a rounding error)
    pre = (x @ w0.T + b0).detach()
    g_o = torch.randn(n * nb, 1, generator=gen)
    g_o[(pre.abs() < 1e-4).any(1)] = 0
    ref.backward(g_o.double())
    s.zero_grad()
    g = N.FFMlpGrad()
    g.weight[0], g.bias[0], g.weight[1] = l0.weight.grad.data_ptr(), l0.bias.grad.data_ptr(), l1.weight.grad.data_ptr()
    g_o_d = g_o.cuda()
    N.call("ff_proposal_head_backward", ctypes.byref(s.desc), N.ptr(grid_r), ctypes.byref(s.mlp_struct()), N.ptr(rt),
           n, N.ptr(g_o_d), N.ptr(s.grid.grad), ctypes.byref(g), st)
    gx = x.grad.float().cuda().contiguous()
    ref_grid = torch.zeros_like(s.grid)
    N.call("ff_proposal_scatter", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(gx), N.ptr(ref_grid), st)
    torch.cuda.synchronize()
    assert rel_err(s.grid.grad, ref_grid.cpu().numpy()) < 1e-2
    assert rel_err(l0.weight.grad, w0.grad.numpy()) < 1e-2
    assert rel_err(l0.bias.grad, b0.grad.numpy()) < 1e-2
    assert rel_err(l1.weight.grad, w1.grad.numpy()) < 1e-3
    # no rays: nothing launched, success
    N.call("ff_proposal_head_forward", ctypes.byref(s.desc), N.ptr(grid_r), ctypes.byref(s.mlp_struct()), N.ptr(rt),
           0, None, st)


@pytest.mark.parametrize("n_rays,n_bins", [(61, 64), (33, 96), (1, 32), (257, 128)])
def test_head_infer_matches_fp64_composition(n_rays, n_bins):
    """ff_proposal_head_infer (the rendering form: one BF16 MMA pass per layer) against the FP64
    MLP of the grid lookup (ff_proposal_encode, pinned to trilinear grid_sample): within 2e-2 of
    the largest output, the BF16 tolerance; 96 bins take the division path of the bin index."""
    from factor_fields_gb300 import _native as N
    m, s = make_sampler(reso=12, n_bins=n_bins, precision="bf16")
    gen = torch.Generator().manual_seed(8)
    with torch.no_grad():
        s.grid.copy_(torch.randn(s.grid.shape, generator=gen).cuda() * 0.5)
        l0, l1 = s.mlp.backbone
        l0.bias.copy_(torch.randn(64, generator=gen).cuda() * 0.2)
    st = N.stream_ptr()
    rt = torch.from_numpy(rays_np(n_rays, 10)).cuda()
    n, nb = n_rays, n_bins
    grid_r = s.grid_read()
    o = torch.full((n * nb + 64, 1), float("nan"), device="cuda")  # rows past n * nb stay untouched
    N.call("ff_proposal_head_infer", ctypes.byref(s.desc), N.ptr(grid_r), ctypes.byref(s.mlp_struct()), N.ptr(rt),
           n, N.ptr(o), st)
    feat = torch.empty(n * nb, 8, device="cuda")
    N.call("ff_proposal_encode", ctypes.byref(s.desc), N.ptr(grid_r), N.ptr(rt), n, N.ptr(feat), st)
    torch.cuda.synchronize()
    x = feat.double().cpu()
    ref = torch.relu(x @ l0.weight.detach().double().cpu().T + l0.bias.detach().double().cpu()) @ \
        l1.weight.detach().double().cpu().T
    assert rel_err(o[:n * nb], ref.numpy()) < 2e-2
    assert torch.isnan(o[n * nb:]).all()
    # the training form agrees to its own (tighter) tolerance, so the two forms differ by rounding
    o_fwd = torch.empty(n * nb, 1, device="cuda")
    N.call("ff_proposal_head_forward", ctypes.byref(s.desc), N.ptr(grid_r), ctypes.byref(s.mlp_struct()), N.ptr(rt),
           n, N.ptr(o_fwd), st)
    assert rel_err(o_fwd, ref.numpy()) < 1e-3
    # float32 grids are refused (the rendering form reads a BF16 grid)
    m32, s32 = make_sampler(reso=12, n_bins=n_bins, precision="fp32")
    with pytest.raises(N.NativeError):
        N.call("ff_proposal_head_infer", ctypes.byref(s32.desc), N.ptr(s32.grid_read()),
               ctypes.byref(s32.mlp_struct()), N.ptr(rt), n, N.ptr(o), st)


def test_resample_is_sample_pdf():
    from factor_fields_gb300 import _native as N
    m, s = make_sampler()
    rays = rays_np(256, 3)
    rt = torch.from_numpy(rays).cuda()
    n, nb, nf = rays.shape[0], s.n_bins, s.n_fine
    rng = np.random.default_rng(4)
    o_p = (rng.standard_normal((n, nb)) * 3).astype(np.float32)
    o_p[:8] = -60  # flat histograms
    u = np.sort(rng.uniform(0, 1, (n, nf)).astype(np.float32), axis=1)
    w_p = torch.empty(n * nb, device="cuda")
    xyz = torch.empty(n * nf, 3, device="cuda")
    zd = torch.empty(n * nf, 2, device="cuda")
    bin_of = torch.empty(n * nf, dtype=torch.int32, device="cuda")
    o_t, u_t = torch.from_numpy(o_p).cuda(), torch.from_numpy(u).cuda()  # keep alive across the call
    N.call("ff_proposal_resample", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(o_t), None, N.ptr(u_t), N.ptr(w_p),
           N.ptr(xyz), N.ptr(zd), N.ptr(bin_of), N.stream_ptr())
    aabb = np.array([[-1.5] * 3, [1.5] * 3])
    t_in, t_out = O.proposal_segments(rays, aabb)
    seg = (t_out - t_in) / nb
    w_ref = O.proposal_weights(o_p, seg, s.desc.density_shift, s.desc.distance_scale)
    assert rel_err(w_p.view(n, nb), w_ref) < 1e-4
    edges = (t_in[:, None] + np.arange(nb + 1)[None] * seg[:, None]).astype(np.float32)
    ref_t = O.sample_pdf(edges, w_p.view(n, nb).cpu().numpy(), u)
    got_t = zd.view(n, nf, 2)[..., 0].cpu().numpy()
    # exclude samples whose u sits within rounding distance of a cdf knot (bin choice ambiguous)
    # or whose bin's cdf step sits at sample_pdf's `denom < 1e-5` switch (a discontinuity)
    w64 = w_p.view(n, nb).cpu().numpy().astype(np.float64) + 1e-5
    cdf = np.concatenate([np.zeros((n, 1)), np.cumsum(w64 / w64.sum(1, keepdims=True), 1)], 1)
    ok = np.min(np.abs(u[:, :, None] - cdf[:, None, :]), -1) > 1e-5
    ins = np.clip(np.stack([np.searchsorted(cdf[r], u[r], side="right") for r in range(n)]), 1, nb)
    step = np.take_along_axis(cdf, ins, 1) - np.take_along_axis(cdf, ins - 1, 1)
    ok &= np.abs(step - 1e-5) > 2e-6
    assert ok.mean() > 0.95
    # inside a bin t moves by bin_len * d(cdf) / step: float32 cdf sums of a different order
    # (up to ~4e-6 apart over 64 bins) are amplified by 1 / step in near-empty bins
    tol = 1e-4 * np.max(np.abs(ref_t)) + 4e-6 / step * seg[:, None]
    assert np.all((np.abs(got_t - ref_t) <= tol)[ok])
    # samples are sorted, inside their segment, dists consistent, positions on the ray
    assert np.all(np.diff(got_t, axis=1) >= -1e-6)
    dist = zd.view(n, nf, 2)[..., 1].cpu().numpy()
    assert np.allclose(dist[:, :-1], np.diff(got_t, axis=1), atol=1e-5)
    p = xyz.view(n, nf, 3).cpu().numpy()
    assert np.allclose(p, rays[:, None, :3] + rays[:, None, 3:6] * got_t[..., None], atol=1e-4)
    b = bin_of.view(n, nf).cpu().numpy()
    assert np.all((b >= 0) & (b < nb))


def _ball_mask(m, reso=32, seed=9):
    """An occupancy mask on m: six random balls in a reso^3 volume over m's aabb; returns the
    0/1 volume [D, H, W]."""
    from factor_fields_gb300.renderer import AlphaGridMask
    rng = np.random.default_rng(seed)
    g = (np.arange(reso) + 0.5) / reso * 2 - 1
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    vol = np.zeros((reso,) * 3, np.float32)
    for _ in range(6):
        c, r = rng.uniform(-0.7, 0.7, 3), rng.uniform(0.15, 0.4)
        vol[(xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2 < r * r] = 1
    m.alphaMask = AlphaGridMask(m.device, m.aabb.detach().clone(), torch.from_numpy(vol))
    return vol


def test_resample_occupied_keeps_the_occupied_rows():
    """ff_proposal_resample_occupied = ff_proposal_resample's rendering samples with the rows that
    fail the alpha-mask test (the oracle's occupancy_test, models/FactorFields.py:865-867) left
    out: counts, offsets and the kept rows bit-exact, in sample order."""
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300.renderer import render_desc
    m, s = make_sampler()
    vol = _ball_mask(m)
    rays = rays_np(300, 8)
    rt = torch.from_numpy(rays).cuda()
    n, nb, nf = rays.shape[0], s.n_bins, s.n_fine
    rng = np.random.default_rng(5)
    o_t = torch.from_numpy((rng.standard_normal((n, nb)) * 3).astype(np.float32)).cuda()
    st = N.stream_ptr()
    w_p = torch.empty(n * nb, device="cuda")
    xyz = torch.empty(n * nf, 3, device="cuda")
    zd = torch.empty(n * nf, 2, device="cuda")
    bin_of = torch.empty(n * nf, dtype=torch.int32, device="cuda")
    N.call("ff_proposal_resample", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(o_t), None, None, N.ptr(w_p),
           N.ptr(xyz), N.ptr(zd), N.ptr(bin_of), st)
    rd = render_desc(m, 1024, True)
    counts = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    offsets = torch.full((n + 1,), -1, dtype=torch.int64, device="cuda")
    wsb = int(N.lib().ff_scan_workspace_bytes(n))
    ws = torch.empty(max(wsb, 8), dtype=torch.uint8, device="cuda")
    xo = torch.full((n * nf, 3), float("nan"), device="cuda")
    zo = torch.full((n * nf, 2), float("nan"), device="cuda")
    N.call("ff_proposal_resample_occupied", ctypes.byref(s.desc), ctypes.byref(rd), N.ptr(rt), n, N.ptr(o_t), None,
           N.ptr(counts), N.ptr(offsets), N.ptr(ws), wsb, N.ptr(xo), N.ptr(zo), st)
    torch.cuda.synchronize()
    xa, za = xyz.cpu().numpy(), zd.cpu().numpy()
    occ = O.occupancy_test(vol, m.alphaMask.aabb.cpu().numpy(), xa).reshape(n, nf)
    assert 0.05 < occ.mean() < 0.95
    np.testing.assert_array_equal(counts.cpu().numpy(), occ.sum(1))
    off = np.concatenate([[0], np.cumsum(occ.sum(1))])
    np.testing.assert_array_equal(offsets.cpu().numpy(), off)
    keep = occ.reshape(-1)
    np.testing.assert_array_equal(xo[:off[-1]].cpu().numpy(), xa[keep])
    np.testing.assert_array_equal(zo[:off[-1]].cpu().numpy(), za[keep])
    # no rays: offsets[0] = 0 and nothing else
    offsets.fill_(-1)
    N.call("ff_proposal_resample_occupied", ctypes.byref(s.desc), ctypes.byref(rd), N.ptr(rt), 0, N.ptr(o_t), None,
           N.ptr(counts), N.ptr(offsets), N.ptr(ws), wsb, N.ptr(xo), N.ptr(zo), st)
    assert int(offsets[0]) == 0 and int(offsets[1]) == -1
    # without an occupancy volume the call is refused
    rd.occ_bits = None
    with pytest.raises(N.NativeError):
        N.call("ff_proposal_resample_occupied", ctypes.byref(s.desc), ctypes.byref(rd), N.ptr(rt), n, N.ptr(o_t),
               None, N.ptr(counts), N.ptr(offsets), N.ptr(ws), wsb, N.ptr(xo), N.ptr(zo), st)


def test_render_through_the_mask_equals_zero_density_samples():
    """A proposal render that evaluates only the occupied samples equals the render of every
    sample with the unoccupied samples' density set to zero (what the reference's alpha mask
    does, models/FactorFields.py:865-870): rgb and depth within 1e-5 (float32 compositing sums
    in a different lane order)."""
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300.renderer import field_eval, render_desc
    m, s = make_sampler(precision="bf16")
    s.cull_render = True
    m.cfg.renderer.density_shift = 0.0  # a random field with partly opaque rays
    vol = _ball_mask(m)
    rays = rays_np(512, 9)
    rt = torch.from_numpy(rays).cuda()
    n, nb, nf = rays.shape[0], s.n_bins, s.n_fine
    with torch.no_grad():
        rgb, depth = s.render(rt, is_train=False)
    # every sample, the unoccupied ones with zero density (softplus of -1e30 is 0)
    st = N.stream_ptr()
    o_p = torch.empty(n * nb, 1, device="cuda")
    N.call("ff_proposal_head_forward", ctypes.byref(s.desc), N.ptr(s.grid_read()), ctypes.byref(s.mlp_struct()),
           N.ptr(rt), n, N.ptr(o_p), st)
    w_p = torch.empty(n * nb, device="cuda")
    xyz = torch.empty(n * nf, 3, device="cuda")
    zd = torch.empty(n * nf, 2, device="cuda")
    bin_of = torch.empty(n * nf, dtype=torch.int32, device="cuda")
    N.call("ff_proposal_resample", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(o_p), None, None, N.ptr(w_p),
           N.ptr(xyz), N.ptr(zd), N.ptr(bin_of), st)
    basis_r, coeff_r, dt = m._read_buffers()
    job = {"fused": True, "fdesc": m.descriptor(dt), "basis_r": basis_r, "coeff_r": coeff_r}
    feat = field_eval(m, job, xyz)
    occ = O.occupancy_test(vol, m.alphaMask.aabb.cpu().numpy(), xyz.cpu().numpy())
    assert 0.05 < occ.mean() < 0.95
    feat[torch.from_numpy(~occ).cuda(), 0] = -1e30
    rd = render_desc(m, s.n_fine, True)
    offsets = torch.arange(n + 1, device="cuda", dtype=torch.int64) * nf
    rgb_ref = torch.empty(n, 3, device="cuda")
    depth_ref = torch.empty(n, device="cuda")
    w_f = torch.empty(n * nf, device="cuda")
    N.call("ff_composite_forward_zd", ctypes.byref(rd), N.ptr(rt), n, N.ptr(offsets), N.ptr(zd), N.ptr(feat),
           feat.shape[1], N.ptr(rgb_ref), N.ptr(depth_ref), N.ptr(w_f), st)
    torch.cuda.synchronize()
    acc = w_f.view(n, nf).sum(1).cpu().numpy()
    assert (acc > 0.1).mean() > 0.2 and (acc < 0.9).mean() > 0.2, (shift, acc.mean())  # partly opaque rays
    assert float((rgb - rgb_ref).abs().max()) < 1e-5
    assert float((depth - depth_ref).abs().max()) < 1e-5 * float(depth_ref.abs().max())


@pytest.mark.parametrize("nf", [32, 64, 128])
def test_fused_render_equals_field_forward_and_compositing(nf):
    """ff_field_render_fixed (field forward with the compositing in its epilogue) against
    ff_field_mlp_forward + ff_composite_forward_zd on the same resampled rays: rgb and depth
    within 1e-5 (rays of 64 and 128 samples are summed per 32-sample chunk). 301 rays: the last
    tile is partly past the end. Through the sampler, a render without gradients takes the fused
    path and gives the unfused render's colours."""
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300 import functional as FN
    from factor_fields_gb300.renderer import field_eval, render_desc
    m, s = make_sampler(n_fine=nf, precision="bf16")
    gen = torch.Generator().manual_seed(12)
    rays = rays_np(301, 11)
    rt = torch.from_numpy(rays).cuda()
    n, nb = rays.shape[0], s.n_bins
    st = N.stream_ptr()
    o_t = (torch.randn(n * nb, generator=gen) * 3).cuda()
    xyz = torch.empty(n * nf, 3, device="cuda")
    zd = torch.empty(n * nf, 2, device="cuda")
    N.call("ff_proposal_resample", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(o_t), None, None, None, N.ptr(xyz),
           N.ptr(zd), None, st)
    basis_r, coeff_r, dt = m._read_buffers()
    job = {"fused": True, "fdesc": m.descriptor(dt), "basis_r": basis_r, "coeff_r": coeff_r}
    feat = field_eval(m, job, xyz)
    offsets = torch.arange(n + 1, device="cuda", dtype=torch.int64) * nf
    rgb_ref = torch.empty(n, 3, device="cuda")
    depth_ref = torch.empty(n, device="cuda")
    w_f = torch.empty(n * nf, device="cuda")
    for shift in (0.0, -2.0, -3.0, -4.0, -5.0, -6.0, -7.0, -8.0, -10.0):  # a density with partly opaque rays
        m.cfg.renderer.density_shift = shift
        rd = render_desc(m, nf, True)
        N.call("ff_composite_forward_zd", ctypes.byref(rd), N.ptr(rt), n, N.ptr(offsets), N.ptr(zd), N.ptr(feat),
               feat.shape[1], N.ptr(rgb_ref), N.ptr(depth_ref), N.ptr(w_f), st)
        if 0.3 < float(w_f.view(n, nf).sum(1).mean()) < 0.7:
            break
    lm = m.linear_mat
    ws, bs = lm.weights()
    mlp = FN.mlp_struct(ws, bs, lm.in_dim, lm.hidden_dim, lm.out_dim)
    rgb = torch.full((n, 3), float("nan"), device="cuda")
    depth = torch.full((n,), float("nan"), device="cuda")
    N.call("ff_field_render_fixed", ctypes.byref(job["fdesc"]), N.ptr(basis_r), N.ptr(coeff_r), ctypes.byref(mlp),
           ctypes.byref(rd), N.ptr(rt), N.ptr(xyz), N.ptr(zd), n, nf, N.ptr(rgb), N.ptr(depth), st)
    torch.cuda.synchronize()
    acc = w_f.view(n, nf).sum(1).cpu().numpy()
    assert (acc > 0.2).mean() > 0.2 and (acc < 0.8).mean() > 0.2  # partly opaque rays
    assert float((rgb - rgb_ref).abs().max()) < 1e-5
    assert float((depth - depth_ref).abs().max()) < 1e-5 * float(depth_ref.abs().max())
    # the sampler: fused when no gradients are wanted, the same colours as the two-call render
    s.render_fine = nf
    with torch.no_grad():
        rgb_f, depth_f = s.render(rt, is_train=False)
        assert s._job["w_f"] is None  # the fused path ran
        s.fuse_render = False
        rgb_u, depth_u = s.render(rt, is_train=False)
        assert s._job["w_f"] is not None
    assert float((rgb_f - rgb_u).abs().max()) < 1e-5
    assert float((depth_f - depth_u).abs().max()) < 1e-5 * float(depth_u.abs().max())
    # unsupported sample counts and heads are refused
    with pytest.raises(N.NativeError):
        N.call("ff_field_render_fixed", ctypes.byref(job["fdesc"]), N.ptr(basis_r), N.ptr(coeff_r),
               ctypes.byref(mlp), ctypes.byref(rd), N.ptr(rt), N.ptr(xyz), N.ptr(zd), n // 2, 48, N.ptr(rgb),
               N.ptr(depth), st)


def test_fused_render_full_view_equals_two_call_render():
    """At the evaluation shape (one 400x400 view: 160,000 rays x 32 samples), the sampler's fused
    render (ff_field_render_fixed) gives the two-call render's colours and depths (1e-5)."""
    from factor_fields_gb300 import workloads as W
    m, s = make_sampler(reso=64, n_fine=48, precision="bf16")
    m.cfg.renderer.density_shift = -4.0  # a denser initial field: some rays opaque, some not
    s.render_fine = 32
    rays = torch.from_numpy(W.BlobScene(0).ray_pool(160000, 6, views=[7])).float().cuda()
    with torch.no_grad():
        rgb_f, depth_f = s.render(rays, is_train=False)
        assert s._job["w_f"] is None
        s.fuse_render = False
        rgb_u, depth_u = s.render(rays, is_train=False)
    assert float((rgb_f - rgb_u).abs().max()) < 1e-5
    assert float((depth_f - depth_u).abs().max()) < 1e-5 * float(depth_u.abs().max())
    assert float(rgb_u.std()) > 1e-3  # not a blank image


def test_proposal_loss_gradient_matches_finite_differences():
    from factor_fields_gb300 import _native as N
    m, s = make_sampler()
    rays = rays_np(32, 5)
    rt = torch.from_numpy(rays).cuda()
    n, nb, nf = rays.shape[0], s.n_bins, s.n_fine
    rng = np.random.default_rng(6)
    o_p = (rng.standard_normal((n, nb)) * 2 - 1).astype(np.float32)
    w_f = rng.uniform(0, 0.08, (n, nf)).astype(np.float32)
    bin_of = rng.integers(0, nb, (n, nf)).astype(np.int32)
    g_o = torch.empty(n * nb, device="cuda")
    loss = torch.zeros(1, device="cuda")
    o_t, wf_t, b_t = (torch.from_numpy(a).cuda() for a in (o_p, w_f, bin_of))  # alive across the call
    N.call("ff_proposal_loss", ctypes.byref(s.desc), N.ptr(rt), n, N.ptr(o_t), N.ptr(wf_t), N.ptr(b_t), 1.0 / n,
           N.ptr(loss), N.ptr(g_o), N.stream_ptr())
    t_in, t_out = O.proposal_segments(rays, np.array([[-1.5] * 3, [1.5] * 3]))
    ref_loss, ref_g = O.proposal_loss(o_p, (t_out - t_in) / nb, s.desc.density_shift, s.desc.distance_scale, w_f,
                                      bin_of, 1.0 / n)
    assert abs(float(loss) - ref_loss) <= 1e-4 * abs(ref_loss)
    assert rel_err(g_o.view(n, nb), ref_g) < 1e-3


def test_proposal_matches_plain_sampler_with_far_fewer_samples():
    """What the trained proposal network gains over the method without it (the reference's
    plain uniform sampler, up to 1024 samples per ray with occupancy pruning): after the same
    training (1500 steps of 4096 rays; the field sees 48 stratified samples per ray in the
    proposal configuration against ~125 live samples in the plain one), rendering with 48
    proposal samples per ray is at least as accurate against the FP64 ground truth (within
    0.1 dB; measured +0.3 / +1.2 dB). Runs of this comparison differ by up to ~0.5 dB from the
    seed alone, so it is made on two seeds and a 10-view test set (their mean)."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    from factor_fields_gb300.renderer import march, render_desc
    from factor_fields_gb300.train import RadianceFieldTrainer
    scene = W.BlobScene(0)
    pool = torch.from_numpy(scene.ray_pool(1 << 17, 5)).float()
    gt = scene.render_gt(pool.double().numpy(), n_steps=512).cuda()
    test = torch.from_numpy(scene.ray_pool(1 << 14, 6, views=list(range(10)))).float()
    gtt = scene.render_gt(test.double().numpy(), n_steps=512).cuda()
    pool, test = pool.cuda(), test.cuda()
    iters = 1500
    diffs, res = [], {}
    for seed in (1, 2):
        for kind in ("plain", "proposal"):
            torch.manual_seed(seed)
            m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
            sampler = ProposalSampler(m, seed=seed) if kind == "proposal" else None
            tr = RadianceFieldTrainer(m, n_samples=1024, n_iters=iters, sampler=sampler)
            g = torch.Generator(device="cuda").manual_seed(seed)
            for it in range(iters):
                idx = torch.randint(0, pool.shape[0], (4096,), device="cuda", generator=g)
                tr.step(pool[idx], gt[idx])
                if kind == "plain" and it in (300, 750):
                    m.updateAlphaMask((128, 128, 128), is_update_alphaMask=True, times=1)
            res[(seed, kind)] = tr.psnr(test, gtt)
            if kind == "plain":
                offsets, _, _ = march(m, test, None, render_desc(m, 1024, True))
                res[(seed, "plain_samples")] = float(offsets[-1]) / test.shape[0]
        diffs.append(res[(seed, "proposal")] - res[(seed, "plain")])
    assert sum(diffs) / len(diffs) >= -0.1, res
    assert min(res[(s, "plain_samples")] for s in (1, 2)) >= 2 * 48, res  # ~125 live samples per ray



def test_trainer_graph_step_matches_eager_step():
    """RadianceFieldTrainer.graph_step (the step captured in a CUDA graph and replayed) gives the
    eager step's loss and gradients on the same batch (fixed jitter), and picks up parameter
    updates made between replays (the BF16 read copies are refreshed in place)."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    from factor_fields_gb300.train import RadianceFieldTrainer
    scene = W.BlobScene(0)
    rays = torch.from_numpy(scene.ray_pool(2048, 11)).float()
    gt = scene.render_gt(rays.double().numpy(), n_steps=256).cuda().float()
    rays = rays.cuda()
    torch.manual_seed(0)
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    # per-ray jitter (fixed below) so that the eager and the replayed step draw the same samples
    tr = RadianceFieldTrainer(m, sampler=ProposalSampler(m, sample_jitter=False), n_iters=100)
    for _ in range(30):
        tr.step(rays, gt)
    tr.jitter = torch.rand(rays.shape[0], device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    params = [m.basis_flat, m.coeff_flat] + list(m.linear_mat.parameters()) + tr.sampler.params
    for rep in range(2):
        loss_e = float(tr.step(rays, gt, optimize=False))
        grads_e = [p.grad.clone() for p in params]
        loss_g = float(tr.graph_step(rays, gt))
        torch.cuda.synchronize()
        assert abs(loss_g - loss_e) <= 1e-5 * abs(loss_e)
        for p, ge in zip(params, grads_e):
            assert rel_err(p.grad, ge) < 1e-3
        tr.opt.step()  # parameters change between replays
        tr.sampler.step()
