"""GPU parity of the renderer (march / compact / composite + SH-2 head) against the reference's
golden renders and the FP64 oracle.

Bit-exact: live-sample set and order (the reference's xyz_sampled[ray_valid]), sample
positions, occupancy decisions. Float32 drop-in path: rgb / depth 1e-5, gradients 1e-4, also
element-wise (gpu_util.assert_close; gradients with the RENDER_GRAD_FLOOR floor).
Fused BF16 path: 2e-2 / 3e-2 against the oracle of the BF16-stored model."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import (RENDER_GRAD_FLOOR, assert_close, load_golden, model_from_golden, need_gpu, rel_err,
                      render_cases)
from oracle import ff_oracle as O

pytestmark = pytest.mark.gpu

CASES = render_cases()


def head_oracle(m, meta, bf=None):
    """The oracle's MLPRender_Fea parameters of model m (None for the SH-2 head)."""
    if meta.get("head") != "mlp":
        return None
    conv = bf or (lambda t: t.detach().cpu().numpy())
    ws, bs = m.renderModule.params()
    r = meta["cfg"]["renderer"]
    return {"w": [conv(w) for w in ws], "b": [None if b is None else b.detach().cpu().numpy() for b in bs],
            "view_pe": r["view_pe"], "fea_pe": r["fea_pe"]}


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


def setup(case, precision="fp32"):
    from factor_fields_gb300.renderer import AlphaGridMask
    d, meta = load_golden(case)
    m = model_from_golden(d, meta, precision=precision)
    if "alpha_volume" in d:
        m.alphaMask = AlphaGridMask(m.device, m.aabb, torch.from_numpy(d["alpha_volume"]).cuda())
    rays = torch.from_numpy(d["rays"]).cuda()
    jitter = torch.from_numpy(d["u"][:, 0]).cuda() if meta["jitter"] else None
    return d, meta, m, rays, jitter


@pytest.mark.parametrize("case", CASES)
def test_march_is_bit_exact(case):
    from factor_fields_gb300.renderer import march, render_desc
    d, meta, m, rays, jitter = setup(case)
    ns = int(d["n_samples"])
    offsets, xyz, sidx = march(m, rays, jitter, render_desc(m, ns, meta["white_bg"]))
    offsets, xyz, sidx = offsets.cpu().numpy(), xyz.cpu().numpy(), sidx.cpu().numpy()
    valid = np.zeros_like(d["valid"])
    for r in range(valid.shape[0]):
        valid[r, sidx[offsets[r]:offsets[r + 1]]] = True
    np.testing.assert_array_equal(valid, d["valid"])
    # positions: the reference's rays_o + rays_d * z in float32, in ray-major order
    z = d["z_vals"]
    o, dd = d["rays"][:, None, :3], d["rays"][:, None, 3:6]
    ref_xyz = (o + (dd * z[..., None]).astype(np.float32)).astype(np.float32)[d["valid"]]
    np.testing.assert_array_equal(xyz, ref_xyz)
    assert np.all(np.diff(sidx[offsets[0]:offsets[1]]) > 0)


@pytest.mark.parametrize("case", CASES)
def test_render_dropin_matches_reference(case):
    d, meta, m, rays, jitter = setup(case, "fp32")
    ns = int(d["n_samples"])
    rgb, depth, _ = m(rays, white_bg=meta["white_bg"], is_train=False, N_samples=ns, jitter=jitter, fused=False)
    assert_close(rgb, d["rgb"], 1e-5)
    assert_close(depth, d["depth"], 1e-5)
    (rgb * torch.from_numpy(d["g_rgb"]).cuda()).sum().backward()
    for l in range(6):
        assert_close(m.layout.basis_view(m.basis_flat.grad, l), d[f"grad_basis{l}"], 1e-4, RENDER_GRAD_FLOOR,
                     what=f"level {l}")
    assert_close(m.layout.coeff_view(m.coeff_flat.grad, 0), d["grad_coeffs0"], 1e-4, RENDER_GRAD_FLOOR)
    for i, lin in enumerate(m.linear_mat.backbone):
        assert_close(lin.weight.grad, d[f"grad_mlp_w{i}"], 1e-4, RENDER_GRAD_FLOOR)
        if lin.bias is not None:
            assert_close(lin.bias.grad, d[f"grad_mlp_b{i}"], 1e-4, RENDER_GRAD_FLOOR)
    if meta.get("head") == "mlp":  # MLPRender_Fea's own parameters
        for i, lin in enumerate(m.renderModule.mlp):
            assert_close(lin.weight.grad, d[f"grad_rm_w{i}"], 1e-4, RENDER_GRAD_FLOOR, what=f"head w{i}")
            if lin.bias is not None:
                assert_close(lin.bias.grad, d[f"grad_rm_b{i}"], 1e-4, RENDER_GRAD_FLOOR, what=f"head b{i}")


@pytest.mark.parametrize("case", CASES)
def test_render_fused_bf16(case):
    d, meta, m, rays, jitter = setup(case, "bf16")
    ns = int(d["n_samples"])
    rgb, depth, _ = m(rays, white_bg=meta["white_bg"], is_train=False, N_samples=ns, jitter=jitter, fused=True)
    assert rel_err(rgb, d["rgb"]) < 2e-2
    assert rel_err(depth, d["depth"]) < 2e-2
    g_rgb = d["g_rgb"]
    (rgb * torch.from_numpy(g_rgb).cuda()).sum().backward()
    # oracle of the BF16-stored model (grids and MLP weights rounded to BF16)
    fspec = O.FieldSpec.from_meta(meta)
    bf = lambda t: t.detach().to(torch.bfloat16).float().cpu().numpy()  # noqa: E731
    bg = [bf(b[0]) for b in m.basises]
    cg = bf(m.coeffs[0][0])
    ws, bs = m.linear_mat.weights()
    r = meta["cfg"]["renderer"]
    rspec = O.RenderSpec(meta["aabb"], d["step_size"], ns, r["density_shift"], r["distance_scale"],
                         r["rayMarch_weight_thres"], meta["white_bg"])
    res = O.render_rays(fspec, rspec, bg, cg, [bf(w) for w in ws], [None if b is None else b.detach().cpu().numpy()
                                                                   for b in bs],
                        d["rays"], jitter=d["u"] if meta["jitter"] else None, alpha_volume=d.get("alpha_volume"),
                        g_rgb=g_rgb, head=head_oracle(m, meta, bf))
    for l in range(6):
        assert rel_err(m.layout.basis_view(m.basis_flat.grad, l)[0], res["grad_basis"][l]) < 3e-2, l
    assert rel_err(m.layout.coeff_view(m.coeff_flat.grad, 0)[0], res["grad_coeff"]) < 3e-2
    if meta.get("head") == "mlp":
        for i, lin in enumerate(m.renderModule.mlp):
            assert rel_err(lin.weight.grad, res["grad_head_w"][i]) < 3e-2, i


def test_render_ray_chunks_and_training_mode():
    """render_ray (renderer.py:8) chunking equals one-shot rendering; training mode returns coeffs."""
    from factor_fields_gb300.renderer import render_ray
    d, meta, m, rays, _ = setup("render_sh_plain.npz")
    ns = int(d["n_samples"])
    rgb1, depth1 = render_ray(rays, m, chunk=7, N_samples=ns, white_bg=True)
    rgb2, depth2, _ = m(rays, white_bg=True, N_samples=ns, fused=False)
    assert torch.allclose(rgb1, rgb2, atol=1e-6) and torch.allclose(depth1, depth2, atol=1e-5)
    out = render_ray(rays, m, chunk=16, N_samples=ns, white_bg=True, is_train=True)
    assert len(out) == 3 and out[0].shape == (rays.shape[0], 3)


def test_scan_edge_cases():
    """The exclusive scan over ray counts: empty, ragged and multi-block sizes."""
    from factor_fields_gb300 import _native as N
    for n in (0, 1, 5, 4095, 4096, 4097, 100003):
        counts = torch.randint(0, 1000, (n,), dtype=torch.int32, device="cuda")
        offsets = torch.empty(n + 1, dtype=torch.int64, device="cuda")
        wsb = N.lib().ff_scan_workspace_bytes(n)
        ws = torch.empty(max(wsb, 8), dtype=torch.uint8, device="cuda")
        N.call("ff_scan_counts", N.ptr(counts) if n else None, n, N.ptr(offsets), N.ptr(ws), wsb, N.stream_ptr())
        ref = torch.zeros(n + 1, dtype=torch.int64)
        ref[1:] = torch.cumsum(counts.cpu().long(), 0)
        assert torch.equal(offsets.cpu(), ref), n


def test_direct_grad_accumulation_matches_autograd_returns():
    """Render gradients accumulated straight into .grad (the default) equal the ones returned
    through autograd (accumulate_grad_directly = False), and they accumulate over two
    backward passes like autograd's."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    rays = torch.from_numpy(W.BlobScene(0).ray_pool(512, 3)).float().cuda()
    jit = torch.rand(512, device="cuda", generator=torch.Generator(device="cuda").manual_seed(0))
    res = []
    for direct in (True, False):
        torch.manual_seed(0)
        m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
        m.accumulate_grad_directly = direct
        for _ in range(2):
            rgb, _, _ = m(rays, white_bg=True, is_train=True, N_samples=256, jitter=jit)
            (rgb * rgb).sum().backward()
        res.append([p.grad.clone() for p in [m.basis_flat, m.coeff_flat] + list(m.linear_mat.parameters())])
    for a, b in zip(*res):
        assert rel_err(a, b) < 1e-5


def test_mlp_head_alone_matches_oracle():
    """MLPRender_Fea.forward(viewdirs, features) on the drop-in kernels against the FP64 oracle,
    4,099 samples (ragged against the GEMM tiles), nerf.yaml sizes (C = 31, 128 hidden, view_pe
    6, fea_pe 2), forward 1e-5 and gradients 1e-4, element-wise."""
    from factor_fields_gb300.renderer import MLPRender_Fea
    torch.manual_seed(0)
    head = MLPRender_Fea(31, num_layers=3, hidden_dim=128, viewpe=6, feape=2).cuda()
    g = torch.Generator().manual_seed(1)
    feat = (torch.randn(4099, 31, generator=g) * 0.7).cuda().requires_grad_(True)
    dirs = torch.nn.functional.normalize(torch.randn(4099, 3, generator=g), dim=-1).cuda()
    g_rgb = torch.randn(4099, 3, generator=g).cuda()
    rgb = head(dirs, feat)
    (rgb * g_rgb).sum().backward()
    ws, bs = head.params()
    wn = [w.detach().cpu().numpy() for w in ws]
    bn = [None if b is None else b.detach().cpu().numpy() for b in bs]
    fn, dn, gn = feat.detach().cpu().numpy(), dirs.cpu().numpy(), g_rgb.cpu().numpy()
    assert_close(rgb, O.render_head_fwd(wn, bn, fn, dn, 6, 2), 1e-5, what="rgb")
    g_feat, gw, gb = O.render_head_bwd(wn, bn, fn, dn, 6, 2, gn)
    assert_close(feat.grad, g_feat, 1e-4, what="dL/dfeat")
    for i in range(3):
        assert_close(ws[i].grad, gw[i], 1e-4, what=f"w{i}")
        if bs[i] is not None:
            assert_close(bs[i].grad, gb[i], 1e-4, what=f"b{i}")


def _head_oracle_args(head, feat, dirs, g_rgb, bf16):
    ws, bs = head.params()
    conv = (lambda t: t.detach().to(torch.bfloat16).float().cpu().numpy()) if bf16 else \
        (lambda t: t.detach().cpu().numpy())
    return ([conv(w) for w in ws], [None if b is None else b.detach().cpu().numpy() for b in bs],
            feat.detach().cpu().numpy(), dirs.cpu().numpy(), g_rgb.cpu().numpy())


def _kink_free(wn, bn, fsel, dsel, band=5e-5):
    """Samples none of whose 256 hidden pre-activations (FP64 oracle) lies within `band` of the
    ReLU kink. There the exact gradient is a step function of the input: any rounding can put the
    sample on the other side and move its input gradient by a whole term, so the per-sample
    comparison is made on the others (~5% of random samples excluded). The band is ~20x the
    pre-activation error of the split-BF16 operands (~2.5e-6 here)."""
    x = O.render_head_input(fsel, dsel, 6, 2)
    p0 = x @ np.asarray(wn[0], np.float64).T + bn[0]
    p1 = np.maximum(p0, 0) @ np.asarray(wn[1], np.float64).T + bn[1]
    return (np.abs(p0).min(1) > band) & (np.abs(p1).min(1) > band)


@pytest.mark.parametrize("channels", [27, 31])
def test_mlp_head_tensor_cores_match_oracle(channels):
    """The tcgen05 head (ff_render_head_forward_tc / _backward_tc) through the C ABI against the
    FP64 oracle of the BF16-stored head (weights rounded to BF16): forward 2e-2, gradients 3e-2,
    on ~1,000 samples scattered over 1,500 rows (ragged last tile) of a 28 / 32-wide feature
    buffer, the samples within 5e-5 of a ReLU kink left out (_kink_free); rows that are not listed
    stay untouched. Calls twice: results repeat (rgb bit-identical; gradients to float32 rounding,
    since they are summed with atomics; the kernel's TMEM accumulators start from zero on every
    launch)."""
    from factor_fields_gb300.renderer import MLPRender_Fea, head_backward, head_forward
    torch.manual_seed(1)
    head = MLPRender_Fea(channels, num_layers=3, hidden_dim=128, viewpe=6, feape=2).cuda()
    g = torch.Generator().manual_seed(2)
    M, n = 1500, 1000
    feat = (torch.randn(M, channels + 1, generator=g) * 0.8).cuda()
    rays = torch.randn(M, 6, generator=g).cuda()
    rays[:, 3:6] = torch.nn.functional.normalize(rays[:, 3:6], dim=-1)
    perm = torch.randperm(M, generator=g)[:n]
    ray_pick = torch.randint(0, M, (n,), generator=g)
    g_rgb = torch.randn(M, 3, generator=g).cuda()
    wn0, bn0, fn0, dn0, _ = _head_oracle_args(head, feat.cpu()[perm, 1:], rays.cpu()[ray_pick, 3:6],
                                              g_rgb.cpu()[perm], bf16=True)
    keep = torch.from_numpy(_kink_free(wn0, bn0, fn0, dn0))
    assert int(keep.sum()) > 0.9 * n
    app_idx = perm[keep].to(torch.int32).cuda()
    app_ray = ray_pick[keep].to(torch.int32).cuda()
    n = app_idx.shape[0]
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    outs = []
    for _ in range(2):
        rgb = torch.full((M, 3), -7.0, device="cuda")
        head_forward(head, feat, rays, app_idx, app_ray, rgb, tc=True, status=status)
        g_feat = torch.full_like(feat, -7.0)
        for p in head.parameters():
            p.grad = None
        gw, gb = head_backward(head, feat, rays, app_idx, app_ray, g_rgb, g_feat, direct=False, tc=True,
                               status=status)
        torch.cuda.synchronize()
        assert int(status) == 0
        outs.append((rgb.clone(), g_feat.clone(), [w.clone() for w in gw], [b.clone() if b is not None else None
                                                                          for b in gb]))
    idx = app_idx.long().cpu()
    ray = app_ray.long().cpu()
    fsel = feat.cpu()[idx, 1:]
    dsel = rays.cpu()[ray, 3:6]
    gsel = g_rgb.cpu()[idx]
    wn, bn, fn, dn, gn = _head_oracle_args(head, fsel, dsel, gsel, bf16=True)
    ref_rgb = O.render_head_fwd(wn, bn, fn, dn, 6, 2)
    ref_gf, ref_gw, ref_gb = O.render_head_bwd(wn, bn, fn, dn, 6, 2, gn)
    rgb, g_feat, gw, gb = outs[0]
    assert rel_err(rgb.cpu()[idx], ref_rgb) < 2e-2
    unlisted = torch.ones(M, dtype=torch.bool)
    unlisted[idx] = False
    assert bool((rgb.cpu()[unlisted] == -7.0).all()) and bool((g_feat.cpu()[unlisted] == -7.0).all())
    assert bool((g_feat.cpu()[idx, 0] == -7.0).all())  # channel 0 (density) is not the head's
    assert rel_err(g_feat.cpu()[idx, 1:], ref_gf) < 3e-2
    for i in range(3):
        assert rel_err(gw[i], ref_gw[i]) < 3e-2, i
        if gb[i] is not None:
            assert rel_err(gb[i], ref_gb[i]) < 3e-2, i
    r2 = outs[1]
    assert torch.equal(r2[0], outs[0][0])
    assert rel_err(r2[1].cpu()[idx, 1:], outs[0][1].cpu()[idx, 1:]) < 1e-5  # per-row sums: shared-memory atomics
    for a, b in zip(r2[2], outs[0][2]):
        assert rel_err(a, b) < 1e-5  # weight-gradient atomics: summation order may differ


def test_static_render_and_plain_graph_step():
    """Rendering without host synchronisation (static=True: live-sample buffers sized for every
    sample slot, the count read on the device by ff_field_mlp_*_counted) equals the default path
    (rgb / depth bit-identical, gradients to float32 rounding), and the plain sampler's training
    step replays from a CUDA graph with the same loss and gradients as the eager step."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.train import RadianceFieldTrainer
    torch.manual_seed(0)
    m = FactorFields(W.field_cfg("cfg2"), device="cuda", precision="bf16")
    rays = torch.from_numpy(W.BlobScene(0).ray_pool(1024, 21)).float().cuda()
    jit = torch.rand(1024, generator=torch.Generator().manual_seed(2)).cuda()
    res = []
    for static in (False, True):
        m.zero_grad(set_to_none=True)
        rgb, depth, _ = m(rays, white_bg=True, is_train=True, N_samples=1024, jitter=jit, static=static)
        (rgb * rgb).sum().backward()
        res.append((rgb.detach().clone(), depth.clone(), m.basis_flat.grad.clone(), m.coeff_flat.grad.clone(),
                    m.linear_mat.backbone[0].weight.grad.clone()))
    assert torch.equal(res[0][0], res[1][0]) and torch.equal(res[0][1], res[1][1])
    for a, b in zip(res[0][2:], res[1][2:]):
        assert rel_err(a, b) < 1e-6
    gt = torch.rand(1024, 3, generator=torch.Generator().manual_seed(3)).cuda()
    tr = RadianceFieldTrainer(m, n_samples=1024)
    tr.jitter = jit
    params = [m.basis_flat, m.coeff_flat] + list(m.linear_mat.parameters())
    l_eager = float(tr.step(rays, gt, optimize=False))
    g_eager = [p.grad.clone() for p in params]
    for _ in range(2):  # capture, then a replay
        l_graph = float(tr.graph_step(rays, gt))
    g_graph = [p.grad.clone() for p in params]
    assert abs(l_graph - l_eager) <= 1e-6 * abs(l_eager)
    for a, b in zip(g_eager, g_graph):
        assert rel_err(b, a) < 1e-5
