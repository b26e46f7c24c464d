"""GPU parity of the renderer (march / compact / composite + SH-2 head) against the reference's
golden renders and the FP64 oracle.

Bit-exact: live-sample set and order (the reference's xyz_sampled[ray_valid]), sample
positions, occupancy decisions. Float32 drop-in path: rgb / depth 1e-5, gradients 1e-4, also
element-wise (gpu_util.close).
Fused BF16 path: 2e-2 / 3e-2 against the oracle of the BF16-stored model."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import close, load_golden, model_from_golden, need_gpu, rel_err, render_cases
from oracle import ff_oracle as O

pytestmark = pytest.mark.gpu

CASES = [c for c in render_cases() if "mlp_head" not in c]


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
    assert close(rgb, d["rgb"], 1e-5)
    assert close(depth, d["depth"], 1e-5)
    (rgb * torch.from_numpy(d["g_rgb"]).cuda()).sum().backward()
    for l in range(6):
        assert close(m.layout.basis_view(m.basis_flat.grad, l), d[f"grad_basis{l}"], 1e-4), l
    assert close(m.layout.coeff_view(m.coeff_flat.grad, 0), d["grad_coeffs0"], 1e-4)
    for i, lin in enumerate(m.linear_mat.backbone):
        assert close(lin.weight.grad, d[f"grad_mlp_w{i}"], 1e-4)
        if lin.bias is not None:
            assert close(lin.bias.grad, d[f"grad_mlp_b{i}"], 1e-4)


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
                        g_rgb=g_rgb)
    for l in range(6):
        assert rel_err(m.layout.basis_view(m.basis_flat.grad, l)[0], res["grad_basis"][l]) < 3e-2, l
    assert rel_err(m.layout.coeff_view(m.coeff_flat.grad, 0)[0], res["grad_coeff"]) < 3e-2


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
