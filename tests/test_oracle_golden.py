"""Pin the CPU oracle against golden vectors produced by running the reference itself.

CPU only. The fixtures come from tests/golden/make_golden.py (reference import + stubs).
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle import ff_oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    d = dict(np.load(os.path.join(GOLD, name)))
    meta = json.loads(str(d.pop("meta"))) if "meta" in d else None
    return d, meta


def grids(d, n_levels):
    return [d[f"basis{i}"][0] for i in range(n_levels)], d["coeffs0"][0]


def mlp_params(d, prefix="mlp"):
    ws, bs, i = [], [], 0
    while f"{prefix}_w{i}" in d:
        ws.append(d[f"{prefix}_w{i}"])
        bs.append(d.get(f"{prefix}_b{i}"))
        i += 1
    return ws, bs


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)


FIELD_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLD, "field_*.npz")))
RENDER_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLD, "render_*.npz")))


def test_fixture_inventory():
    assert len(FIELD_CASES) >= 7 and len(RENDER_CASES) >= 4


def test_mapping_bit_exact():
    d, _ = load("primitives.npz")
    for mode in ("sawtooth", "triangle"):
        got = O.grid_mapping(d["map_pos"], d["map_freqs"], np.float32([-1, -1, -1]), np.float32(2.0), mode)
        np.testing.assert_array_equal(got, d[f"map_{mode}"])


def test_dct_init_matches_reference():
    d, _ = load("primitives.npz")
    for dim in (2, 3):
        for c, r in zip([4, 4, 4, 2, 2, 2], [32, 51, 70, 89, 108, 128]):
            k = O.dct_dict(int(np.power(c, 1.0 / dim) + 1), r, c, dim)
            np.testing.assert_array_equal(k[:, :64], d[f"dct{dim}_{c}_{r}_head"])
            assert abs(k.astype(np.float64).sum() - d[f"dct{dim}_{c}_{r}_sum"]) <= 1e-9 * max(1, abs(d[f"dct{dim}_{c}_{r}_sum"]))


def test_n_to_reso():
    d, _ = load("primitives.npz")
    for (n, dim), ref in zip(d["n2r_cases"], d["n2r_out"]):
        assert O.n_to_reso(int(n), [[-1.5] * dim, [1.5] * dim])[0] == ref


def test_config_shapes_and_init():
    """Derived sizes of the benchmark configurations and checksums of the DCT initialisation."""
    with open(os.path.join(GOLD, "config_shapes.json")) as f:
        shapes = json.load(f)
    for key, in_dim in (("cfg0", 2), ("cfg1", 3), ("cfg2", 3), ("cfg4", 2)):
        rec = shapes[key]
        init = O.basis_init([4, 4, 4, 2, 2, 2], rec["basis_reso"], in_dim)
        for g, shp, s in zip(init, rec["basis_shapes"], rec["basis_sums"]):
            assert list(g.shape) == shp[1:]
            assert abs(g.astype(np.float64).sum() - s) <= 1e-6 * max(1.0, abs(s))
    assert shapes["cfg0"]["coeff_shape"] == [1, 18, 271, 271]
    assert shapes["cfg1"]["basis_reso"] == [32, 51, 70, 89, 108, 128]
    assert shapes["cfg4"]["coeff_shape"] == [1, 18, 256, 32, 32]
    step, ns = O.step_size([[-1.5] * 3, [1.5] * 3], shapes["cfg2"]["grid_size"], 0.5)
    assert np.float32(step) == np.float32(shapes["cfg2"]["step_size"]) and ns == shapes["cfg2"]["n_samples"]


@pytest.mark.parametrize("case", FIELD_CASES)
def test_field_forward(case):
    d, meta = load(case)
    spec = O.FieldSpec.from_meta(meta)
    bg, cg = grids(d, meta["n_levels"])
    feats, coeff = O.get_coding(spec, bg, cg, d["x"])
    basis = O.get_basis(spec, bg, d["x"])
    assert rel_err(coeff, d["coeff"]) < 1e-6
    assert rel_err(basis, d["basis"]) < 1e-6
    assert rel_err(feats, d["feats"]) < 1e-6
    ws, bs = mlp_params(d)
    out, _ = O.mlp_fwd(ws, bs, d["feats"])
    assert rel_err(out, d["mlp_out"]) < 1e-5


@pytest.mark.parametrize("case", FIELD_CASES)
def test_field_backward(case):
    d, meta = load(case)
    spec = O.FieldSpec.from_meta(meta)
    bg, cg = grids(d, meta["n_levels"])
    gb, gc = O.get_coding_bwd(spec, bg, cg, d["x"], d["g_feats"], d["g_coeff"])
    for i, g in enumerate(gb):
        assert rel_err(g, d[f"grad_basis{i}"][0]) < 1e-5, i
    assert rel_err(gc, d["grad_coeffs0"][0]) < 1e-5
    ws, bs = mlp_params(d)
    gin, gw, gbias = O.mlp_bwd(ws, bs, d["feats"], d["g_out"])
    assert rel_err(gin, d["grad_mlp_in"]) < 1e-5
    for i in range(len(ws)):
        assert rel_err(gw[i], d[f"grad_mlp_w{i}"]) < 1e-5
        if bs[i] is not None:
            assert rel_err(gbias[i], d[f"grad_mlp_b{i}"]) < 1e-5


def head_params(d, meta):
    """MLPRender_Fea parameters of a golden render (None for the SH-2 head)."""
    if meta.get("head") != "mlp":
        return None
    ws, bs = mlp_params(d, "rm")
    r = meta["cfg"]["renderer"]
    return {"w": ws, "b": bs, "view_pe": r["view_pe"], "fea_pe": r["fea_pe"]}


@pytest.mark.parametrize("case", RENDER_CASES)
def test_render_forward_backward(case):
    d, meta = load(case)
    fspec = O.FieldSpec.from_meta(meta)
    bg, cg = grids(d, 6)
    r = meta["cfg"]["renderer"]
    rspec = O.RenderSpec(meta["aabb"], d["step_size"], int(d["n_samples"]), r["density_shift"],
                         r["distance_scale"], r["rayMarch_weight_thres"], meta["white_bg"])
    ws, bs = mlp_params(d)
    head = head_params(d, meta)
    res = O.render_rays(fspec, rspec, bg, cg, ws, bs, d["rays"], jitter=d["u"] if meta["jitter"] else None,
                        alpha_volume=d.get("alpha_volume"), g_rgb=d["g_rgb"], head=head)
    # sample positions, in-box mask and occupancy decisions are bit-exact
    np.testing.assert_array_equal(res["z"], d["z_vals"])
    np.testing.assert_array_equal(res["valid"], d["valid"])
    assert rel_err(res["rgb"], d["rgb"]) < 1e-5
    assert rel_err(res["depth"], d["depth"]) < 1e-5
    for i in range(6):
        assert rel_err(res["grad_basis"][i], d[f"grad_basis{i}"][0]) < 1e-4, i
    assert rel_err(res["grad_coeff"], d["grad_coeffs0"][0]) < 1e-4
    for i in range(len(ws)):
        assert rel_err(res["grad_mlp_w"][i], d[f"grad_mlp_w{i}"]) < 1e-4
    if head is not None:  # MLPRender_Fea's own parameters
        for i in range(len(head["w"])):
            assert rel_err(res["grad_head_w"][i], d[f"grad_rm_w{i}"]) < 1e-4, i
            if head["b"][i] is not None:
                assert rel_err(res["grad_head_b"][i], d[f"grad_rm_b{i}"]) < 1e-4, i


def test_positional_encoding_layout():
    """positional_encoding (models/FactorFields.py:74-79): sin block then cos block, index
    d * F + f, frequencies 2^f."""
    x = np.array([[0.3, -1.2]])
    pe = O.positional_encoding(x, 3)
    want_sin = [np.sin(0.3), np.sin(0.6), np.sin(1.2), np.sin(-1.2), np.sin(-2.4), np.sin(-4.8)]
    want_cos = [np.cos(0.3), np.cos(0.6), np.cos(1.2), np.cos(-1.2), np.cos(-2.4), np.cos(-4.8)]
    np.testing.assert_allclose(pe[0], want_sin + want_cos, rtol=1e-12)


def test_render_head_backward_finite_differences():
    """MLPRender_Fea's backward through the positional encoding against FP64 central
    differences (the oracle's analytic gradient is what the GPU kernels are checked against)."""
    rng = np.random.default_rng(0)
    c, hid = 5, 16
    w = [rng.standard_normal((hid, 3 + c + 36 + 4 * c)) * 0.3, rng.standard_normal((hid, hid)) * 0.3,
         rng.standard_normal((3, hid)) * 0.3]
    b = [rng.standard_normal(hid) * 0.1, rng.standard_normal(hid) * 0.1, None]
    feat = rng.standard_normal((7, c))
    dirs = rng.standard_normal((7, 3))
    g = rng.standard_normal((7, 3))
    g_feat, gw, _ = O.render_head_bwd(w, b, feat, dirs, 6, 2, g)
    eps = 1e-6
    num = np.zeros_like(feat)
    for i in range(feat.shape[0]):
        for k in range(c):
            fp, fm = feat.copy(), feat.copy()
            fp[i, k] += eps
            fm[i, k] -= eps
            num[i, k] = ((O.render_head_fwd(w, b, fp, dirs, 6, 2) - O.render_head_fwd(w, b, fm, dirs, 6, 2)) * g).sum() \
                / (2 * eps)
    np.testing.assert_allclose(g_feat, num, rtol=1e-6, atol=1e-8)
    wp = [x.copy() for x in w]
    wm = [x.copy() for x in w]
    wp[1][2, 3] += eps
    wm[1][2, 3] -= eps
    fd = ((O.render_head_fwd(wp, b, feat, dirs, 6, 2) - O.render_head_fwd(wm, b, feat, dirs, 6, 2)) * g).sum() / (2 * eps)
    assert abs(gw[1][2, 3] - fd) <= 1e-6 * max(abs(fd), 1e-3)


def test_raw2alpha_and_sh():
    d, _ = load("primitives.npz")
    a, w, t = O.raw2alpha(d["r2a_sigma"], d["r2a_dist"])
    assert rel_err(a, d["r2a_alpha"]) < 1e-6
    assert rel_err(w, d["r2a_weight"]) < 1e-5
    assert rel_err(t, d["r2a_bg"]) < 1e-5
    assert rel_err(O.eval_sh2(d["sh_coef"], d["sh_dirs"]), d["sh_out"]) < 1e-6


def _well_conditioned(w, u):
    """Mask of samples whose bin choice does not hinge on the last ulp of the float32 cdf.

    searchsorted(cdf, u) flips bins when u is within rounding distance of a cdf knot (e.g.
    u == 1.0 against a cdf total of 0.99999994 or 1.0000001); the reference itself gives
    different answers there on different CPUs because torch.sum's vector reduction order
    differs (x86 AVX vs Arm NEON)."""
    w64 = w.astype(np.float64) + 1e-5
    cdf = np.concatenate([np.zeros((w.shape[0], 1)), np.cumsum(w64 / w64.sum(1, keepdims=True), 1)], 1)
    dist = np.min(np.abs(u[:, :, None].astype(np.float64) - cdf[:, None, :]), -1)
    return dist > 1e-6


def test_sample_pdf():
    d, _ = load("primitives.npz")
    b, w = d["pdf_bins"], d["pdf_weights"]
    u_det = np.broadcast_to(np.linspace(0.0, 1.0, 48, dtype=np.float32), (b.shape[0], 48))
    for u, ref in ((u_det, d["pdf_det"]), (d["pdf_u_fixed"], d["pdf_fixed"])):
        got = O.sample_pdf(b, w, u)
        ok = _well_conditioned(w, u)
        assert ok.mean() > 0.95
        assert rel_err(got[ok], ref[ok]) < 1e-5


@pytest.mark.parametrize("case", FIELD_CASES)
def test_torch_cpu_baseline_matches_reference(case):
    """oracle/ref_torch.py (the timed CPU baseline) reproduces the reference's outputs/grads."""
    import torch
    from oracle.ref_torch import RefField
    d, meta = load(case)
    ws, bs = mlp_params(d)
    r = RefField(meta["cfg"]["defaults"]["mode"], meta["cfg"]["dataset"]["aabb"],
                 [d[f"basis{i}"] for i in range(meta["n_levels"])], d["coeffs0"], ws, bs, meta["freq_bands"],
                 meta["cfg"]["model"]["basis_mapping"], meta["cfg"]["model"]["basis_mode"],
                 meta["cfg"]["model"]["coef_mode"])
    x = torch.from_numpy(d["x"])
    feats, coeff = r.get_coding(x)
    np.testing.assert_array_equal(feats.detach().numpy(), d["feats"])
    loss = (feats * torch.from_numpy(d["g_feats"])).sum() + (coeff * torch.from_numpy(d["g_coeff"])).sum()
    loss.backward()
    for i in range(meta["n_levels"]):
        assert rel_err(r.basises[i].grad.numpy(), d[f"grad_basis{i}"]) < 1e-6
    assert rel_err(r.coeff.grad.numpy(), d["grad_coeffs0"]) < 1e-6


@pytest.mark.parametrize("case", [c for c in RENDER_CASES if "sh" in c])
def test_torch_cpu_render_matches_reference(case):
    """oracle/ref_torch.py's render (the radiance configurations' timed CPU baseline) reproduces the
    reference's own render of the golden SH-head fixtures: rgb, depth and the gradients of
    sum(rgb * g_rgb)."""
    import torch
    from oracle.ref_torch import RefField, RefRender
    d, meta = load(case)
    ws, bs = mlp_params(d)
    cfg = meta["cfg"]
    f = RefField(cfg["defaults"]["mode"], cfg["dataset"]["aabb"], [d[f"basis{i}"] for i in range(6)], d["coeffs0"],
                 ws, bs, meta["freq_bands"], cfg["model"]["basis_mapping"], cfg["model"]["basis_mode"],
                 cfg["model"]["coef_mode"])
    r = cfg["renderer"]
    rr = RefRender(f, float(d["step_size"]), int(d["n_samples"]), d.get("alpha_volume"), r["density_shift"],
                   r["distance_scale"], r["rayMarch_weight_thres"], r["fea2denseAct"])
    jitter = torch.from_numpy(d["u"]) if meta["jitter"] else None
    rgb, depth = rr.forward(torch.from_numpy(d["rays"]), white_bg=meta["white_bg"], jitter=jitter)
    assert rel_err(rgb.detach().numpy(), d["rgb"]) < 1e-6
    assert rel_err(depth.numpy(), d["depth"]) < 1e-6
    (rgb * torch.from_numpy(d["g_rgb"])).sum().backward()
    for i in range(6):
        assert rel_err(f.basises[i].grad.numpy(), d[f"grad_basis{i}"]) < 1e-5, i
    assert rel_err(f.coeff.grad.numpy(), d["grad_coeffs0"]) < 1e-5
    for i in range(len(ws)):
        assert rel_err(f.weights[i].grad.numpy(), d[f"grad_mlp_w{i}"]) < 1e-5
