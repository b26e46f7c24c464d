"""Host-side logic on the CPU: config derivation (setup_params), DCT init, channels-last layout
and converters, the native descriptor, checkpoints in the reference's format."""
import json
import os

import numpy as np
import torch

from factor_fields_gb300 import FactorFields, make_cfg
from factor_fields_gb300.config import FieldGeometry, n_to_reso, render_step
from factor_fields_gb300.layout import FieldLayout
from factor_fields_gb300 import workloads as W

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def shapes():
    with open(os.path.join(GOLD, "config_shapes.json")) as f:
        return json.load(f)


def test_geometry_matches_reference_configs():
    ref = shapes()
    for key in ("cfg0", "cfg1", "cfg2", "cfg4"):
        cfg = W.field_cfg(key)
        g = FieldGeometry(cfg)
        if key == "cfg0":
            g.freq_bands = torch.tensor(W.FREQ6)
        assert g.basis_reso == ref[key]["basis_reso"], key
        assert [1, g.n_feat] + g.coeff_reso == ref[key]["coeff_shape"], key
        np.testing.assert_array_equal(g.freq_bands.numpy(), np.float32(ref[key]["freq_bands"]))


def test_dct_init_and_views():
    ref = shapes()
    m = FactorFields(W.field_cfg("cfg1"), device="cpu")
    for b, s, shp in zip(m.basises, ref["cfg1"]["basis_sums"], ref["cfg1"]["basis_shapes"]):
        assert list(b.shape) == shp
        assert abs(b.double().sum().item() - s) <= 1e-6 * max(1, abs(s))
    assert list(m.coeffs[0].shape) == ref["cfg1"]["coeff_shape"]
    # the count includes the MLPRender_Fea colour head (39 -> 128 -> 128 -> 3 for out_dim = 1),
    # which the reference builds for every reconstruction model
    assert m.n_parameters() == ref["cfg1"]["n_params"]


def test_step_size_matches_reference():
    ref = shapes()["cfg2"]
    step, n = render_step(torch.tensor([[-1.5] * 3, [1.5] * 3]), ref["grid_size"], 0.5)
    assert np.float32(step.item()) == np.float32(ref["step_size"]) and n == ref["n_samples"]


def test_layout_round_trip_and_padding():
    lay = FieldLayout([4, 4, 5, 2, 1, 2], [3, 4, 5, 6, 7, 8], 3, [4, 5, 6])
    rng = np.random.default_rng(0)
    levels = [torch.from_numpy(rng.standard_normal([1, c] + [r] * 3).astype(np.float32))
              for c, r in zip(lay.basis_dims, lay.basis_reso)]
    flat = lay.basis_from_reference(levels)
    for l, g in enumerate(levels):
        assert torch.equal(lay.basis_view(flat, l), g)
    # padded channels stay zero, offsets are 8-aligned, vector widths divide everything
    assert all(o % 8 == 0 for o in lay.level_offset)
    assert lay.level_vec[2] == 1 and lay.level_stride[2] == 8
    mask = torch.ones_like(flat, dtype=torch.bool)
    for l in range(len(levels)):
        mask[lay.level_offset[l]:lay.level_offset[l] + lay.basis_reso[l] ** 3 * lay.level_stride[l]] = False
        v = lay.basis_view(flat, l)
        assert v.numel() == levels[l].numel()
    coef = torch.from_numpy(rng.standard_normal([1, 18, 4, 5, 6]).astype(np.float32))
    cf = lay.coeff_from_reference([coef])
    assert torch.equal(lay.coeff_view(cf, 0), coef)
    assert lay.coeff_stride == 24


def test_descriptor_fields():
    m = FactorFields(W.field_cfg("cfg2"), device="cpu")
    d = m.descriptor(0)
    assert d.basis_dim == 3 and d.coord_dim == 3 and d.n_levels == 6 and d.mapping == 1
    scale = (torch.tensor(3.0) / m.freq_bands).numpy()
    for l in range(6):
        assert np.float32(d.level_scale[l]) == scale[l]
        assert d.level_vec[l] == (4 if l < 3 else 2)
    assert list(d.coeff_reso) == [64, 64, 64] and d.coeff_stride == 24
    assert np.float32(d.coeff_inv_size[0]) == np.float32(2.0) / np.float32(3.0)


def test_reference_state_dict_round_trip(tmp_path):
    cfg = W.field_cfg("cfg4", small=True)
    m = FactorFields(cfg, device="cpu")
    with torch.no_grad():
        m.basis_flat.normal_()
        m.coeff_flat.normal_()
    sd = m.reference_state_dict()
    assert sd["coeffs.0"].shape == (1, 18, 16, 8, 8)
    m2 = FactorFields(cfg, device="cpu")
    m2.load_reference_state_dict(sd)
    for a, b in zip(m.basises, m2.basises):
        assert torch.equal(a, b)
    assert torch.equal(m.coeffs[0], m2.coeffs[0])
    p = tmp_path / "ck.th"
    m.save(str(p))
    m3 = FactorFields(cfg, device="cpu")
    m3.load(torch.load(str(p), weights_only=False))
    assert torch.equal(m3.coeffs[0], m.coeffs[0])


def test_occupancy_oracle_known_answer():
    """The oracle's remove_small_objects restatement: 6-connectivity (diagonal neighbours are
    separate components), components below min_size removed, max-pool before the threshold."""
    from oracle import ff_oracle as O
    a = np.zeros((12, 12, 12), np.float32)
    a[2, 2, 2] = 1.0                  # pooled: a 3x3x3 cube = 27 voxels
    a[8, 8, 8] = 0.9                  # another 27-voxel cube
    a[8, 8, 11] = 0.7                 # pooled cube clipped at the x border: 3x3x2 = 18, touching the
    occ, _, box = O.occupancy_mask(a, 0.5, 28)  # previous one (x 9 / x 10): one 45-voxel component
    assert occ.sum() == 45 and not occ[2, 2, 2]
    assert box == (7, 7, 7, 11, 9, 9)
    occ, words, _ = O.occupancy_mask(a, 0.5, 1)
    assert occ.sum() == 27 + 45
    c = np.zeros((10, 10, 10), np.float32)
    c[2, 2, 2] = c[2, 5, 5] = 1.0     # pooled cubes touching only along an edge (diagonal in y-x)
    occ, _, _ = O.occupancy_mask(c, 0.5, 28)
    assert occ.sum() == 0             # two 27-voxel components under 6-connectivity, both < 28
    occ, _, _ = O.occupancy_mask(c, 0.5, 27)
    assert occ.sum() == 54


def _small_rec_cfg(mode="reconstruction", n_scene=1, **dataset):
    """A small 3-D reconstruction config (levels of 5..10 cells, 6^3 coefficients)."""
    from factor_fields_gb300.config import merged_cfg
    aabb = [[-1.5] * 3, [1.5] * 3]
    if mode == "reconstructions":
        aabb = [[-1.5] * 3 + [0], [1.5] * 3 + [n_scene]]
    return merged_cfg({"defaults": {"mode": mode},
                       "model": {"basis_resos": [5, 6, 7, 8, 9, 10], "coeff_reso": 6, "total_params": 11106,
                                 "out_dim": 28, "basis_mapping": "triangle"},
                       "dataset": {"aabb": aabb, "scene_reso": 1024, **dataset}})


def _tv(x):
    """TV regulariser of utils.py:160-175 (restated for the check)."""
    h, w = x.size()[2], x.size()[3]
    count_h = x[:, :, 1:, :].numel() // x.size()[0]
    count_w = x[:, :, :, 1:].numel() // x.size()[0]
    h_tv = torch.pow(x[:, :, 1:, :] - x[:, :, :h - 1, :], 2).sum()
    w_tv = torch.pow(x[:, :, :, 1:] - x[:, :, :, :w - 1], 2).sum()
    return 2 * (h_tv / count_h + w_tv / count_w) / x.size()[0]


def test_surface_methods_follow_reference():
    """normalize_basis (:519-521), TV_loss (:569-573), set_optimizable (:556-567) and
    upsample_volume_grid (:701-707) on the reference-layout views of the flat parameters."""
    torch.manual_seed(0)
    m = FactorFields(_small_rec_cfg(), device="cpu")
    with torch.no_grad():
        m.basis_flat.normal_()
    ref_levels = [b.detach().clone() for b in m.basises]
    m.normalize_basis()
    for got, ref in zip(m.basises, ref_levels):
        want = ref / torch.norm(ref, dim=(2, 3), keepdim=True)
        assert torch.allclose(got, want, rtol=1e-6, atol=1e-7)
    # TV_loss: the reference's sum over levels, gradient reaching the flat basis
    total = m.TV_loss(_tv)
    want = sum(_tv(b.detach().contiguous()) * 1e-2 for b in m.basises)
    assert torch.allclose(total.detach(), want, rtol=1e-5)
    total.backward()
    assert m.basis_flat.grad is not None and float(m.basis_flat.grad.abs().sum()) > 0
    # set_optimizable: 'basis' and 'coeff' both toggle the basis grids, as in the reference
    m.set_optimizable(["coeff"], False)
    assert not m.basis_flat.requires_grad and m.coeff_flat.requires_grad
    m.set_optimizable(["basis", "proj", "renderer"], True)
    assert m.basis_flat.requires_grad and m.linear_mat.requires_grad is True and m.renderModule.requires_grad is True
    # upsample_volume_grid: render parameters for the new resolution; coefficients unchanged
    coeff0 = m.coeffs[0].detach().clone()
    m.upsample_volume_grid([64, 64, 64])
    assert m.gridSize.tolist() == [64, 64, 64]
    assert torch.equal(m.coeffs[0], coeff0)
    step, n = render_step(torch.tensor(m.cfg.dataset.aabb), [64, 64, 64], 0.5)
    assert float(m.stepSize) == float(step) and m.nSamples == n
    # google_objs with one scene: the coefficient grid resampled by 1.3 (trilinear, align_corners)
    g = FactorFields(_small_rec_cfg(dataset_name="google_objs"), device="cpu")
    with torch.no_grad():
        g.coeff_flat.normal_()
    old = g.coeffs[0].detach().contiguous()
    g.upsample_volume_grid([32, 32, 32])
    want = torch.nn.functional.interpolate(old, scale_factor=1.3, align_corners=True, mode="trilinear")
    assert g.coeffs[0].shape == want.shape == (1, 18, 7, 7, 7)
    assert torch.equal(g.coeffs[0], want)
    assert g.descriptor(0).coeff_reso[0] == 7


def test_save_averages_scene_coefficients(tmp_path):
    """save() in the reconstruction modes writes the scenes' mean coefficients as coeffs.0
    (cal_mean_coef, :645-667, :677-679); load() recomputes the render parameters (:689-691)."""
    cfg = _small_rec_cfg("reconstructions", n_scene=3)
    m = FactorFields(cfg, device="cpu")
    assert m.n_scene == 3
    with torch.no_grad():
        m.coeff_flat.normal_()
    mean = sum(c.detach() for c in m.coeffs) / 3
    p = tmp_path / "multi.th"
    m.save(str(p))
    ck = torch.load(str(p), weights_only=False)
    keys = [k for k in ck["state_dict"] if k.startswith("coeffs.")]
    assert keys == ["coeffs.0"]
    assert torch.allclose(ck["state_dict"]["coeffs.0"], mean, rtol=1e-6, atol=1e-7)
    m2 = FactorFields(cfg, device="cpu")
    m2.load(ck)
    for c in m2.coeffs:
        assert torch.allclose(c, mean, rtol=1e-6, atol=1e-7)
    assert m2.gridSize.tolist() == n_to_reso(300 ** 3, m2.aabb.cpu())


def test_proposal_sampler_refuses_mlp_fea_shading():
    """The proposal sampler composites with the degree-2 SH head; a model shaded by MLPRender_Fea
    is refused instead of being rendered with the wrong colour head."""
    import pytest
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    cfg = W.field_cfg("cfg2")
    cfg.renderer.shadingMode = "MLP_Fea"
    m = FactorFields(cfg, device="cpu")
    with pytest.raises(NotImplementedError, match="SH"):
        ProposalSampler(m)


def test_fit_runner_host_batch_rules():
    """A fit step takes a host batch only on the binned path and only from page-locked memory
    (FF_FIT_HOST_BATCH copies it asynchronously); anything else is refused before a call."""
    import pytest
    import torch
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.train import FieldFitRunner
    m = FactorFields(W.field_cfg("cfg1"), device="cpu", precision="bf16")
    x, y = torch.zeros(16, 3), torch.zeros(16, 1)
    with pytest.raises(ValueError, match="page-locked"):
        FieldFitRunner(m, loss="l1")._host_batch(x, y)
    with pytest.raises(ValueError, match="binned"):
        FieldFitRunner(m, loss="l1", fused=True, binned=False)._host_batch(x, y)
    with pytest.raises(ValueError, match="binned"):
        FieldFitRunner(m, loss="l1", fused=False)._host_batch(x, y)


def test_fused_adam_device_schedule_host_logic():
    """FusedAdam's device schedule bookkeeping without a GPU: enable_device_schedule takes every
    parameter with a gradient (creating its Adam state), refuses mixed step counts, decays the
    learning rates as float64 products exactly like the host schedule, and sync_host /
    state_dict write them back; load_state_dict drops the schedule."""
    import pytest
    import torch
    from factor_fields_gb300.optim import FusedAdam
    ps = [torch.nn.Parameter(torch.zeros(5)), torch.nn.Parameter(torch.zeros(3)), torch.nn.Parameter(torch.zeros(2))]
    for p in ps[:2]:
        p.grad = torch.zeros_like(p)  # ps[2] has no gradient: not scheduled
    opt = FusedAdam([{"params": ps[:1], "lr": 2e-2}, {"params": ps[1:], "lr": 1e-3}], betas=(0.9, 0.99))
    opt.enable_device_schedule()
    assert opt.device_schedule and len(opt.state) == 2
    lrs = [2e-2, 1e-3]
    for _ in range(7):
        opt.decay_lr(0.93)
        lrs = [v * 0.93 for v in lrs]
    opt._dev["t"] += 7  # what seven replayed updates would have counted
    sd = opt.state_dict()  # synchronises first
    assert [g["lr"] for g in sd["param_groups"]] == lrs
    assert all(int(s["step"]) == 7 for s in sd["state"].values())
    opt.load_state_dict(sd)
    assert not opt.device_schedule
    # mixed step counts cannot share one device counter
    opt.state[ps[0]]["step"] = torch.tensor(3.0)
    with pytest.raises(ValueError, match="same step"):
        opt.enable_device_schedule()


def test_fit_runner_optimize_needs_an_optimizer():
    import pytest
    import torch
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.train import FieldFitRunner
    m = FactorFields(W.field_cfg("cfg1"), device="cpu", precision="bf16")
    r = FieldFitRunner(m, loss="l1")
    with pytest.raises(ValueError, match="optimizer"):
        r.step(torch.zeros(4, 3), torch.zeros(4, 1), optimize=True)
