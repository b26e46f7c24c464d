"""Host-side logic on the CPU: config derivation (setup_params), DCT init, channels-last layout
and converters, the native descriptor, checkpoints in the reference's format."""
import json
import os

import numpy as np
import torch

from factor_fields_gb300 import FactorFields, make_cfg
from factor_fields_gb300.config import FieldGeometry, render_step
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
    # the reference also counts its MLPRender_Fea colour head (39 -> 128 -> 128 -> 3 for
    # out_dim = 1: 22,016 parameters); this library's default head is the parameter-free SH-2 head
    fea_head = 39 * 128 + 128 + 128 * 128 + 128 + 128 * 3
    assert m.n_parameters() == ref["cfg1"]["n_params"] - fea_head


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
