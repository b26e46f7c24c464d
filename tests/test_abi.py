"""The C-ABI library loads and exports every symbol include/*.h declares (CPU only: no
compute call is made; the ctypes struct layouts are checked against the library's sizeof)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names.update(re.findall(r"FF_API\s+[\w\s\*]+?\b(ff_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from factor_fields_gb300 import build
    from factor_fields_gb300 import _native as N
    build.build()
    return N.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "ff_field_forward" in names and "ff_field_backward" in names and len(names) >= 8


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(lib):
    from factor_fields_gb300 import _native as N
    assert set(declared_symbols()) == set(N.SIGNATURES), set(declared_symbols()) ^ set(N.SIGNATURES)


def test_struct_layouts_match(lib):
    from factor_fields_gb300 import _native as N
    assert lib.ff_abi_version() == 1
    for i, st in enumerate([N.FFField, N.FFMlp, N.FFMlpGrad, N.FFRender, N.FFProposal, N.FFAdamParam,
                            N.FFRenderMlp]):
        assert lib.ff_struct_size(i) == ctypes.sizeof(st), st.__name__


def test_argument_validation_before_any_launch(lib):
    """Bad arguments are rejected with the documented codes and a message, before any CUDA
    call (so this runs without a GPU)."""
    from factor_fields_gb300 import _native as N
    vp = ctypes.c_void_p
    # ff_adam_step: negative count, unknown flag, betas out of range, step < 1
    assert lib.ff_adam_step(None, -1, 0.9, 0.99, 1e-8, 0, None) == N.FF_ERR_ARG
    p = N.FFAdamParam()
    p.param = p.grad = p.exp_avg = p.exp_avg_sq = 16
    p.n, p.step, p.lr = 4, 1, 1e-3
    arr = (N.FFAdamParam * 1)(p)
    assert lib.ff_adam_step(ctypes.cast(arr, vp), 1, 0.9, 0.99, 1e-8, 4, None) == N.FF_ERR_ARG
    assert lib.ff_adam_step(ctypes.cast(arr, vp), 1, 1.0, 0.99, 1e-8, 0, None) == N.FF_ERR_ARG
    arr[0].step = 0
    assert lib.ff_adam_step(ctypes.cast(arr, vp), 1, 0.9, 0.99, 1e-8, 0, None) == N.FF_ERR_ARG
    assert b"step" in lib.ff_last_error()
    # the scheduled form reads lr and step from device memory: both pointers are required
    assert lib.ff_adam_step_scheduled(ctypes.cast(arr, vp), 1, 0.9, 0.99, 1e-8, 0, None, vp(16), None) == N.FF_ERR_ARG
    assert lib.ff_adam_step_scheduled(ctypes.cast(arr, vp), 1, 0.9, 0.99, 1e-8, 0, vp(16), vp(12), None) == N.FF_ERR_ALIGN
    # ff_zero_f32: NULL buffer with a count
    ptrs = (vp * 1)(None)
    counts = (ctypes.c_int64 * 1)(5)
    assert lib.ff_zero_f32(ptrs, counts, 1, None) == N.FF_ERR_ARG
    # ff_occupancy_mask / ff_image_metrics: bad dimensions, missing workspace
    assert lib.ff_occupancy_workspace_bytes(0, 4, 4) < 0
    assert lib.ff_occupancy_mask(vp(16), 4, 4, 4, 0.5, 1, vp(16), None, vp(16), None, 0, None) == N.FF_ERR_ARG
    ws = lib.ff_occupancy_workspace_bytes(4, 4, 4)
    assert lib.ff_occupancy_mask(vp(16), 4, 4, 4, 0.5, 1, vp(16), None, vp(16), vp(256), ws - 1, None) == N.FF_ERR_SIZE
    assert lib.ff_image_metrics_workspace_bytes(10, 20, 3) < 0  # SSIM's window needs >= 11 pixels
    out = (ctypes.c_double * 2)()
    assert lib.ff_image_metrics(vp(16), vp(16), 11, 11, 3, 1.0, out, None, 0, None) == N.FF_ERR_ARG
    # ff_field_fit_step_binned: unknown flags / too small a workspace are reported
    assert lib.ff_field_fit_binned_workspace_bytes(None, 10, 1) < 0
    # ff_filter_rays: needs an occupancy bitfield unless bbox_only
    r = N.FFRender()
    r.step, r.n_samples, r.distance_scale = 0.01, 16, 25.0
    for k in range(3):
        r.aabb_min[k], r.aabb_max[k] = -1.0, 1.0
    assert lib.ff_filter_rays(ctypes.byref(r), vp(16), 4, 16, 0, vp(16), None) == N.FF_ERR_ARG


def test_binned_fit_halves_validate_their_flags(lib):
    """ff_field_fit_bin takes FF_FIT_ZERO_GRADS and FF_FIT_HOST_BATCH, ff_field_fit_step_on_bins
    FF_FIT_MEAN_LOSS and FF_FIT_LEVEL0_SHARED; both reject a missing or short workspace (all
    before any launch)."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import functional as FN
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300 import _native as N
    m = FactorFields(W.field_cfg("cfg1"), device="cpu", precision="bf16")
    desc = m.descriptor(N.FF_BF16)
    ws_, bs_ = m.linear_mat.weights()
    mlp = FN.mlp_struct(ws_, bs_, m.linear_mat.in_dim, m.linear_mat.hidden_dim, m.linear_mat.out_dim)
    g = N.FFMlpGrad()
    vp = ctypes.c_void_p
    n = 1024
    need = lib.ff_field_fit_binned_workspace_bytes(ctypes.byref(desc), n, 1)
    assert need > 0
    ws = vp(256)
    args_bin = (ctypes.byref(desc), ctypes.byref(mlp), vp(16), vp(16), n, vp(16), vp(16), vp(16), ctypes.byref(g))
    assert lib.ff_field_fit_bin(*args_bin, N.FF_FIT_MEAN_LOSS, ws, need, None) == N.FF_ERR_ARG
    assert lib.ff_field_fit_bin(*args_bin, N.FF_FIT_ZERO_GRADS, None, need, None) == N.FF_ERR_ARG
    assert lib.ff_field_fit_bin(*args_bin, N.FF_FIT_ZERO_GRADS, ws, need - 1, None) == N.FF_ERR_SIZE
    args_fit = (ctypes.byref(desc), vp(16), vp(16), ctypes.byref(mlp), n, N.FF_LOSS["l1"], 1.0 / n, vp(16), vp(16),
                vp(16), ctypes.byref(g))
    assert lib.ff_field_fit_step_on_bins(*args_fit, N.FF_FIT_ZERO_GRADS, ws, need, None) == N.FF_ERR_ARG
    assert lib.ff_field_fit_step_on_bins(*args_fit, N.FF_FIT_MEAN_LOSS, ws, need - 1, None) == N.FF_ERR_SIZE
    assert lib.ff_field_fit_step_on_bins(*args_fit, N.FF_FIT_MEAN_LOSS, vp(128), need, None) == N.FF_ERR_ALIGN
    assert lib.ff_field_fit_step_binned(ctypes.byref(desc), vp(16), vp(16), ctypes.byref(mlp), vp(16), vp(16), n,
                                        N.FF_LOSS["l1"], 1.0 / n, vp(16), vp(16), vp(16), ctypes.byref(g), 16, ws, need,
                                        None) == N.FF_ERR_ARG
    # the host batch is the binning half's input: the fit half has none
    assert lib.ff_field_fit_step_on_bins(*args_fit, N.FF_FIT_HOST_BATCH, ws, need, None) == N.FF_ERR_ARG


def test_render_head_validation(lib):
    """The MLPRender_Fea entry points check the descriptor before any launch: in_dim must follow
    the reference's formula, the last layer has no bias, and the tensor-core head rejects shapes
    it does not implement."""
    from factor_fields_gb300 import _native as N
    h = N.FFRenderMlp()
    h.n_layers, h.in_channels, h.hidden_dim, h.view_pe, h.fea_pe = 3, 31, 128, 6, 2
    h.in_dim = 3 + 31 + 36 + 124
    for i in range(3):
        h.weight[i] = 256
    h.bias[0] = h.bias[1] = 256
    args = (ctypes.c_void_p(256), 32, ctypes.c_void_p(256), ctypes.c_void_p(256), ctypes.c_void_p(256), 0)
    assert lib.ff_render_head_forward_tc(ctypes.byref(h), *args, None, None, None) == N.FF_OK  # n = 0: no launch
    h.in_dim += 1
    assert lib.ff_render_head_forward_tc(ctypes.byref(h), *args, None, None, None) == N.FF_ERR_ARG
    h.in_dim -= 1
    h.bias[2] = 256
    assert lib.ff_render_head_forward_tc(ctypes.byref(h), *args, None, None, None) == N.FF_ERR_ARG
    h.bias[2] = None
    h.hidden_dim = 64
    assert lib.ff_render_head_forward_tc(ctypes.byref(h), *args, None, None, None) == N.FF_ERR_UNSUPPORTED
    assert b"hidden_dim" in lib.ff_last_error()
    assert lib.ff_render_head_workspace_bytes(ctypes.byref(h), 100) > 0


def test_rendering_forms_validate_before_any_launch(lib):
    """The proposal's rendering entry points reject what they do not implement before any CUDA
    call: ff_field_render_fixed takes 32, 64 or 128 samples per ray and the 28-wide SH head,
    ff_proposal_head_infer a BF16 grid, ff_proposal_resample_occupied an occupancy volume and a
    large enough scan workspace."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import functional as FN
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300.renderer import render_desc
    vp = ctypes.c_void_p
    m = FactorFields(W.field_cfg("cfg2"), device="cpu", precision="bf16")
    desc = m.descriptor(N.FF_BF16)
    ws_, bs_ = m.linear_mat.weights()
    mlp = FN.mlp_struct(ws_, bs_, m.linear_mat.in_dim, m.linear_mat.hidden_dim, m.linear_mat.out_dim)
    rd = render_desc(m, 32, True)
    args = (ctypes.byref(desc), vp(256), vp(256), ctypes.byref(mlp), ctypes.byref(rd), vp(256), vp(256), vp(256))
    assert lib.ff_field_render_fixed(*args, 100, 48, vp(256), None, None) == N.FF_ERR_UNSUPPORTED
    assert lib.ff_field_render_fixed(*args, 100, 32, None, None, None) == N.FF_ERR_ARG  # rgb NULL
    assert lib.ff_field_render_fixed(*args, -1, 32, vp(256), None, None) == N.FF_ERR_ARG
    mlp.out_dim = 3
    assert lib.ff_field_render_fixed(*args, 100, 32, vp(256), None, None) == N.FF_ERR_UNSUPPORTED
    assert b"28-wide" in lib.ff_last_error()
    # the proposal head's rendering form reads a BF16 grid
    p = N.FFProposal()
    for k in range(3):
        p.aabb_min[k], p.aabb_max[k], p.inv_cell[k] = -1.5, 1.5, 21.0
    p.reso, p.n_bins, p.n_fine, p.param_dtype = 64, 64, 32, N.FF_F32
    head = N.FFMlp()
    head.n_layers, head.in_dim, head.hidden_dim, head.out_dim = 2, 8, 64, 1
    head.weight[0], head.weight[1], head.bias[0] = 256, 256, 256
    assert lib.ff_proposal_head_infer(ctypes.byref(p), vp(256), ctypes.byref(head), vp(256), 10, vp(256),
                                      None) == N.FF_ERR_UNSUPPORTED
    # occupancy-culled resampling needs occ_bits and the scan workspace
    p.param_dtype = N.FF_BF16
    need = lib.ff_scan_workspace_bytes(10)
    rd.occ_bits = None
    assert lib.ff_proposal_resample_occupied(ctypes.byref(p), ctypes.byref(rd), vp(256), 10, vp(256), None, vp(256),
                                             vp(256), vp(256), need, vp(256), vp(256), None) == N.FF_ERR_ARG
    rd.occ_bits = 256
    for k in range(3):
        rd.occ_reso[k] = 8
    assert lib.ff_proposal_resample_occupied(ctypes.byref(p), ctypes.byref(rd), vp(256), 10, vp(256), None, vp(256),
                                             vp(256), vp(256), need - 1, vp(256), vp(256), None) == N.FF_ERR_ARG
