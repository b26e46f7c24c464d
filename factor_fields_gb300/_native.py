"""ctypes binding of libffgb.so (the C ABI declared in include/ff_native.h).

The library is built in-tree by factor_fields_gb300.build and loaded from this package's
directory. There is no fallback: if the library is missing or cannot be loaded, every
operation raises. Device pointers come from torch tensors; work is enqueued on torch's
current CUDA stream.
"""
import ctypes
import os
import threading

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libffgb.so")

FF_MAX_LEVELS = 8
FF_MAX_MLP_LAYERS = 4
FF_OK, FF_ERR_ARG, FF_ERR_UNSUPPORTED, FF_ERR_ALIGN, FF_ERR_CUDA, FF_ERR_SIZE, FF_ERR_LIMIT = 0, -1, -2, -3, -4, -5, -6
FF_MAP = {"sawtooth": 0, "triangle": 1}
FF_INTERP = {"bilinear": 0, "linear": 0, "trilinear": 0, "nearest": 1}
FF_F32, FF_BF16 = 0, 1
FF_LOSS = {"l1": 0, "mse": 1}
FF_FIT_ZERO_GRADS = 1
FF_FIT_MEAN_LOSS = 2
FF_FIT_LEVEL0_SHARED = 4
FF_FIT_HOST_BATCH = 8
FF_ADAM_ZERO_GRAD = 1

c_i32, c_i64, c_f32, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p


class FFField(ctypes.Structure):
    _fields_ = [
        ("basis_dim", c_i32), ("coord_dim", c_i32), ("n_levels", c_i32), ("mapping", c_i32),
        ("basis_interp", c_i32), ("coeff_interp", c_i32), ("param_dtype", c_i32), ("n_feat", c_i32),
        ("level_channels", c_i32 * FF_MAX_LEVELS), ("level_stride", c_i32 * FF_MAX_LEVELS),
        ("level_vec", c_i32 * FF_MAX_LEVELS), ("level_reso", c_i32 * FF_MAX_LEVELS),
        ("level_offset", c_i64 * FF_MAX_LEVELS), ("level_scale", c_f32 * FF_MAX_LEVELS),
        ("map_origin", c_f32 * 3), ("coeff_reso", c_i32 * 3), ("coeff_stride", c_i32),
        ("coeff_origin", c_f32 * 3), ("coeff_inv_size", c_f32 * 3),
        ("level_inv_scale", c_f32 * FF_MAX_LEVELS), ("level_inv_half", c_f32 * FF_MAX_LEVELS),
    ]


class FFMlp(ctypes.Structure):
    _fields_ = [("n_layers", c_i32), ("in_dim", c_i32), ("hidden_dim", c_i32), ("out_dim", c_i32),
                ("weight", c_vp * FF_MAX_MLP_LAYERS), ("bias", c_vp * FF_MAX_MLP_LAYERS)]


class FFMlpGrad(ctypes.Structure):
    _fields_ = [("weight", c_vp * FF_MAX_MLP_LAYERS), ("bias", c_vp * FF_MAX_MLP_LAYERS)]


class FFRender(ctypes.Structure):
    _fields_ = [("aabb_min", c_f32 * 3), ("aabb_max", c_f32 * 3), ("step", c_f32), ("n_samples", c_i32),
                ("distance_scale", c_f32), ("density_shift", c_f32), ("density_act", c_i32),
                ("weight_thres", c_f32), ("white_bg", c_i32), ("occ_bits", c_vp), ("occ_reso", c_i32 * 3),
                ("occ_origin", c_f32 * 3), ("occ_inv", c_f32 * 3)]


class FFRenderMlp(ctypes.Structure):
    _fields_ = [("n_layers", c_i32), ("in_channels", c_i32), ("hidden_dim", c_i32), ("view_pe", c_i32),
                ("fea_pe", c_i32), ("in_dim", c_i32), ("weight", c_vp * FF_MAX_MLP_LAYERS),
                ("bias", c_vp * FF_MAX_MLP_LAYERS)]


class FFAdamParam(ctypes.Structure):
    _fields_ = [("param", c_vp), ("grad", c_vp), ("exp_avg", c_vp), ("exp_avg_sq", c_vp), ("param_bf16", c_vp),
                ("n", c_i64), ("step", c_i64), ("lr", c_f32), ("reserved", c_f32)]


class FFProposal(ctypes.Structure):
    _fields_ = [("aabb_min", c_f32 * 3), ("aabb_max", c_f32 * 3), ("inv_cell", c_f32 * 3), ("reso", c_i32),
                ("param_dtype", c_i32), ("n_bins", c_i32), ("n_fine", c_i32), ("density_shift", c_f32),
                ("distance_scale", c_f32), ("uniform_mix", c_f32), ("u_stratified", c_i32)]


# (name, restype, argtypes) of every exported entry point.
_P = ctypes.POINTER
SIGNATURES = {
    "ff_abi_version": (c_i32, []),
    "ff_last_error": (ctypes.c_char_p, []),
    "ff_struct_size": (c_i64, [c_i32]),
    "ff_device_info": (c_i32, [_P(c_i32), _P(c_i32)]),
    "ff_field_forward": (c_i32, [_P(FFField), c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "ff_field_backward": (c_i32, [_P(FFField), c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ff_mlp_forward": (c_i32, [_P(FFMlp), c_vp, c_i64, c_vp, c_vp]),
    "ff_mlp_backward": (c_i32, [_P(FFMlp), c_vp, c_i64, c_vp, c_vp, _P(FFMlpGrad), c_vp]),
    "ff_field_mlp_forward": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp]),
    "ff_field_mlp_backward": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp, c_vp,
                                      _P(FFMlpGrad), c_vp]),
    "ff_field_mlp_forward_counted": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp, c_vp]),
    "ff_field_mlp_backward_counted": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp, c_vp,
                                              c_vp, _P(FFMlpGrad), c_vp]),
    "ff_field_fit_step": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_vp, c_vp, c_i64, c_i32, c_f32, c_vp, c_vp,
                                  c_vp, _P(FFMlpGrad), c_vp]),
    "ff_field_fit_binned_workspace_bytes": (c_i64, [_P(FFField), c_i64, c_i32]),
    "ff_field_fit_step_binned": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_vp, c_vp, c_i64, c_i32, c_f32, c_vp,
                                         c_vp, c_vp, _P(FFMlpGrad), c_i32, c_vp, c_i64, c_vp]),
    "ff_field_fit_bin": (c_i32, [_P(FFField), _P(FFMlp), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, _P(FFMlpGrad), c_i32,
                                 c_vp, c_i64, c_vp]),
    "ff_field_fit_step_on_bins": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), c_i64, c_i32, c_f32, c_vp, c_vp, c_vp,
                                          _P(FFMlpGrad), c_i32, c_vp, c_i64, c_vp]),
    "ff_zero_f32": (c_i32, [c_vp, c_vp, c_i32, c_vp]),
    "ff_adam_step": (c_i32, [c_vp, c_i32, c_f32, c_f32, c_f32, c_i32, c_vp]),
    "ff_adam_step_scheduled": (c_i32, [c_vp, c_i32, c_f32, c_f32, c_f32, c_i32, c_vp, c_vp, c_vp]),
    "ff_image_metrics_workspace_bytes": (c_i64, [c_i32, c_i32, c_i32]),
    "ff_image_metrics": (c_i32, [c_vp, c_vp, c_i32, c_i32, c_i32, c_f32, c_vp, c_vp, c_i64, c_vp]),
    "ff_filter_rays": (c_i32, [_P(FFRender), c_vp, c_i64, c_i32, c_i32, c_vp, c_vp]),
    "ff_occupancy_workspace_bytes": (c_i64, [c_i32, c_i32, c_i32]),
    "ff_occupancy_mask": (c_i32, [c_vp, c_i32, c_i32, c_i32, c_f32, c_i32, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "ff_march_count": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "ff_scan_workspace_bytes": (c_i64, [c_i64]),
    "ff_scan_counts": (c_i32, [c_vp, c_i64, c_vp, c_vp, c_i64, c_vp]),
    "ff_scan_noalloc_max_counts": (c_i64, []),
    "ff_scan_counts_noalloc": (c_i32, [c_vp, c_i64, c_vp, c_vp]),
    "ff_march_emit": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "ff_composite_forward": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp,
                                     c_vp, c_vp]),
    "ff_composite_backward": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp,
                                      c_vp]),
    "ff_composite_forward_zd": (c_i32, [_P(FFRender), c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "ff_composite_backward_zd": (c_i32, [_P(FFRender), c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "ff_composite_weights": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "ff_app_emit": (c_i32, [c_i64, c_vp, c_vp, c_f32, c_vp, c_vp, c_vp, c_vp]),
    "ff_render_head_workspace_bytes": (c_i64, [_P(FFRenderMlp), c_i64]),
    "ff_render_head_forward": (c_i32, [_P(FFRenderMlp), c_vp, c_i32, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64,
                                       c_vp]),
    "ff_render_head_backward": (c_i32, [_P(FFRenderMlp), c_vp, c_i32, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp,
                                        _P(FFMlpGrad), c_vp, c_i64, c_vp]),
    "ff_render_head_forward_tc": (c_i32, [_P(FFRenderMlp), c_vp, c_i32, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "ff_render_head_backward_tc": (c_i32, [_P(FFRenderMlp), c_vp, c_i32, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp,
                                           _P(FFMlpGrad), c_vp, c_vp]),
    "ff_composite_forward_rgb": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp,
                                         c_vp, c_vp, c_vp]),
    "ff_composite_backward_rgb": (c_i32, [_P(FFRender), c_vp, c_vp, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp,
                                          c_vp, c_vp, c_vp, c_vp]),
    "ff_proposal_encode": (c_i32, [_P(FFProposal), c_vp, c_vp, c_i64, c_vp, c_vp]),
    "ff_proposal_resample": (c_i32, [_P(FFProposal), c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ff_proposal_resample_occupied": (c_i32, [_P(FFProposal), _P(FFRender), c_vp, c_i64, c_vp, c_vp, c_vp, c_vp,
                                              c_vp, c_i64, c_vp, c_vp, c_vp]),
    "ff_proposal_loss": (c_i32, [_P(FFProposal), c_vp, c_i64, c_vp, c_vp, c_vp, c_f32, c_vp, c_vp, c_vp]),
    "ff_proposal_scatter": (c_i32, [_P(FFProposal), c_vp, c_i64, c_vp, c_vp, c_vp]),
    "ff_proposal_head_forward": (c_i32, [_P(FFProposal), c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp]),
    "ff_field_render_fixed": (c_i32, [_P(FFField), c_vp, c_vp, _P(FFMlp), _P(FFRender), c_vp, c_vp, c_vp, c_i64,
                                      c_i32, c_vp, c_vp, c_vp]),
    "ff_proposal_head_infer": (c_i32, [_P(FFProposal), c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp]),
    "ff_proposal_head_backward": (c_i32, [_P(FFProposal), c_vp, _P(FFMlp), c_vp, c_i64, c_vp, c_vp,
                                          _P(FFMlpGrad), c_vp]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Load (once) and return the ctypes handle of libffgb.so; raises if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise NativeError(f"{path} is not built: run `python -m factor_fields_gb300.build` "
                              "(the CUDA extension is required; there is no fallback)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def lib():
    return _lib if _lib is not None else load()


def check(rc, what):
    if rc != FF_OK:
        msg = lib().ff_last_error().decode(errors="replace")
        raise NativeError(f"{what} failed (code {rc}): {msg}")


def ptr(t):
    """Device pointer of a tensor (or None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise NativeError("expected a CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def host_ptr(t):
    """Address of a page-locked host tensor (the FF_FIT_HOST_BATCH inputs)."""
    if t.is_cuda or not t.is_pinned():
        raise NativeError("expected a page-locked host tensor")
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


_launches = [0]
_NON_LAUNCHING = {"ff_abi_version", "ff_last_error", "ff_device_info", "ff_struct_size", "ff_scan_workspace_bytes",
                  "ff_field_fit_binned_workspace_bytes", "ff_occupancy_workspace_bytes",
                  "ff_image_metrics_workspace_bytes", "ff_render_head_workspace_bytes",
                  "ff_scan_noalloc_max_counts"}


# entry points that enqueue more than one kernel of this library
_KERNELS_PER_CALL = {"ff_scan_counts": 3, "ff_scan_counts_noalloc": 3,
                     "ff_field_fit_bin": 3,  # bin (+ zeroing), alloc, permute
                     "ff_occupancy_mask": 5,  # init, pool, unite, size, filter (3 when min_size <= 1)
                     "ff_image_metrics": 2,
                     "ff_proposal_resample_occupied": 5}  # count, scan (3), emit


def reset_launch_count():
    _launches[0] = 0


def launch_count():
    """Kernels of this library enqueued through call() since the last reset."""
    return _launches[0]


def call(name, *args, kernels=None):
    """Call an entry point and raise on a non-zero return code. kernels: how many kernels the
    call enqueues when that depends on its arguments (else _KERNELS_PER_CALL, default 1)."""
    rc = getattr(lib(), name)(*args)
    check(rc, name)
    if name not in _NON_LAUNCHING:
        _launches[0] += kernels if kernels is not None else _KERNELS_PER_CALL.get(name, 1)
