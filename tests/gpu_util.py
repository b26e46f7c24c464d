"""Helpers shared by the GPU tests: build models from golden fixtures, error metrics."""
import glob
import json
import os

import numpy as np
import pytest
import torch

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from factor_fields_gb300 import build
    build.build()


def load_golden(name):
    d = dict(np.load(os.path.join(GOLD, name)))
    meta = json.loads(str(d.pop("meta"))) if "meta" in d else None
    return d, meta


def field_cases():
    return sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLD, "field_*.npz")))


def render_cases():
    return sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLD, "render_*.npz")))


def reference_sd(d, n_levels, prefix_mlp="mlp"):
    sd = {f"basises.{i}": torch.from_numpy(d[f"basis{i}"]) for i in range(n_levels)}
    sd["coeffs.0"] = torch.from_numpy(d["coeffs0"])
    i = 0
    while f"{prefix_mlp}_w{i}" in d:
        sd[f"linear_mat.backbone.{i}.weight"] = torch.from_numpy(d[f"{prefix_mlp}_w{i}"])
        if f"{prefix_mlp}_b{i}" in d:
            sd[f"linear_mat.backbone.{i}.bias"] = torch.from_numpy(d[f"{prefix_mlp}_b{i}"])
        i += 1
    i = 0
    while f"rm_w{i}" in d:  # MLPRender_Fea (renderModule.mlp.i)
        sd[f"renderModule.mlp.{i}.weight"] = torch.from_numpy(d[f"rm_w{i}"])
        if f"rm_b{i}" in d:
            sd[f"renderModule.mlp.{i}.bias"] = torch.from_numpy(d[f"rm_b{i}"])
        i += 1
    return sd


def model_from_golden(d, meta, precision="fp32"):
    """The model of a golden fixture with the reference's parameters. Render fixtures made with
    the SH-2 head (meta head != 'mlp') get renderer.shadingMode = 'SH'; the others keep the
    reference's MLPRender_Fea."""
    import copy
    from factor_fields_gb300 import FactorFields, make_cfg
    cfg = make_cfg(copy.deepcopy(meta["cfg"]))
    if "head" in meta:
        cfg.renderer = cfg.renderer or make_cfg({})
        cfg.renderer["shadingMode"] = "MLP_Fea" if meta["head"] == "mlp" else "SH"
    m = FactorFields(cfg, device="cuda", precision=precision)
    m.freq_bands = meta["freq_bands"]
    m.load_reference_state_dict(reference_sd(d, len(m.basis_dims)))
    return m


def rel_err(a, b):
    """max |a - b| / max |b| (the tolerance convention of every parity test)."""
    a = np.asarray(a.detach().cpu().numpy() if torch.is_tensor(a) else a, np.float64)
    b = np.asarray(b.detach().cpu().numpy() if torch.is_tensor(b) else b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def elem_err(a, b, rtol, atol_rel=1e-6):
    """Element-wise check beside rel_err: the largest ratio |a - b| / (rtol |b| + atol) over the
    elements, with atol = atol_rel * max|b| (<= 1 passes). rel_err alone lets entries far below
    the maximum drift by much more than rtol of their own size; this bounds each entry by rtol
    of itself plus a floor. The floor 1e-6 * max|ref| sits above the reference's own float32
    rounding: its golden outputs differ from the exact (FP64 oracle) values by up to
    ~6e-7 * max|ref| element-wise."""
    a = np.asarray(a.detach().cpu().numpy() if torch.is_tensor(a) else a, np.float64)
    b = np.asarray(b.detach().cpu().numpy() if torch.is_tensor(b) else b, np.float64)
    atol = atol_rel * max(float(np.max(np.abs(b))), 1e-30)
    return float(np.max(np.abs(a - b) / (rtol * np.abs(b) + atol)))


def assert_close(a, b, rtol, atol_rel=1e-6, what=""):
    """rel_err(a, b) < rtol and elem_err(a, b, rtol, atol_rel) <= 1, with both in the message."""
    r, e = rel_err(a, b), elem_err(a, b, rtol, atol_rel)
    assert r < rtol and e <= 1.0, f"{what}: rel_err {r:.3g} (< {rtol:g}), elem_err {e:.3g} (<= 1, floor {atol_rel:g} max|ref|)"


# Floor of the element-wise check for gradients that pass through the compositing chain (the
# reverse transmittance scan, the colour head and the MLP before the grid scatter): the
# reference's own float32 render gradients differ from the exact (FP64 oracle) values by up to
# ~7e-7 * max|ref| element-wise on the golden renders.
RENDER_GRAD_FLOOR = 3e-6
