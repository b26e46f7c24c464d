"""GPU parity of the drop-in field (get_coding / get_basis / get_coeff) and MLP head against the
reference's golden outputs and the FP64 oracle.

Tolerances: float32 drop-in forward 1e-5 relative, gradients 1e-4;
BF16 storage forward 2e-2, gradients 3e-2. Relative = max|a-b| / max|ref|; the float32 drop-in
checks are also element-wise (gpu_util.assert_close: |a-b| <= rtol |ref| + 1e-6 max|ref| per entry)."""
import numpy as np
import pytest
import torch

from gpu_util import assert_close, field_cases, load_golden, model_from_golden, need_gpu, rel_err
from oracle import ff_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    need_gpu()


@pytest.mark.parametrize("case", field_cases())
def test_forward_matches_reference(case):
    d, meta = load_golden(case)
    m = model_from_golden(d, meta)
    x = torch.from_numpy(d["x"]).cuda()
    feats, coeff = m.get_coding(x)
    assert_close(feats, d["feats"], 1e-5)
    assert_close(coeff, d["coeff"], 1e-5)
    assert_close(m.get_basis(x), d["basis"], 1e-5)
    assert_close(m.get_coeff(x), d["coeff"], 1e-5)
    out = m.linear_mat(torch.from_numpy(d["feats"]).cuda())
    assert_close(out, d["mlp_out"], 1e-5)


@pytest.mark.parametrize("case", field_cases())
def test_backward_matches_reference(case):
    d, meta = load_golden(case)
    m = model_from_golden(d, meta)
    x = torch.from_numpy(d["x"]).cuda()
    feats, coeff = m.get_coding(x)
    loss = (feats * torch.from_numpy(d["g_feats"]).cuda()).sum() + (coeff * torch.from_numpy(d["g_coeff"]).cuda()).sum()
    loss.backward()
    for l in range(len(m.basis_dims)):
        assert_close(m.layout.basis_view(m.basis_flat.grad, l), d[f"grad_basis{l}"], 1e-4, what=f"level {l}")
    assert_close(m.layout.coeff_view(m.coeff_flat.grad, 0), d["grad_coeffs0"], 1e-4)
    # padding channels of the gradient stay exactly zero
    mask = torch.ones_like(m.basis_flat.grad, dtype=torch.bool)
    for l in range(len(m.basis_dims)):
        m.layout.basis_view(mask, l).fill_(False)
    assert float(m.basis_flat.grad[mask].abs().max() if mask.any() else 0) == 0.0


@pytest.mark.parametrize("case", field_cases())
def test_mlp_backward_matches_reference(case):
    d, meta = load_golden(case)
    m = model_from_golden(d, meta)
    fin = torch.from_numpy(d["feats"]).cuda().requires_grad_(True)
    out = m.linear_mat(fin)
    (out * torch.from_numpy(d["g_out"]).cuda()).sum().backward()
    assert_close(fin.grad, d["grad_mlp_in"], 1e-5)
    for i, lin in enumerate(m.linear_mat.backbone):
        assert_close(lin.weight.grad, d[f"grad_mlp_w{i}"], 1e-5)
        if lin.bias is not None:
            assert_close(lin.bias.grad, d[f"grad_mlp_b{i}"], 1e-5)


@pytest.mark.parametrize("case", field_cases())
def test_bf16_storage_within_tolerance(case):
    d, meta = load_golden(case)
    m = model_from_golden(d, meta, precision="bf16")
    x = torch.from_numpy(d["x"]).cuda()
    feats, coeff = m.get_coding(x)
    assert rel_err(feats, d["feats"]) < 2e-2
    loss = (feats * torch.from_numpy(d["g_feats"]).cuda()).sum() + (coeff * torch.from_numpy(d["g_coeff"]).cuda()).sum()
    loss.backward()
    for l in range(len(m.basis_dims)):
        assert rel_err(m.layout.basis_view(m.basis_flat.grad, l), d[f"grad_basis{l}"]) < 3e-2
    assert rel_err(m.layout.coeff_view(m.coeff_flat.grad, 0), d["grad_coeffs0"]) < 3e-2


def _oracle_spec(m):
    return O.FieldSpec(m.cfg.defaults.mode, m.cfg.dataset.aabb, m.basis_dims, m.basis_reso,
                       m.freq_bands.cpu().numpy(), m.coeff_reso, m.cfg.model.basis_mapping,
                       m.cfg.model.basis_mode, m.cfg.model.coef_mode)


@pytest.mark.parametrize("key", ["cfg0", "cfg1", "cfg2", "cfg4"])
def test_full_size_configs_against_oracle(key):
    """The benchmark configurations at full grid size, 16k points, against the FP64 oracle."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    m = FactorFields(W.field_cfg(key), device="cuda")
    if key == "cfg0":
        m.freq_bands = W.FREQ6
    g = torch.Generator(device="cpu").manual_seed(3)
    with torch.no_grad():
        m.coeff_flat.copy_(torch.rand(m.coeff_flat.shape, generator=g) * 2 - 1)
        m.basis_flat.add_((torch.rand(m.basis_flat.shape, generator=g) * 0.2 - 0.1).cuda())
    n = 16384
    aabb = np.array(m.cfg.dataset.aabb, np.float32)
    rng = np.random.default_rng(5)
    x = rng.uniform(aabb[0], aabb[1], (n, aabb.shape[1])).astype(np.float32)
    if key == "cfg4":
        x[:, 2] = rng.integers(0, 256, n) + 0.5
    spec = _oracle_spec(m)
    bg = [b[0].detach().cpu().numpy() for b in m.basises]
    cg = m.coeffs[0][0].detach().cpu().numpy()
    ref_f, ref_c = O.get_coding(spec, bg, cg, x)
    xt = torch.from_numpy(x).cuda()
    feats, coeff = m.get_coding(xt)
    assert_close(feats, ref_f, 1e-5)
    assert_close(coeff, ref_c, 1e-5)
    gf = rng.standard_normal(ref_f.shape).astype(np.float32)
    (feats * torch.from_numpy(gf).cuda()).sum().backward()
    gb, gc = O.get_coding_bwd(spec, bg, cg, x, gf)
    for l in range(len(m.basis_dims)):
        assert_close(m.layout.basis_view(m.basis_flat.grad, l)[0], gb[l], 1e-4, what=f"level {l}")
    assert_close(m.layout.coeff_view(m.coeff_flat.grad, 0)[0], gc, 1e-4)


def test_empty_batch_and_errors():
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300._native import NativeError
    m = FactorFields(W.field_cfg("cfg4", small=True), device="cuda")
    feats, coeff = m.get_coding(torch.zeros(0, 3, device="cuda"))
    assert feats.shape == (0, 18)
    with pytest.raises(NativeError):
        m.get_coding(torch.zeros(4, 3))  # CPU tensor: no fallback
