"""Generate the golden fixtures in tests/golden/ by running the REFERENCE itself.

This script is the only place that imports autonomousvision/factor-fields. It runs in a
container where a checkout of the reference is readable; its path is given by the
FF_REFERENCE_ROOT environment variable (required). It writes small .npz fixtures next to itself. The tests
and the oracle only ever read those .npz files; nothing at test time needs the reference.

How the reference is imported (it is pure Python / PyTorch):
  * modules that the field/render path never calls (skimage, cv2, plyfile, PIL,
    torchvision, kornia) are replaced by empty stub modules in sys.modules;
  * OmegaConf is replaced by a dict subclass with attribute access;
  * byte-code writing is disabled so the read-only checkout stays untouched;
  * dataLoader/ray_utils.py is loaded straight from its file (its package __init__
    imports every dataset loader).

Each fixture stores its own inputs, parameters (small grids only), outputs and gradients,
so a fixture is a complete known-answer test. Full-size configurations store the derived
shapes/resolutions and checksums of the reference's DCT initialisation instead of the
(large) parameters themselves.

Run:  FF_REFERENCE_ROOT=<checkout> PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py
"""
import importlib.util
import json
import os
import sys
import types

sys.dont_write_bytecode = True
os.environ["PYTHONDONTWRITEBYTECODE"] = "1"

import numpy as np
import torch

REF_ROOT = os.environ.get("FF_REFERENCE_ROOT")
if not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, "models")):
    sys.exit("set FF_REFERENCE_ROOT to a checkout of autonomousvision/factor-fields")
OUT_DIR = os.path.dirname(os.path.abspath(__file__))


def _install_stubs():
    for name in ["skimage", "skimage.morphology", "skimage.measure", "cv2", "plyfile",
                 "PIL", "PIL.Image", "torchvision", "torchvision.transforms", "kornia"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["cv2"].COLORMAP_JET = 2
    sys.modules["kornia"].create_meshgrid = None
    sys.modules["PIL"].Image = sys.modules["PIL.Image"]
    sys.modules["torchvision"].transforms = sys.modules["torchvision.transforms"]


_install_stubs()
sys.path.insert(0, REF_ROOT)
import models.FactorFields as RFF  # noqa: E402  (reference module)
import models.sh as RSH  # noqa: E402
import utils as RUTILS  # noqa: E402

_spec = importlib.util.spec_from_file_location("ref_ray_utils",
                                               os.path.join(REF_ROOT, "dataLoader", "ray_utils.py"))
RRAY = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(RRAY)


class Cfg(dict):
    """OmegaConf stand-in: attribute access, missing keys read as None."""
    __getattr__ = dict.get

    def __setattr__(self, k, v):
        self[k] = v


def mkcfg(d):
    return Cfg({k: (mkcfg(v) if isinstance(v, dict) else v) for k, v in d.items()})


def base_cfg(mode, aabb, **model):
    m = dict(coeff_type="grid", basis_type="grid", basis_mapping="sawtooth",
             basis_dims=[4, 4, 4, 2, 2, 2], basis_resos=[32, 51, 70, 89, 108, 128],
             freq_bands=[2.0, 3.2, 4.4, 5.6, 6.8, 8.0], coeff_reso=32, total_params=0,
             T_basis=0, T_coeff=0, coef_init=1.0, coef_mode="bilinear", basis_mode="bilinear",
             num_layers=2, hidden_dim=64, out_dim=3, with_dropout=False)
    m.update(model)
    return mkcfg({
        "defaults": {"mode": mode},
        "model": m,
        "dataset": {"aabb": aabb, "scene_reso": 1024, "is_unbound": False, "dataset_name": "synthetic"},
        "training": {"volume_resoInit": 128, "volume_resoFinal": 300, "linear_mat": True,
                     "coeff": True, "basis": True, "renderModule": True},
        "renderer": {"view_pe": 6, "fea_pe": 2, "num_layers": 3, "hidden_dim": 128,
                     "fea2denseAct": "softplus", "density_shift": -10.0, "distance_scale": 25.0,
                     "step_ratio": 0.5, "rayMarch_weight_thres": 1e-3, "alphaMask_thres": 0.02},
    })


def plain(cfg):
    """cfg -> plain nested dict for JSON."""
    return {k: (plain(v) if isinstance(v, dict) else v) for k, v in cfg.items()}


def build(cfg, freq_override=None):
    torch.manual_seed(0)
    m = RFF.FactorFields(cfg, "cpu")
    if freq_override is not None:
        m.freq_bands = torch.tensor(freq_override, dtype=torch.float32)
    return m


def randomise(m, rng, coeff_scale=1.0, basis_noise=0.25):
    """Seeded, stored perturbation of every parameter so the fixtures exercise real values."""
    with torch.no_grad():
        for b in m.basises:
            b.add_(torch.from_numpy(rng.uniform(-basis_noise, basis_noise, b.shape).astype(np.float32)))
        for c in m.coeffs:
            c.copy_(torch.from_numpy(rng.uniform(-coeff_scale, coeff_scale, c.shape).astype(np.float32)))
        for lin in m.linear_mat.backbone:
            lin.weight.copy_(torch.from_numpy(rng.uniform(-0.3, 0.3, lin.weight.shape).astype(np.float32)))
            if lin.bias is not None:
                lin.bias.copy_(torch.from_numpy(rng.uniform(-0.1, 0.1, lin.bias.shape).astype(np.float32)))


def boundary_points(m, rng, n):
    """Points that sit exactly on mapping period boundaries (x - aabb0 = k * scale_l)."""
    aabb = m.aabb[:, :m.in_dim].numpy()
    size = np.float32(max(aabb[1] - aabb[0]))
    scale = (torch.tensor(size) / m.freq_bands).numpy()
    pts = []
    for _ in range(n):
        lvl = rng.integers(0, len(scale))
        p = rng.uniform(aabb[0], aabb[1]).astype(np.float32)
        ax = rng.integers(0, m.in_dim)
        k = rng.integers(0, int(np.floor((aabb[1][ax] - aabb[0][ax]) / scale[lvl])) + 1)
        p[ax] = np.float32(aabb[0][ax] + np.float32(k * scale[lvl]))
        pts.append(p)
    return np.stack(pts).astype(np.float32)


def field_case(name, cfg, n_pts, seed, freq_override=None, outside=0.0, extra_dim_values=None):
    rng = np.random.default_rng(seed)
    m = build(cfg, freq_override)
    randomise(m, rng)
    in_dim = m.in_dim
    full_dim = len(cfg.dataset.aabb[0])
    aabb_full = np.array(cfg.dataset.aabb, dtype=np.float32)
    lo, hi = aabb_full[0], aabb_full[1]
    span = hi - lo
    x = rng.uniform(lo - outside * span, hi + outside * span, size=(n_pts, full_dim)).astype(np.float32)
    nb = max(4, n_pts // 8)
    xb = boundary_points(m, rng, nb)
    if full_dim > in_dim:  # images mode: last coordinate is the image index + 0.5
        zb = (rng.integers(0, int(hi[-1]), size=(nb, 1)) + 0.5).astype(np.float32)
        xb = np.concatenate([xb, zb], 1)
    x = np.concatenate([x, xb], 0)
    if extra_dim_values is not None:
        x[:, -1] = extra_dim_values(rng, x.shape[0])
    xt = torch.from_numpy(x)

    feats, coeff = m.get_coding(xt)
    basis = m.get_basis(xt)
    out = m.linear_mat(feats, is_train=False)
    g_feats = rng.standard_normal(feats.shape).astype(np.float32)
    g_coeff = rng.standard_normal(coeff.shape).astype(np.float32)
    g_out = rng.standard_normal(out.shape).astype(np.float32)
    # gradients of a linear test loss through each output
    m.zero_grad()
    loss = (feats * torch.from_numpy(g_feats)).sum() + (coeff * torch.from_numpy(g_coeff)).sum()
    loss.backward()
    d = dict(x=x, feats=feats.detach().numpy(), coeff=coeff.detach().numpy(), basis=basis.detach().numpy(),
             mlp_out=out.detach().numpy(), g_feats=g_feats, g_coeff=g_coeff, g_out=g_out)
    for i, b in enumerate(m.basises):
        d[f"basis{i}"] = b.detach().numpy()
        d[f"grad_basis{i}"] = b.grad.numpy().copy()
    d["coeffs0"] = m.coeffs[0].detach().numpy()
    d["grad_coeffs0"] = m.coeffs[0].grad.numpy().copy()
    # MLP: gradient of sum(out * g_out) wrt MLP weights and wrt its input
    m.zero_grad()
    fin = feats.detach().clone().requires_grad_(True)
    out2 = m.linear_mat(fin, is_train=False)
    (out2 * torch.from_numpy(g_out)).sum().backward()
    d["grad_mlp_in"] = fin.grad.numpy()
    for i, lin in enumerate(m.linear_mat.backbone):
        d[f"mlp_w{i}"] = lin.weight.detach().numpy()
        d[f"grad_mlp_w{i}"] = lin.weight.grad.numpy().copy()
        if lin.bias is not None:
            d[f"mlp_b{i}"] = lin.bias.detach().numpy()
            d[f"grad_mlp_b{i}"] = lin.bias.grad.numpy().copy()
    meta = dict(cfg=plain(cfg), freq_bands=m.freq_bands.tolist(), basis_reso=list(map(int, m.basis_reso)),
                coeff_reso=list(map(int, m.coeff_reso)), aabb=m.aabb.tolist(), in_dim=int(m.in_dim),
                n_levels=len(m.basises))
    d["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT_DIR, f"field_{name}.npz"), **d)
    print("field", name, x.shape, [b.shape for b in m.basises], m.coeffs[0].shape)


class SHRender(torch.nn.Module):
    """Config-2 colour head composed from the reference's own eval_sh (models/sh.py:34)."""

    def forward(self, viewdirs, features):
        sh = features.view(-1, 3, 9)
        return torch.sigmoid(RSH.eval_sh(2, sh, viewdirs))


def hemisphere_rays(rng, n, radius, target_jitter):
    th = rng.uniform(0, 2 * np.pi, n)
    ph = np.arccos(rng.uniform(0.05, 1.0, n))  # upper hemisphere
    o = np.stack([radius * np.sin(ph) * np.cos(th), radius * np.sin(ph) * np.sin(th), radius * np.cos(ph)], 1)
    tgt = rng.uniform(-target_jitter, target_jitter, (n, 3))
    dvec = tgt - o
    dvec /= np.linalg.norm(dvec, axis=1, keepdims=True)
    return np.concatenate([o, dvec], 1).astype(np.float32)


def render_case(name, seed, n_rays, n_samples, head, alpha_volume_shape=None, white_bg=True,
                jitter=False, resos=(5, 6, 7, 8, 9, 10), coeff_reso=6, axis_rays=0):
    rng = np.random.default_rng(seed)
    out_dim = 28 if head == "sh" else 28
    cfg = base_cfg("reconstruction", [[-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]], basis_mapping="triangle",
                   basis_resos=list(resos), coeff_reso=coeff_reso, out_dim=out_dim)
    n_basis = int(sum(np.power(np.array(resos), 3) * np.array(cfg.model.basis_dims)))
    cfg.model.total_params = 18 * coeff_reso ** 3 + n_basis
    m = build(cfg)
    randomise(m, rng, coeff_scale=1.0)
    with torch.no_grad():
        # Calibrate the density row so that softplus(f0 - 10) spans transparent to opaque: make the
        # row positive and scale it so that f0 has a mean of about 9 over the box.
        probe = torch.from_numpy(rng.uniform(-1.5, 1.5, (4096, 3)).astype(np.float32))
        w_last = m.linear_mat.backbone[-1].weight
        w_last[0].abs_()
        f0 = m.linear_mat(m.get_coding(probe)[0])[:, 0]
        w_last[0].mul_(9.0 / float(f0.mean()))
        if head == "mlp":
            for lin in m.renderModule.mlp:
                lin.weight.copy_(torch.from_numpy(rng.uniform(-0.2, 0.2, lin.weight.shape).astype(np.float32)))
                if lin.bias is not None:
                    lin.bias.copy_(torch.from_numpy(rng.uniform(-0.1, 0.1, lin.bias.shape).astype(np.float32)))
    if head == "sh":
        m.renderModule = SHRender()
    alpha_vol = None
    if alpha_volume_shape is not None:
        alpha_vol = (rng.uniform(0, 1, alpha_volume_shape) < 0.6).astype(np.float32)  # [D,H,W]
        m.alphaMask = RFF.AlphaGridMask("cpu", m.aabb, torch.from_numpy(alpha_vol))
    rays = hemisphere_rays(rng, n_rays, 4.0, 0.8)
    if axis_rays:  # rays with exactly-zero direction components (the 1e-6 substitution)
        ax = np.zeros((axis_rays, 6), np.float32)
        ax[:, 0] = rng.uniform(-1.0, 1.0, axis_rays)
        ax[:, 1] = rng.uniform(-1.0, 1.0, axis_rays)
        ax[:, 2] = 4.0
        ax[:, 5] = -1.0
        rays = np.concatenate([rays, ax], 0)
    u = rng.uniform(0, 1, (rays.shape[0], 1)).astype(np.float32)
    rays_t = torch.from_numpy(rays)

    orig_rand_like, orig_rand = torch.rand_like, torch.rand
    try:
        if jitter:
            torch.rand_like = lambda t, *a, **k: torch.from_numpy(u).to(t.dtype).reshape(t.shape)
            torch.rand = lambda *a, **k: torch.ones(1)  # white-background coin: never flips
        m.zero_grad()
        rgb, depth, coeffs = m(rays_t, white_bg=white_bg, is_train=jitter, N_samples=n_samples)
        xyz, z_vals, inner = m.sample_point(rays_t[:, :3], rays_t[:, 3:6], is_train=jitter, N_samples=n_samples)
    finally:
        torch.rand_like, torch.rand = orig_rand_like, orig_rand
    g_rgb = rng.standard_normal(rgb.shape).astype(np.float32)
    (rgb * torch.from_numpy(g_rgb)).sum().backward()
    valid = inner.clone()
    if alpha_vol is not None:
        valid[inner.clone()] = m.alphaMask.sample_alpha(xyz[inner]) > 0.5
    d = dict(rays=rays, u=u, rgb=rgb.detach().numpy(), depth=depth.detach().numpy(), g_rgb=g_rgb,
             z_vals=z_vals.numpy(), inner=inner.numpy(), valid=valid.numpy(),
             step_size=np.float32(m.stepSize.item()), n_samples=np.int64(n_samples))
    if alpha_vol is not None:
        d["alpha_volume"] = alpha_vol
    for i, b in enumerate(m.basises):
        d[f"basis{i}"] = b.detach().numpy()
        d[f"grad_basis{i}"] = b.grad.numpy().copy()
    d["coeffs0"] = m.coeffs[0].detach().numpy()
    d["grad_coeffs0"] = m.coeffs[0].grad.numpy().copy()
    for i, lin in enumerate(m.linear_mat.backbone):
        d[f"mlp_w{i}"] = lin.weight.detach().numpy()
        d[f"grad_mlp_w{i}"] = lin.weight.grad.numpy().copy()
        if lin.bias is not None:
            d[f"mlp_b{i}"] = lin.bias.detach().numpy()
            d[f"grad_mlp_b{i}"] = lin.bias.grad.numpy().copy()
    if head == "mlp":
        for i, lin in enumerate(m.renderModule.mlp):
            d[f"rm_w{i}"] = lin.weight.detach().numpy()
            d[f"grad_rm_w{i}"] = lin.weight.grad.numpy().copy()
            if lin.bias is not None:
                d[f"rm_b{i}"] = lin.bias.detach().numpy()
                d[f"grad_rm_b{i}"] = lin.bias.grad.numpy().copy()
    meta = dict(cfg=plain(cfg), head=head, white_bg=white_bg, jitter=jitter, freq_bands=m.freq_bands.tolist(),
                basis_reso=list(map(int, m.basis_reso)), coeff_reso=list(map(int, m.coeff_reso)),
                aabb=m.aabb.tolist(), grid_size=m.gridSize.tolist(), n_samples_default=int(m.nSamples))
    d["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT_DIR, f"render_{name}.npz"), **d)
    print("render", name, rays.shape, "valid", int(valid.sum()), "of", valid.numel(),
          "rgb mean", float(rgb.mean()), "depth mean", float(depth.mean()))


def small_primitives():
    rng = np.random.default_rng(7)
    d = {}
    # raw2alpha (models/FactorFields.py:82)
    sigma = np.abs(rng.standard_normal((16, 40))).astype(np.float32) * 3
    sigma[:, ::5] = 0
    dist = rng.uniform(0, 0.05, (16, 40)).astype(np.float32)
    dist[:, -1] = 0
    a, w, t = RFF.raw2alpha(torch.from_numpy(sigma), torch.from_numpy(dist))
    d.update(r2a_sigma=sigma, r2a_dist=dist, r2a_alpha=a.numpy(), r2a_weight=w.numpy(), r2a_bg=t.numpy())
    # eval_sh degree 2 (models/sh.py:34)
    sh = rng.standard_normal((64, 3, 9)).astype(np.float32)
    dirs = rng.standard_normal((64, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    d.update(sh_coef=sh, sh_dirs=dirs, sh_out=RSH.eval_sh(2, torch.from_numpy(sh), torch.from_numpy(dirs)).numpy())
    # sample_pdf (dataLoader/ray_utils.py:132): deterministic and fixed-u variants
    bins = np.sort(rng.uniform(0, 6, (32, 65)).astype(np.float32), axis=1)
    wts = rng.uniform(0, 1, (32, 64)).astype(np.float32)
    wts[:4] = 0
    wts[4:8, 10:] = 0
    s_det = RRAY.sample_pdf(torch.from_numpy(bins), torch.from_numpy(wts), 48, det=True)
    s_fix = RRAY.sample_pdf(torch.from_numpy(bins), torch.from_numpy(wts), 48, det=False, pytest=True)
    np.random.seed(0)
    u_fix = np.random.rand(32, 48).astype(np.float32)
    d.update(pdf_bins=bins, pdf_weights=wts, pdf_det=s_det.numpy(), pdf_fixed=s_fix.numpy(), pdf_u_fixed=u_fix)
    # grid_mapping (models/FactorFields.py:11) incl. negative offsets and boundaries
    aabb = torch.tensor([[-1.0, -1.0, -1.0], [1.0, 1.0, 1.0]])
    freqs = torch.tensor([2.0, 3.2, 4.4, 5.6, 6.8, 8.0])
    pos = rng.uniform(-1.2, 1.2, (256, 3)).astype(np.float32)
    scale = (torch.tensor(2.0) / freqs).numpy()
    for i in range(0, 64):
        pos[i, i % 3] = np.float32(-1.0 + np.float32((i // 3) % 9) * scale[i % 6])
    for mode in ["sawtooth", "triangle"]:
        d[f"map_{mode}"] = RFF.grid_mapping(torch.from_numpy(pos), freqs, aabb, mode).numpy()
    d["map_pos"] = pos
    d["map_freqs"] = freqs.numpy()
    # dct_dict checksums (models/FactorFields.py:36) for the 2-D and 3-D default levels
    for dim in (2, 3):
        for C, R in zip([4, 4, 4, 2, 2, 2], [32, 51, 70, 89, 108, 128]):
            k = RFF.dct_dict(int(np.power(C, 1.0 / dim) + 1), R, n_selete=C, dim=dim).numpy()
            d[f"dct{dim}_{C}_{R}_sum"] = np.float64(k.astype(np.float64).sum())
            d[f"dct{dim}_{C}_{R}_abs"] = np.float64(np.abs(k.astype(np.float64)).sum())
            d[f"dct{dim}_{C}_{R}_head"] = k[:, :64].copy()
    # N_to_reso (utils.py:53)
    d["n2r_cases"] = np.array([[128 ** 3, 3], [32 ** 3, 3], [271 * 271, 2], [64 ** 3, 3]], dtype=np.int64)
    d["n2r_out"] = np.array([RUTILS.N_to_reso(int(n), torch.tensor([[-1.5] * dm, [1.5] * dm]))[0]
                             for n, dm in d["n2r_cases"]], dtype=np.int64)
    np.savez_compressed(os.path.join(OUT_DIR, "primitives.npz"), **d)
    print("primitives ok")


def config_shapes():
    """Derived sizes of the five benchmark configurations (setup_params, :262-309)."""
    out = {}
    base_resos = [32, 51, 70, 89, 108, 128]
    n_basis3 = int(sum(np.power(np.array(base_resos), 3) * np.array([4, 4, 4, 2, 2, 2])))
    recipes = {
        "cfg0": (base_cfg("image", [[0, 0], [512, 512]], total_params=1426063, out_dim=3),
                 [2.0, 3.2, 4.4, 5.6, 6.8, 8.0]),
        "cfg1": (base_cfg("reconstruction", [[-1, -1, -1], [1, 1, 1]], coeff_reso=32,
                          total_params=18 * 32 ** 3 + n_basis3, out_dim=1), None),
        "cfg2": (base_cfg("reconstruction", [[-1.5] * 3, [1.5] * 3], coeff_reso=64, basis_mapping="triangle",
                          total_params=18 * 64 ** 3 + n_basis3, out_dim=28), None),
        "cfg4": (base_cfg("images", [[0, 0, 0], [256, 256, 256]], T_coeff=32 * 32 * 18, out_dim=3), None),
    }
    for k, (cfg, fo) in recipes.items():
        m = build(cfg, fo)
        rec = dict(basis_reso=list(map(int, m.basis_reso)), coeff_shape=list(m.coeffs[0].shape),
                   freq_bands=[float(f) for f in m.freq_bands], basis_shapes=[list(b.shape) for b in m.basises],
                   n_params=int(m.n_parameters()))
        if hasattr(m, "stepSize"):
            rec.update(step_size=float(m.stepSize), n_samples=int(m.nSamples), grid_size=m.gridSize.tolist())
        rec["basis_sums"] = [float(b.detach().double().sum()) for b in m.basises]
        out[k] = rec
    with open(os.path.join(OUT_DIR, "config_shapes.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("config shapes ok")


def main():
    small_primitives()
    config_shapes()
    # field cases: small grids, every parameter stored
    f6 = [2.0, 3.2, 4.4, 5.6, 6.8, 8.0]
    field_case("img2d_saw", base_cfg("image", [[0, 0], [40, 30]], basis_resos=[3, 4, 5, 6, 7, 9],
                                     total_params=0, T_coeff=18 * 63, out_dim=3), 400, 1, freq_override=f6)
    field_case("img2d_tri", base_cfg("image", [[0, 0], [40, 30]], basis_resos=[3, 4, 5, 6, 7, 9],
                                     basis_mapping="triangle", T_coeff=18 * 63, out_dim=3), 400, 2,
               freq_override=f6, outside=0.05)
    field_case("img2d_nearest", base_cfg("image", [[0, 0], [40, 30]], basis_resos=[3, 4, 5, 6, 7, 9],
                                         T_coeff=18 * 63, out_dim=3, coef_mode="nearest",
                                         basis_mode="nearest"), 400, 3, freq_override=f6)
    n3 = int(sum(np.power(np.array([3, 4, 5, 6, 7, 8]), 3) * np.array([4, 4, 4, 2, 2, 2])))
    field_case("rec3d_saw", base_cfg("reconstruction", [[-1, -1, -1], [1, 1, 1]], basis_resos=[3, 4, 5, 6, 7, 8],
                                     coeff_reso=5, total_params=18 * 125 + n3, out_dim=1), 400, 4, outside=0.03)
    field_case("rec3d_tri", base_cfg("reconstruction", [[-1.5] * 3, [1.5] * 3], basis_resos=[3, 4, 5, 6, 7, 8],
                                     basis_mapping="triangle", coeff_reso=5, total_params=18 * 125 + n3,
                                     out_dim=28), 400, 5)
    field_case("rec3d_aniso", base_cfg("reconstruction", [[-1.0, -0.5, -0.25], [1.0, 0.5, 0.25]],
                                       basis_resos=[3, 4, 5, 6, 7, 8], basis_mapping="triangle", coeff_reso=6,
                                       total_params=18 * 216 + n3, out_dim=4, num_layers=3), 400, 6)
    field_case("images", base_cfg("images", [[0, 0, 0], [16, 12, 5]], basis_resos=[3, 4, 5, 6, 7, 9],
                                  T_coeff=18 * 30, out_dim=3), 400, 8,
               extra_dim_values=lambda rng, n: (rng.integers(0, 5, n) + 0.5).astype(np.float32))
    # render cases
    render_case("sh_plain", 11, 48, 400, "sh", axis_rays=4)
    render_case("sh_alpha", 12, 48, 400, "sh", alpha_volume_shape=(9, 10, 11))
    render_case("sh_jitter_black", 13, 40, 300, "sh", white_bg=False, jitter=True)
    render_case("mlp_head", 14, 24, 400, "mlp")


if __name__ == "__main__":
    main()
