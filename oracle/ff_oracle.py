"""CPU oracle for the Factor Fields field-evaluation and ray-rendering path.

TEST INFRASTRUCTURE ONLY. This module is the oracle: only tests/, the smoke check in
__graft_entry__.py and bench.py's CPU-baseline leg may import it. The product path
(factor_fields_gb300) never calls into it.

It is a NumPy restatement of the reference's algorithm (autonomousvision/factor-fields), with
each function citing the reference file:line it follows. Conventions:
  * Everything that decides WHICH cell / sample / bit is used (coordinate mapping, grid
    unnormalisation, floor/round, in-box tests, sample positions) is evaluated in float32
    with the same operation order as the reference's PyTorch ops, so indices, masks and
    interpolation weights are bit-identical to the reference.
  * Accumulations (interpolation sums, MLP matmuls, compositing sums, gradients) run in
    float64: this is the FP64 oracle that the GPU results are measured against.
Parity is pinned: tests/test_oracle_golden.py checks this module against fixtures produced
by running the reference itself (tests/golden/make_golden.py).
"""
import math

import numpy as np

f32 = np.float32
f64 = np.float64


# ----------------------------------------------------------------------------------------
# configuration derivation
# ----------------------------------------------------------------------------------------

def n_to_reso(n_voxels, aabb):
    """utils.py:53-57 — voxel resolution with n_voxels cells over aabb (float32 like torch)."""
    aabb = np.asarray(aabb, dtype=f32)
    size = (aabb[1] - aabb[0]).astype(f32)
    dim = size.shape[0]
    # torch: ((xyz_max - xyz_min).prod() / n_voxels).pow(1 / dim) in float32
    prod = f32(np.prod(size, dtype=f32))
    voxel = f32(np.power(f32(prod / f32(n_voxels)), f32(1.0 / dim)))
    return [int(v) for v in np.round((size / voxel).astype(f32))]


def dct_dict(n_atoms_fre, size, n_select, dim=2):
    """models/FactorFields.py:36-71 — DCT dictionary used to initialise each basis level."""
    p = n_atoms_fre
    dct = np.zeros((p, size))
    for k in range(p):
        basis = np.cos(np.arange(size) * k * math.pi / p)
        if k > 0:
            basis = basis - np.mean(basis)
        dct[k] = basis
    kron = np.kron(dct, dct)
    if dim == 3:
        kron = np.kron(kron, dct)
    if n_select < kron.shape[0]:
        idx = [x[0] for x in np.array_split(np.arange(kron.shape[0]), n_select)]
        kron = kron[idx]
    for col in range(kron.shape[0]):
        norm = np.linalg.norm(kron[col]) or 1
        kron[col] /= norm
    return kron.astype(f32)


def basis_init(basis_dims, basis_reso, in_dim):
    """models/FactorFields.py:397-409 — DCT initialisation of each grid level, [C, R(,R),R]."""
    out = []
    for c, r in zip(basis_dims, basis_reso):
        k = dct_dict(int(np.power(c, 1.0 / in_dim) + 1), r, n_select=c, dim=in_dim)
        out.append(k.reshape([c] + [r] * in_dim))
    return out


# ----------------------------------------------------------------------------------------
# float32 arithmetic helpers with PyTorch (Python) semantics
# ----------------------------------------------------------------------------------------

def py_remainder(a, b):
    """torch.remainder on floats: fmod, then shift into the divisor's sign."""
    a = np.asarray(a, f32)
    b = np.asarray(b, f32)
    mod = np.fmod(a, b).astype(f32)
    fix = (mod != 0) & ((b < 0) != (mod < 0))
    return np.where(fix, (mod + b).astype(f32), mod).astype(f32)


def py_floordiv(a, b):
    """torch.floor_divide on floats (c10::div_floor_floating)."""
    a = np.asarray(a, f32)
    b = np.asarray(b, f32)
    mod = np.fmod(a, b).astype(f32)
    div = ((a - mod).astype(f32) / b).astype(f32)
    fix = (mod != 0) & ((b < 0) != (mod < 0))
    div = np.where(fix, (div - f32(1)).astype(f32), div)
    fl = np.floor(div).astype(f32)
    fl = np.where((div - fl).astype(f32) > f32(0.5), (fl + f32(1)).astype(f32), fl)
    basic = (a / b).astype(f32)
    fl = np.where(div == 0, np.copysign(f32(0), basic), fl)
    return fl.astype(f32)


def grid_mapping(pos, freq_bands, aabb0, aabb_size, mode):
    """models/FactorFields.py:11-33 — per-level local coordinates, [N, d] -> [N, d, L] float32.

    aabb_size is max(aabb[1]-aabb[0]) over the mapped dims (a scalar), as at :12.
    """
    pos = np.asarray(pos, f32)
    freq = np.asarray(freq_bands, f32)
    scale = (f32(aabb_size) / freq).astype(f32)  # :13
    half = (scale / f32(2)).astype(f32)
    rel = (pos - np.asarray(aabb0, f32)).astype(f32)[..., None]
    if mode == "triangle":  # :14-18
        loc = py_remainder(rel, scale)
        odd = py_remainder(py_floordiv(rel, scale), f32(2))
        loc = ((loc / half).astype(f32) - f32(1)).astype(f32)
        return np.where(odd == 1, -loc, loc).astype(f32)
    if mode == "sawtooth":  # :19-22
        loc = py_remainder(rel, scale)
        loc = ((loc / half).astype(f32) - f32(1)).astype(f32)
        return np.clip(loc, f32(-1), f32(1)).astype(f32)
    raise ValueError(f"unsupported basis_mapping {mode!r}")


def normalize_coord(x, aabb0, aabb1):
    """models/FactorFields.py:635-637 — map the aabb to [-1, 1] (float32)."""
    inv = (f32(2.0) / (np.asarray(aabb1, f32) - np.asarray(aabb0, f32)).astype(f32)).astype(f32)
    return (((np.asarray(x, f32) - np.asarray(aabb0, f32)).astype(f32) * inv).astype(f32) - f32(1)).astype(f32)


# ----------------------------------------------------------------------------------------
# grid_sample (ATen semantics) forward and backward
# ----------------------------------------------------------------------------------------

def _unnormalize(coord, size, align_corners):
    """ATen grid_sampler_unnormalize, in float32."""
    c = np.asarray(coord, f32)
    if align_corners:
        return (((c + f32(1)).astype(f32) / f32(2)).astype(f32) * f32(size - 1)).astype(f32)
    return ((((c + f32(1)).astype(f32) * f32(size)).astype(f32) - f32(1)).astype(f32) / f32(2)).astype(f32)


def _source_index(coord, size, align_corners, padding):
    ix = _unnormalize(coord, size, align_corners)
    if padding == "border":
        ix = np.minimum(f32(size - 1), np.maximum(ix, f32(0))).astype(f32)
    return ix


def sample_corners(coords, sizes, align_corners, padding, mode):
    """Corner list for bi/trilinear (or nearest) sampling.

    coords: [N, d] normalised coordinates, component k indexes grid axis sizes[k]
    (sizes given in x, y, z order = W, H, D). Returns a list of (flat_index[N], weight[N] f32,
    valid[N]) with flat index = ((z * H) + y) * W + x.
    """
    n, d = coords.shape
    idx = [_source_index(coords[:, k], sizes[k], align_corners, padding) for k in range(d)]
    if mode == "nearest":
        ri = [np.rint(v).astype(np.int64) for v in idx]  # nearbyint: round half to even
        valid = np.ones(n, bool)
        for k in range(d):
            valid &= (ri[k] >= 0) & (ri[k] < sizes[k])
        flat = np.zeros(n, np.int64)
        for k in reversed(range(d)):
            flat = flat * sizes[k] + np.clip(ri[k], 0, sizes[k] - 1)
        return [(flat, np.ones(n, f32), valid)]
    lo = [np.floor(v).astype(f32) for v in idx]
    hi = [(v + f32(1)).astype(f32) for v in lo]
    w_lo = [(hi[k] - idx[k]).astype(f32) for k in range(d)]  # weight of the low corner
    w_hi = [(idx[k] - lo[k]).astype(f32) for k in range(d)]
    corners = []
    for bits in range(1 << d):
        # ATen order: x fastest varying low->high (nw, ne, sw, se, then the back z slice)
        w = None
        flat = np.zeros(n, np.int64)
        valid = np.ones(n, bool)
        ci = []
        for k in range(d):
            hi_k = (bits >> k) & 1
            c = (hi[k] if hi_k else lo[k]).astype(np.int64)
            wk = w_hi[k] if hi_k else w_lo[k]
            w = wk if w is None else (w * wk).astype(f32)
            valid &= (c >= 0) & (c < sizes[k])
            ci.append(c)
        for k in reversed(range(d)):
            flat = flat * sizes[k] + np.clip(ci[k], 0, sizes[k] - 1)
        corners.append((flat, w.astype(f32), valid))
    return corners


def grid_sample_fwd(grid, coords, align_corners, padding, mode):
    """F.grid_sample for a single [C, (D,) H, W] grid at N points -> [N, C] float64."""
    c = grid.shape[0]
    sizes = list(grid.shape[1:][::-1])  # x, y, z sizes
    g = np.asarray(grid, f64).reshape(c, -1)
    out = np.zeros((coords.shape[0], c), f64)
    for flat, w, valid in sample_corners(coords, sizes, align_corners, padding, mode):
        out += g[:, flat].T * (w.astype(f64) * valid)[:, None]
    return out


def grid_sample_bwd(grid_shape, coords, grad_out, align_corners, padding, mode):
    """Gradient of sum(grad_out * grid_sample(grid)) wrt the grid (ATen scatter-add), float64."""
    c = grid_shape[0]
    sizes = list(grid_shape[1:][::-1])
    gg = np.zeros((c, int(np.prod(grid_shape[1:]))), f64)
    go = np.asarray(grad_out, f64)
    for flat, w, valid in sample_corners(coords, sizes, align_corners, padding, mode):
        contrib = go * (w.astype(f64) * valid)[:, None]
        for ch in range(c):
            np.add.at(gg[ch], flat[valid], contrib[valid, ch])
    return gg.reshape(grid_shape)


# ----------------------------------------------------------------------------------------
# the field: get_coeff / get_basis / get_coding (+ backward)
# ----------------------------------------------------------------------------------------

class FieldSpec:
    """Derived configuration of one grid/grid factor field (models/FactorFields.py:262-309)."""

    def __init__(self, mode, aabb, basis_dims, basis_reso, freq_bands, coeff_reso, mapping,
                 basis_mode="bilinear", coef_mode="bilinear"):
        self.mode = mode
        self.aabb_full = np.asarray(aabb, f32)
        self.full_dim = self.aabb_full.shape[1]
        self.in_dim = self.full_dim - 1 if mode in ("images", "reconstructions") else self.full_dim
        self.basis_dims = list(basis_dims)
        self.basis_reso = list(basis_reso)
        self.freq_bands = np.asarray(freq_bands, f32)
        self.coeff_reso = list(coeff_reso)  # grid axes order (D,) H, W as in the reference
        self.mapping = mapping
        self.basis_mode = basis_mode
        self.coef_mode = coef_mode
        a = self.aabb_full[:, :self.in_dim]
        self.map_aabb0 = a[0]
        self.map_size = f32(np.max((a[1] - a[0]).astype(f32)))
        # normalize_coord uses the model aabb: all dims in 'images' mode, else the in_dim dims
        self.coef_aabb = self.aabb_full if mode == "images" else a

    @classmethod
    def from_meta(cls, meta):
        m = meta["cfg"]["model"]
        return cls(meta["cfg"]["defaults"]["mode"], meta["cfg"]["dataset"]["aabb"], m["basis_dims"],
                   meta["basis_reso"], meta["freq_bands"], meta["coeff_reso"], m["basis_mapping"],
                   m.get("basis_mode", "bilinear"), m.get("coef_mode", "bilinear"))


def _basis_coords(spec, x):
    xb = np.asarray(x, f32)[:, :spec.in_dim]  # :469-470 drops the image index in 'images' mode
    return grid_mapping(xb, spec.freq_bands, spec.map_aabb0, spec.map_size, spec.mapping)  # [N, d, L]


def get_coeff(spec, coeff_grid, x):
    """models/FactorFields.py:425-434 — coefficient gather, align_corners=False, border."""
    pts = normalize_coord(x, spec.coef_aabb[0], spec.coef_aabb[1])
    return grid_sample_fwd(coeff_grid, pts, False, "border", spec.coef_mode)


def get_basis(spec, basis_grids, x):
    """models/FactorFields.py:467-490, 512-513 — per-level basis gathers, concatenated."""
    loc = _basis_coords(spec, x)
    outs = [grid_sample_fwd(basis_grids[l], loc[..., l], True, "zeros", spec.basis_mode)
            for l in range(len(basis_grids))]
    return np.concatenate(outs, 1)


def get_coding(spec, basis_grids, coeff_grid, x):
    """models/FactorFields.py:523-527 — returns (basis * coeff, coeff)."""
    coeff = get_coeff(spec, coeff_grid, x)
    basis = get_basis(spec, basis_grids, x)
    return basis * coeff, coeff


def get_coding_bwd(spec, basis_grids, coeff_grid, x, g_feats, g_coeff=None):
    """Gradients of sum(g_feats*feats + g_coeff*coeff) wrt every basis level and the coeff grid."""
    coeff = get_coeff(spec, coeff_grid, x)
    basis = get_basis(spec, basis_grids, x)
    g_feats = np.asarray(g_feats, f64)
    g_basis = g_feats * coeff
    g_c = g_feats * basis
    if g_coeff is not None:
        g_c = g_c + np.asarray(g_coeff, f64)
    loc = _basis_coords(spec, x)
    grads, off = [], 0
    for l, g in enumerate(basis_grids):
        c = g.shape[0]
        grads.append(grid_sample_bwd(g.shape, loc[..., l], g_basis[:, off:off + c], True, "zeros",
                                     spec.basis_mode))
        off += c
    pts = normalize_coord(x, spec.coef_aabb[0], spec.coef_aabb[1])
    gcoef = grid_sample_bwd(coeff_grid.shape, pts, g_c, False, "border", spec.coef_mode)
    return grads, gcoef


# ----------------------------------------------------------------------------------------
# MLP heads
# ----------------------------------------------------------------------------------------

def mlp_fwd(weights, biases, x):
    """models/FactorFields.py:113-159 (MLPMixer): Linear+ReLU ..., last layer without bias.

    weights[i]: [out, in]; biases[i] or None. Returns (out, list of pre-activations)."""
    h = np.asarray(x, f64)
    pre = []
    for i, w in enumerate(weights):
        h = h @ np.asarray(w, f64).T
        if biases[i] is not None:
            h = h + np.asarray(biases[i], f64)
        pre.append(h)
        if i != len(weights) - 1:
            h = np.maximum(h, 0)
    return h, pre


def mlp_bwd(weights, biases, x, g_out):
    """Backward of mlp_fwd: (grad_in, grad_weights, grad_biases)."""
    _, pre = mlp_fwd(weights, biases, x)
    acts = [np.asarray(x, f64)] + [np.maximum(p, 0) for p in pre[:-1]]
    g = np.asarray(g_out, f64)
    gw, gb = [None] * len(weights), [None] * len(weights)
    for i in reversed(range(len(weights))):
        if i != len(weights) - 1:
            g = g * (pre[i] > 0)
        gw[i] = g.T @ acts[i]
        gb[i] = g.sum(0) if biases[i] is not None else None
        g = g @ np.asarray(weights[i], f64)
    return g, gw, gb


def positional_encoding(x, freqs):
    """models/FactorFields.py:74-79: [sin(x_d 2^f)]_{d,f} ++ [cos(x_d 2^f)]_{d,f}, index d * F + f."""
    x = np.asarray(x, f64)
    fb = 2.0 ** np.arange(freqs)
    pts = (x[..., None] * fb).reshape(x.shape[:-1] + (freqs * x.shape[-1],))
    return np.concatenate([np.sin(pts), np.cos(pts)], -1)


def render_head_input(feat, dirs, view_pe, fea_pe):
    """MLPRender_Fea's input rows (models/FactorFields.py:188-195): [feat, dirs, PE(feat), PE(dirs)]."""
    parts = [np.asarray(feat, f64), np.asarray(dirs, f64)]
    if fea_pe > 0:
        parts.append(positional_encoding(feat, fea_pe))
    if view_pe > 0:
        parts.append(positional_encoding(dirs, view_pe))
    return np.concatenate(parts, -1)


def render_head_fwd(weights, biases, feat, dirs, view_pe, fea_pe):
    """MLPRender_Fea.forward (models/FactorFields.py:188-203): sigmoid(MLP(input)) [N, 3]."""
    out, _ = mlp_fwd(weights, biases, render_head_input(feat, dirs, view_pe, fea_pe))
    return sigmoid(out)


def render_head_bwd(weights, biases, feat, dirs, view_pe, fea_pe, g_rgb):
    """Backward of render_head_fwd for dL/drgb: (dL/dfeat [N, C], grad_weights, grad_biases)."""
    x = render_head_input(feat, dirs, view_pe, fea_pe)
    out, _ = mlp_fwd(weights, biases, x)
    rgb = sigmoid(out)
    g_out = np.asarray(g_rgb, f64) * rgb * (1 - rgb)
    g_x, gw, gb = mlp_bwd(weights, biases, x, g_out)
    feat = np.asarray(feat, f64)
    c = feat.shape[-1]
    g_feat = g_x[:, :c].copy()
    if fea_pe > 0:
        off = c + 3
        fb = 2.0 ** np.arange(fea_pe)
        arg = feat[..., None] * fb  # [N, C, F]
        g_sin = g_x[:, off:off + c * fea_pe].reshape(-1, c, fea_pe)
        g_cos = g_x[:, off + c * fea_pe:off + 2 * c * fea_pe].reshape(-1, c, fea_pe)
        g_feat += (fb * (g_sin * np.cos(arg) - g_cos * np.sin(arg))).sum(-1)
    return g_feat, gw, gb


# ----------------------------------------------------------------------------------------
# rendering: sampling, occupancy, density, compositing, SH colour
# ----------------------------------------------------------------------------------------

def step_size(aabb, grid_size, step_ratio):
    """models/FactorFields.py:693-699 — stepSize and default nSamples in float32."""
    aabb = np.asarray(aabb, f32)
    size = (aabb[1] - aabb[0]).astype(f32)
    units = (size / (np.asarray(grid_size, f32) - f32(1))).astype(f32)
    acc = f32(0)
    for u in units:
        acc = f32(acc + u)
    step = f32(f32(acc / f32(len(units))) * f32(step_ratio))
    diag = f32(np.sqrt(f32(np.sum((size * size).astype(f32), dtype=f32))))
    return step, int(f32(diag / step)) + 1


def sample_point(rays_o, rays_d, aabb, step, n_samples, jitter=None):
    """models/FactorFields.py:586-602 — uniform samples from the slab entry; float32 exact.

    jitter: [R, 1] per-ray uniform offset (training) or None. Returns (xyz [R,S,3], z [R,S],
    inside [R,S])."""
    o = np.asarray(rays_o, f32)
    d = np.asarray(rays_d, f32)
    aabb = np.asarray(aabb, f32)
    vec = np.where(d == 0, f32(1e-6), d).astype(f32)
    ra = ((aabb[1] - o).astype(f32) / vec).astype(f32)
    rb = ((aabb[0] - o).astype(f32) / vec).astype(f32)
    t_min = np.clip(np.max(np.minimum(ra, rb), -1), f32(0.05), f32(1e3)).astype(f32)
    rng = np.arange(n_samples, dtype=f32)[None]
    if jitter is not None:
        rng = (rng + np.asarray(jitter, f32).reshape(-1, 1)).astype(f32)
    z = (t_min[:, None] + (f32(step) * rng).astype(f32)).astype(f32)
    xyz = (o[:, None, :] + (d[:, None, :] * z[..., None]).astype(f32)).astype(f32)
    outside = ((aabb[0] > xyz) | (xyz > aabb[1])).any(-1)
    return xyz, z, ~outside


def occupancy_test(alpha_volume, aabb, xyz, thres=0.5):
    """models/FactorFields.py:103-110 + :866 — trilinear sample of a 0/1 volume > thres (0.5 in
    the ray march, 0 in filtering_rays :836)."""
    aabb = np.asarray(aabb, f32)
    # AlphaGridMask.invgridSize = 1.0 / aabbSize * 2 (two roundings)
    inv = ((f32(1.0) / (aabb[1] - aabb[0]).astype(f32)).astype(f32) * f32(2)).astype(f32)
    pts = (((np.asarray(xyz, f32) - aabb[0]).astype(f32) * inv).astype(f32) - f32(1)).astype(f32)
    vol = np.asarray(alpha_volume, f32)[None]
    val = np.zeros(pts.shape[0], f32)
    sizes = list(vol.shape[1:][::-1])
    flatv = vol.reshape(-1)
    # float32 accumulation in ATen's corner order (the test is a threshold on a float32 sum)
    for flat, w, valid in sample_corners(pts, sizes, True, "zeros", "bilinear"):
        val = (val + np.where(valid, (flatv[flat] * w).astype(f32), f32(0))).astype(f32)
    return val > f32(thres)


def occupancy_mask(alpha, threshold, min_size):
    """updateAlphaMask's volume steps (models/FactorFields.py:763-774): alpha [D, H, W] clamped to
    [0, 1], 3x3x3 max-pool (stride 1, padding 1), >= threshold, then remove_small_objects(...,
    min_size, connectivity=1). That last function is scikit-image's (requirements.txt:8, version
    unpinned; not installed here): it labels the True voxels into connected components with
    the connectivity-1 structure (6 neighbours in 3-D) and clears every component with fewer
    than min_size voxels. Restated here with scipy.ndimage.label, the labelling routine it
    wraps; parity with scikit-image itself is unpinned. Returns (keep [D, H, W] bool, bitfield
    words int32 [ceil(V / 32)], bbox (x_min, y_min, z_min, x_max, y_max, z_max) or None)."""
    from scipy import ndimage
    a = np.clip(np.asarray(alpha, f32), f32(0), f32(1))
    pooled = ndimage.maximum_filter(a, size=3, mode="constant", cval=-np.inf)
    occ = pooled >= f32(threshold)
    if min_size > 1:
        labels, _ = ndimage.label(occ, structure=ndimage.generate_binary_structure(3, 1))
        sizes = np.bincount(labels.reshape(-1))
        small = sizes < min_size
        small[0] = True  # background
        occ = ~small[labels]
    flat = occ.reshape(-1)
    pad = (-flat.size) % 32
    b = np.concatenate([flat, np.zeros(pad, bool)]).reshape(-1, 32).astype(np.uint64)
    words = (b << np.arange(32, dtype=np.uint64)).sum(1).astype(np.uint32).view(np.int32)
    if not flat.any():
        return occ, words, None
    z, y, x = np.nonzero(occ)
    return occ, words, (x.min(), y.min(), z.min(), x.max(), y.max(), z.max())


def softplus_shift(f, shift):
    """models/FactorFields.py:639-641 with torch.nn.functional.softplus (threshold 20)."""
    x = np.asarray(f, f64) + shift
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def softplus_grad(f, shift):
    x = np.asarray(f, f64) + shift
    return np.where(x > 20, 1.0, 1.0 / (1.0 + np.exp(-x)))


def raw2alpha(sigma, dist):
    """models/FactorFields.py:82-88 — alpha, weights and background transmittance (float64)."""
    alpha = 1.0 - np.exp(-np.asarray(sigma, f64) * np.asarray(dist, f64))
    fac = 1.0 - alpha + 1e-10
    t = np.cumprod(np.concatenate([np.ones_like(alpha[..., :1]), fac], -1), -1)
    return alpha, alpha * t[..., :-1], t[..., -1:]


SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792,
         0.5462742152960396)


def sh2_basis(dirs):
    """models/sh.py:49-64 — the 9 real SH basis values of degree <= 2, with signs."""
    d = np.asarray(dirs, f64)
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    xx, yy, zz, xy, yz, xz = x * x, y * y, z * z, x * y, y * z, x * z
    return np.stack([np.full_like(x, SH_C0), -SH_C1 * y, SH_C1 * z, -SH_C1 * x,
                     SH_C2[0] * xy, SH_C2[1] * yz, SH_C2[2] * (2.0 * zz - xx - yy),
                     SH_C2[3] * xz, SH_C2[4] * (xx - yy)], -1)


def eval_sh2(sh, dirs):
    """models/sh.py:34-64 — eval_sh(2, sh[..., 3, 9], dirs) -> [..., 3]."""
    return np.einsum("...ck,...k->...c", np.asarray(sh, f64), sh2_basis(dirs))


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


class RenderSpec:
    """Renderer constants (configs/nerf.yaml:73-92 keys)."""

    def __init__(self, aabb, step, n_samples, density_shift=-10.0, distance_scale=25.0,
                 weight_thres=1e-3, white_bg=True):
        self.aabb = np.asarray(aabb, f32)
        self.step = f32(step)
        self.n_samples = int(n_samples)
        self.density_shift = density_shift
        self.distance_scale = distance_scale
        self.weight_thres = weight_thres
        self.white_bg = white_bg


def render_rays(fspec, rspec, basis_grids, coeff_grid, mlp_w, mlp_b, rays, jitter=None,
                alpha_volume=None, g_rgb=None, head=None):
    """models/FactorFields.py:843-898 (bounded scene) forward, and — when g_rgb is given — the
    backward of sum(g_rgb * rgb). Colour head: the SH-2 head composed from models/sh.py:34
    (head=None), or MLPRender_Fea (:162-203) with head = dict(w=[...], b=[...], view_pe, fea_pe).

    Returns dict(rgb, depth, weight, valid, z, acc) and, with g_rgb, the parameter gradients
    grad_basis (list), grad_coeff, grad_mlp_w, grad_mlp_b (and grad_head_w, grad_head_b)."""
    rays = np.asarray(rays, f32)
    o, d = rays[:, :3], rays[:, 3:6]
    xyz, z, inside = sample_point(o, d, rspec.aabb, rspec.step, rspec.n_samples, jitter)
    r, s = z.shape
    dists = np.concatenate([(z[:, 1:] - z[:, :-1]).astype(f32), np.zeros((r, 1), f32)], 1)  # :861
    valid = inside.copy()
    if alpha_volume is not None:
        valid[inside] = occupancy_test(alpha_volume, rspec.aabb, xyz[inside])
    pts = xyz[valid]
    feats, coeff = get_coding(fspec, basis_grids, coeff_grid, pts)
    out, _ = mlp_fwd(mlp_w, mlp_b, feats)
    sigma = np.zeros((r, s), f64)
    sigma[valid] = softplus_shift(out[:, 0], rspec.density_shift)
    delta = dists.astype(f64) * rspec.distance_scale
    alpha, weight, _ = raw2alpha(sigma, delta)
    app = weight > rspec.weight_thres  # :879
    colour = np.zeros((r, s, 3), f64)
    dirs = np.broadcast_to(d[:, None, :], (r, s, 3))[valid]
    app_v = app[valid]
    if head is None:
        sh = out[:, 1:28].reshape(-1, 3, 9)
        lin = eval_sh2(sh, dirs)
        c_valid = sigmoid(lin)
    else:  # the head runs on feat[app_mask, 1:] only (:884)
        c_valid = np.zeros((pts.shape[0], 3), f64)
        if app_v.any():
            c_valid[app_v] = render_head_fwd(head["w"], head["b"], out[app_v, 1:], dirs[app_v],
                                             head["view_pe"], head["fea_pe"])
    tmp = np.zeros((pts.shape[0], 3), f64)
    tmp[app_v] = c_valid[app_v]
    colour[valid] = tmp
    acc = weight.sum(-1)
    rgb = (weight[..., None] * colour).sum(-2)
    if rspec.white_bg:
        rgb = rgb + (1.0 - acc[:, None])
    rgb_c = np.clip(rgb, 0, 1)
    depth = (weight * z.astype(f64)).sum(-1)
    res = dict(rgb=rgb_c, depth=depth, weight=weight, valid=valid, z=z, acc=acc)
    if g_rgb is None:
        return res
    # ---- backward of sum(g_rgb * rgb) ----
    g = np.asarray(g_rgb, f64) * ((rgb >= 0) & (rgb <= 1))  # clamp backward
    g_w = (g[:, None, :] * colour).sum(-1)
    if rspec.white_bg:
        g_w = g_w - g.sum(-1, keepdims=True)
    g_col = g[:, None, :] * weight[..., None]  # [R,S,3], only app samples matter
    fac = 1.0 - alpha + 1e-10
    t = np.cumprod(np.concatenate([np.ones((r, 1)), fac], -1), -1)[:, :-1]
    # dL/dalpha_i = T_i * (g_w_i - S_i),  S_i = sum_{j>i} g_w_j alpha_j prod_{i<k<j} fac_k
    s_acc = np.zeros(r)
    g_alpha = np.zeros((r, s))
    for i in reversed(range(s)):
        g_alpha[:, i] = t[:, i] * (g_w[:, i] - s_acc)
        s_acc = g_w[:, i] * alpha[:, i] + fac[:, i] * s_acc
    g_sigma = g_alpha * np.exp(-sigma * delta) * delta
    g_out = np.zeros_like(out)
    g_out[:, 0] = g_sigma[valid] * softplus_grad(out[:, 0], rspec.density_shift)
    gc = g_col[valid] * app_v[:, None]
    if head is None:
        g_lin = gc * c_valid * (1 - c_valid)
        basis9 = sh2_basis(dirs)
        g_out[:, 1:28] = (g_lin[:, :, None] * basis9[:, None, :]).reshape(-1, 27)
    else:
        hw = [np.zeros_like(np.asarray(w, f64)) for w in head["w"]]
        hb = [None if b is None else np.zeros_like(np.asarray(b, f64)) for b in head["b"]]
        if app_v.any():
            g_f, hw, hb = render_head_bwd(head["w"], head["b"], out[app_v, 1:], dirs[app_v], head["view_pe"],
                                          head["fea_pe"], gc[app_v])
            g_out[app_v, 1:] = g_f
        res.update(grad_head_w=hw, grad_head_b=hb)
    g_feats, gw, gb = mlp_bwd(mlp_w, mlp_b, feats, g_out)
    gbasis, gcoef = get_coding_bwd(fspec, basis_grids, coeff_grid, pts, g_feats)
    res.update(grad_basis=gbasis, grad_coeff=gcoef, grad_mlp_w=gw, grad_mlp_b=gb)
    return res


def composite_rows(rspec, feat, z, dist, offsets, dirs, rgb_rows=None, white_bg=None):
    """raw2alpha + colour + compositing (models/FactorFields.py:82-88, :876-896) over ragged rays
    of live samples, in float64: feat [M, >= 1] (channel 0 density feature, 1..27 the SH-2
    coefficients unless rgb_rows [M, 3] gives the colours), z / dist [M] (dist before
    distance_scale), offsets [R + 1], dirs [R, 3] ray directions. Returns the clamped rgb [R, 3]."""
    feat = np.asarray(feat, f64)
    offsets = np.asarray(offsets)
    wb = rspec.white_bg if white_bg is None else white_bg
    out = np.zeros((len(offsets) - 1, 3))
    for r in range(len(offsets) - 1):
        a, b = int(offsets[r]), int(offsets[r + 1])
        if b == a:
            rgb = np.zeros(3)
            acc = 0.0
        else:
            sigma = softplus_shift(feat[a:b, 0], rspec.density_shift)
            _, w, _ = raw2alpha(sigma[None], np.asarray(dist[a:b], f64)[None] * rspec.distance_scale)
            w = w[0]
            app = w > rspec.weight_thres
            if rgb_rows is None:
                sh = feat[a:b, 1:28].reshape(-1, 3, 9)
                col = sigmoid(eval_sh2(sh, np.broadcast_to(np.asarray(dirs[r], f64), (b - a, 3))))
            else:
                col = np.asarray(rgb_rows[a:b], f64)
            col = col * app[:, None]
            acc = w.sum()
            rgb = (w[:, None] * col).sum(0)
        if wb:
            rgb = rgb + (1.0 - acc)
        out[r] = np.clip(rgb, 0, 1)
    return out


# ----------------------------------------------------------------------------------------
# inverse-CDF resampling
# ----------------------------------------------------------------------------------------

def sample_pdf(bins, weights, u):
    """dataLoader/ray_utils.py:132-174 with the uniform numbers u given ([B, S]).

    The pdf/cdf and the interpolation run in float32 like the reference (searchsorted on the
    float32 cdf decides the bin, so it must see the same cdf values)."""
    w = (np.asarray(weights, f32) + f32(1e-5)).astype(f32)
    tot = np.zeros(w.shape[0], f32)
    for j in range(w.shape[1]):
        tot = (tot + w[:, j]).astype(f32)
    pdf = (w / tot[:, None]).astype(f32)
    cdf = np.zeros((w.shape[0], w.shape[1] + 1), f32)
    run = np.zeros(w.shape[0], f32)
    for j in range(w.shape[1]):
        run = (run + pdf[:, j]).astype(f32)
        cdf[:, j + 1] = run
    u = np.asarray(u, f32)
    inds = np.stack([np.searchsorted(cdf[b], u[b], side="right") for b in range(u.shape[0])])
    below = np.maximum(0, inds - 1)
    above = np.minimum(cdf.shape[-1] - 1, inds)
    cb = np.take_along_axis(cdf, below, 1)
    ca = np.take_along_axis(cdf, above, 1)
    bb = np.take_along_axis(np.asarray(bins, f32), below, 1)
    ba = np.take_along_axis(np.asarray(bins, f32), above, 1)
    denom = (ca - cb).astype(f32)
    denom = np.where(denom < f32(1e-5), f32(1), denom).astype(f32)
    t = ((u - cb).astype(f32) / denom).astype(f32)
    return (bb + (t * (ba - bb).astype(f32)).astype(f32)).astype(f32)


# ----------------------------------------------------------------------------------------
# proposal sampler (no reference implementation; resampling = sample_pdf above)
# ----------------------------------------------------------------------------------------

def proposal_segments(rays, aabb):
    """Per ray: the segment inside the aabb, t_in clamped to >= 0.05 (as sample_point :591)."""
    rays = np.asarray(rays, f64)
    aabb = np.asarray(aabb, f64)
    o, d = rays[:, :3], rays[:, 3:6]
    vec = np.where(d == 0, 1e-6, d)
    ra, rb = (aabb[1] - o) / vec, (aabb[0] - o) / vec
    t_in = np.maximum(np.minimum(ra, rb).max(-1), 0.05)
    t_out = np.maximum(np.maximum(ra, rb).min(-1), t_in)
    return t_in, t_out


def proposal_weights(o, seg_len, shift, distance_scale):
    """Proposal compositing weights of [R, nb] MLP outputs: softplus(o + shift) densities,
    alpha = 1 - exp(-sigma * len * scale), exclusive transmittance (raw2alpha :82-88)."""
    x = np.asarray(o, f64) + shift
    sigma = np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))
    delta = np.asarray(seg_len, f64)[:, None] * distance_scale
    alpha, w, _ = raw2alpha(sigma, np.broadcast_to(delta, sigma.shape))
    return w


def proposal_loss(o, seg_len, shift, distance_scale, w_field, bin_of, loss_scale, eps=1e-5):
    """sum over rays and bins of max(0, m_k - w_k)^2 / (w_k + eps) * loss_scale, with m_k the
    field weight mass in bin k; returns (loss, dL/do) — the gradient by central finite
    differences in float64 (a restatement independent of the kernels' reverse scan)."""
    o = np.asarray(o, f64)
    nb = o.shape[1]
    mass = np.zeros_like(o)
    for r in range(o.shape[0]):
        np.add.at(mass[r], np.asarray(bin_of[r]), np.asarray(w_field[r], f64))

    def loss_of(oo):
        w = proposal_weights(oo, seg_len, shift, distance_scale)
        rr = np.maximum(mass - w, 0)
        return (rr * rr / (w + eps)).sum(-1) * loss_scale  # per ray

    base = loss_of(o)
    grad = np.zeros_like(o)
    h = 1e-4
    for k in range(nb):
        op, om = o.copy(), o.copy()
        op[:, k] += h
        om[:, k] -= h
        grad[:, k] = (loss_of(op) - loss_of(om)) / (2 * h)
    return base.sum(), grad


def image_metrics(img0, img1, max_val=1.0):
    """utils.py:110-156 (rgb_ssim) and renderer.py:64 (the MSE behind PSNR) on [H, W, C] float32
    images: (mse, ssim). The squared and product images are float32 like the reference's tensor
    ops; the blurs run in float64 through scipy.signal.convolve2d as the reference's do."""
    from scipy import signal
    a = np.asarray(img0, f32)
    b = np.asarray(img1, f32)
    mse = float(np.mean((a.astype(f64) - b.astype(f64)) ** 2))
    fs, sigma = 11, 1.5
    hw = fs // 2
    shift = (2 * hw - fs + 1) / 2
    filt = np.exp(-0.5 * ((np.arange(fs) - hw + shift) / sigma) ** 2)
    filt /= np.sum(filt)

    def blur(z):
        return np.stack([signal.convolve2d(signal.convolve2d(z[..., i], filt[:, None], mode="valid"),
                                           filt[None, :], mode="valid") for i in range(z.shape[-1])], -1)
    mu0, mu1 = blur(a), blur(b)
    mu00, mu11, mu01 = mu0 * mu0, mu1 * mu1, mu0 * mu1
    s00 = np.maximum(0.0, blur((a * a).astype(f32)) - mu00)
    s11 = np.maximum(0.0, blur((b * b).astype(f32)) - mu11)
    s01 = blur((a * b).astype(f32)) - mu01
    s01 = np.sign(s01) * np.minimum(np.sqrt(s00 * s11), np.abs(s01))
    c1, c2 = (0.01 * max_val) ** 2, (0.03 * max_val) ** 2
    ssim = np.mean(((2 * mu01 + c1) * (2 * s01 + c2)) / ((mu00 + mu11 + c1) * (s00 + s11 + c2)))
    return mse, float(ssim)
