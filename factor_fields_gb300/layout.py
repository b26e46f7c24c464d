"""Channels-last HBM layout of the basis and coefficient grids, and converters to and from the
reference's channels-first tensors ([1, C, R, R(, R)] per level, [1, C, (D,) H, W] coefficients).

Basis: all levels in ONE flat buffer. Level l is [R_l]^d cells x stride_l channels (stride_l =
C_l for C_l in {1, 2, 4}, else C_l rounded up to a multiple of 4), starting at an element
offset that is a multiple of 8. Coefficients: per scene [(D,) H, W] cells x coeff_stride
channels with coeff_stride = n_feat rounded up to a multiple of 8 (16-byte cells in BF16).
Padding channels are zero and never written by the kernels. The float32 gradient buffers use
the same element layout, for both float32 and BF16 parameter storage.
"""
import torch

from . import _native as N


def _round_up(v, m):
    return (v + m - 1) // m * m


def _vec_for(*vals):
    for v in (4, 2):
        if all(x % v == 0 for x in vals):
            return v
    return 1


class FieldLayout:
    def __init__(self, basis_dims, basis_reso, basis_dim, coeff_reso, n_scene=1):
        self.basis_dims = list(basis_dims)
        self.basis_reso = list(basis_reso)
        self.basis_dim = basis_dim
        self.coeff_reso = list(coeff_reso)  # reference order: (D,) H, W
        self.n_scene = n_scene
        self.n_feat = sum(self.basis_dims)
        self.coeff_stride = _round_up(self.n_feat, 8)
        self.level_stride, self.level_offset, self.level_vec = [], [], []
        off, foff = 0, 0
        for c, r in zip(self.basis_dims, self.basis_reso):
            stride = c if c in (1, 2, 4) else _round_up(c, 4)
            self.level_stride.append(stride)
            self.level_offset.append(off)
            self.level_vec.append(_vec_for(c, stride, off, foff, self.coeff_stride))
            off = _round_up(off + r ** basis_dim * stride, 8)
            foff += c
        self.basis_numel = off
        self.coeff_cells = 1
        for r in self.coeff_reso:
            self.coeff_cells *= r
        self.coeff_scene_numel = self.coeff_cells * self.coeff_stride
        self.coeff_numel = self.coeff_scene_numel * n_scene

    # ---- views in the reference's layout ------------------------------------------------
    def basis_view(self, flat, l):
        """Level l of a flat basis buffer as the reference's [1, C, R, R(, R)] (a strided view)."""
        c, r, s, o = self.basis_dims[l], self.basis_reso[l], self.level_stride[l], self.level_offset[l]
        cells = [r] * self.basis_dim
        v = flat[o:o + r ** self.basis_dim * s].view(*cells, s)[..., :c]
        perm = [self.basis_dim] + list(range(self.basis_dim))
        return v.permute(*perm).unsqueeze(0)

    def coeff_view(self, flat, scene=0):
        """Coefficients of one scene as the reference's [1, C, (D,) H, W] (a strided view)."""
        n = self.coeff_scene_numel
        nd = len(self.coeff_reso)
        v = flat[scene * n:(scene + 1) * n].view(*self.coeff_reso, self.coeff_stride)[..., :self.n_feat]
        return v.permute(nd, *range(nd)).unsqueeze(0)

    def basis_from_reference(self, levels, device=None, dtype=torch.float32):
        flat = torch.zeros(self.basis_numel, dtype=dtype, device=device)
        for l, g in enumerate(levels):
            self.basis_view(flat, l).copy_(g.reshape(self.basis_view(flat, l).shape))
        return flat

    def coeff_from_reference(self, grids, device=None, dtype=torch.float32):
        flat = torch.zeros(self.coeff_numel, dtype=dtype, device=device)
        for s, g in enumerate(grids):
            self.coeff_view(flat, s).copy_(g.reshape(self.coeff_view(flat, s).shape))
        return flat

    # ---- native descriptor ---------------------------------------------------------------
    def descriptor(self, geom, mapping, basis_mode, coef_mode, param_dtype):
        """FFField for the geometry (FieldGeometry) with the given storage dtype."""
        f = N.FFField()
        f.basis_dim = self.basis_dim
        f.coord_dim = geom.coord_dim
        f.n_levels = len(self.basis_dims)
        if f.n_levels > N.FF_MAX_LEVELS:
            raise NotImplementedError(f"at most {N.FF_MAX_LEVELS} basis levels are supported")
        if mapping not in N.FF_MAP:
            raise NotImplementedError(f"basis_mapping {mapping!r} is not implemented (sawtooth, triangle)")
        f.mapping = N.FF_MAP[mapping]
        f.basis_interp = N.FF_INTERP[basis_mode]
        f.coeff_interp = N.FF_INTERP[coef_mode]
        f.param_dtype = param_dtype
        f.n_feat = self.n_feat
        aabb = geom.aabb
        map_aabb = aabb[:, :self.basis_dim]
        size = torch.max(map_aabb[1] - map_aabb[0])  # max(aabb[1] - aabb[0]) (:12)
        scale = size[..., None] / geom.freq_bands.to(torch.float32)  # (:13), float32
        for l in range(f.n_levels):
            f.level_channels[l] = self.basis_dims[l]
            f.level_stride[l] = self.level_stride[l]
            f.level_vec[l] = self.level_vec[l]
            f.level_reso[l] = self.basis_reso[l]
            f.level_offset[l] = self.level_offset[l]
            f.level_scale[l] = float(scale[l])
            f.level_inv_scale[l] = 1.0 / float(scale[l])
            f.level_inv_half[l] = 2.0 / float(scale[l])
        for k in range(self.basis_dim):
            f.map_origin[k] = float(map_aabb[0, k])
        inv = 2.0 / (aabb[1] - aabb[0])  # normalize_coord (:636), float32
        nd = geom.coord_dim
        reso_xyz = self.coeff_reso[::-1]
        for k in range(nd):
            f.coeff_reso[k] = reso_xyz[k]
            f.coeff_origin[k] = float(aabb[0, k])
            f.coeff_inv_size[k] = float(inv[k])
        f.coeff_stride = self.coeff_stride
        return f
