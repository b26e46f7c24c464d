"""FactorFields: the reference's model surface (models/FactorFields.py:206) on the native kernels.

The module keeps the reference's constructor, attributes (basis_dims, basis_reso, freq_bands,
coeff_reso, aabb, in_dim, basises, coeffs, linear_mat, renderModule, alphaMask, stepSize,
nSamples, scene_idx) and methods (get_coding, get_basis, get_coeff, linear_mat(feats,
is_train), forward(rays...), get_optparam_groups, n_parameters, save/load), for
basis_type = coeff_type = 'grid'.

Storage differs from the reference: the grids are channels-last flat float32 parameters
(basis_flat, coeff_flat; see layout.py). `basises[l]` / `coeffs[s]` return strided views of
that storage in the reference's [1, C, R, R(, R)] shape, so reading, in-place writes and
autograd through them work as in the reference.

precision='fp32' is the drop-in path (float32 storage and math, parity 1e-5 with the
reference). precision='bf16' reads BF16 copies of the grids (refreshed automatically after
the float32 master parameters change) with float32 accumulation and float32 gradients.
"""
import ctypes
import math

import numpy as np
import torch
import torch.nn.functional as F

from . import _native as N
from . import functional as FN
from .config import FieldGeometry, make_cfg, n_to_reso, render_step
from .layout import FieldLayout


def dct_dict(n_atoms_fre, size, n_select, dim=2):
    """DCT dictionary used to initialise each basis level (models/FactorFields.py:36-71):
    cosine atoms cos(pi*k*i/p) with the mean removed (k > 0), their Kronecker product over the
    dims, n_select evenly spaced atoms, each normalised to unit L2 norm."""
    p = n_atoms_fre
    rows = []
    for k in range(p):
        atom = np.cos(np.arange(size) * k * math.pi / p)
        rows.append(atom - np.mean(atom) if k > 0 else atom)
    table = np.stack(rows)
    kron = np.kron(table, table)
    if dim == 3:
        kron = np.kron(kron, table)
    if n_select < kron.shape[0]:
        pick = [chunk[0] for chunk in np.array_split(np.arange(kron.shape[0]), n_select)]
        kron = kron[pick]
    for r in range(kron.shape[0]):  # row by row, as the reference does, for a bit-identical init
        kron[r] /= np.linalg.norm(kron[r]) or 1
    return torch.from_numpy(kron.astype(np.float32))


class MLPMixer(torch.nn.Module):
    """models/FactorFields.py:113-159: Linear(+bias)+ReLU per hidden layer, last layer without
    bias and activation. Same parameter names (backbone.i.weight/bias) and init as the
    reference; the math runs on the native float32 kernels."""

    def __init__(self, in_dim, out_dim=16, num_layers=2, hidden_dim=64, pe=0, with_dropout=False):
        super().__init__()
        if pe:
            raise NotImplementedError("positional encoding inside MLPMixer is not on the grid/grid path")
        self.with_dropout = with_dropout
        self.in_dim, self.out_dim = in_dim, out_dim
        self.num_layers, self.hidden_dim, self.pe = num_layers, hidden_dim, pe
        layers = []
        for l in range(num_layers):
            din = in_dim if l == 0 else hidden_dim
            last = l == num_layers - 1
            layers.append(torch.nn.Linear(din, out_dim if last else hidden_dim, bias=not last))
        self.backbone = torch.nn.ModuleList(layers)

    def weights(self):
        return [l.weight for l in self.backbone], [l.bias for l in self.backbone]

    def forward(self, x, is_train=False):
        h = x
        if self.with_dropout and is_train:
            h = F.dropout(h, p=0.1)
        w, b = self.weights()
        return FN.mlp(h, w, b, self.in_dim, self.hidden_dim, self.out_dim)


class FactorFields(torch.nn.Module):
    def __init__(self, cfg, device="cuda", precision="fp32"):
        super().__init__()
        cfg = make_cfg(cfg)
        if precision not in ("fp32", "bf16"):
            raise ValueError("precision must be 'fp32' or 'bf16'")
        self.cfg, self.device, self.precision = cfg, torch.device(device), precision
        self.matMode, self.vecMode = [[0, 1], [0, 2], [1, 2]], [2, 1, 0]
        self.n_scene, self.scene_idx = 1, 0
        self.alphaMask = None
        self.coeff_type, self.basis_type = cfg.model.coeff_type, cfg.model.basis_type
        self._setup(cfg)
        self.linear_mat = MLPMixer(self.n_feat, cfg.model.out_dim, num_layers=cfg.model.num_layers,
                                   hidden_dim=cfg.model.hidden_dim,
                                   with_dropout=bool(cfg.model.with_dropout)).to(self.device)
        if "reconstruction" in cfg.defaults.mode:
            from .renderer import make_render_module
            self.renderModule = make_render_module(cfg, cfg.model.out_dim - 1).to(self.device)
            self.is_unbound = bool(cfg.dataset.is_unbound)
            if self.is_unbound:
                raise NotImplementedError("unbounded scenes (sample_point_unbound) are not on this path")
            self.inward_aabb = self.aabb
            self.cur_volumeSize = n_to_reso(cfg.training.volume_resoInit ** self.in_dim, self.aabb.cpu())
            self.update_renderParams(self.cur_volumeSize)

    # ---- construction -----------------------------------------------------------------
    def _setup(self, cfg):
        g = FieldGeometry(cfg)
        self.geom = g
        self.in_dim = g.in_dim
        self.aabb = g.aabb.to(self.device)
        self.basis_dims, self.basis_reso = g.basis_dims, g.basis_reso
        self.T_basis, self.T_coeff = g.T_basis, g.T_coeff
        self.coeff_reso = g.coeff_reso
        self.n_scene = g.n_scene
        self.n_feat = g.n_feat
        self._freq_bands = g.freq_bands.to(self.device)
        self._freq_host = tuple(float(v) for v in g.freq_bands)  # host copy: no device sync per call
        self.layout = FieldLayout(g.basis_dims, g.basis_reso, g.in_dim, g.coeff_reso, g.n_scene)
        levels = [dct_dict(int(np.power(c, 1.0 / self.in_dim) + 1), r, n_select=c, dim=self.in_dim)
                  .reshape([1, c] + [r] * self.in_dim) for c, r in zip(g.basis_dims, g.basis_reso)]
        self.basis_flat = torch.nn.Parameter(self.layout.basis_from_reference(levels, device=self.device))
        coef = torch.zeros(self.layout.coeff_numel, device=self.device)
        for s in range(self.n_scene):
            self.layout.coeff_view(coef, s).fill_(float(cfg.model.coef_init))
        self.coeff_flat = torch.nn.Parameter(coef)
        self._desc_cache = {}
        self._bf16 = None

    @property
    def freq_bands(self):
        return self._freq_bands

    @freq_bands.setter
    def freq_bands(self, v):
        t = torch.as_tensor(v, dtype=torch.float32)
        self._freq_host = tuple(float(x) for x in t.cpu())
        self._freq_bands = t.to(self.device)
        self._desc_cache = {}

    @property
    def basises(self):
        """Each basis level as the reference's [1, C, R, R(, R)] tensor (a view of basis_flat)."""
        return [self.layout.basis_view(self.basis_flat, l) for l in range(len(self.basis_dims))]

    @property
    def coeffs(self):
        """Each scene's coefficient grid as the reference's [1, C, (D,) H, W] (a view)."""
        return [self.layout.coeff_view(self.coeff_flat, s) for s in range(self.n_scene)]

    def descriptor(self, dtype):
        key = (dtype, self._freq_host)
        d = self._desc_cache.get(key)
        if d is None:
            self.geom.freq_bands = torch.tensor(self._freq_host, dtype=torch.float32)
            d = self.layout.descriptor(self.geom, self.cfg.model.basis_mapping, self.cfg.model.basis_mode,
                                       self.cfg.model.coef_mode, dtype)
            self._desc_cache[key] = d
        return d

    def _read_buffers(self):
        """(basis, coeff, dtype code) the kernels read: float32 params or their BF16 copies."""
        if self.precision == "fp32":
            return self.basis_flat, self.coeff_flat, N.FF_F32
        # The BF16 copies are refreshed IN PLACE whenever the float32 masters changed (their
        # version counters move on every in-place update, e.g. an optimizer step), so captured
        # CUDA graphs that read them stay valid.
        if (self._bf16 is None or self._bf16[1].numel() != self.basis_flat.numel()
                or self._bf16[2].numel() != self.coeff_flat.numel()):
            self._bf16 = [None, torch.empty_like(self.basis_flat, dtype=torch.bfloat16),
                          torch.empty_like(self.coeff_flat, dtype=torch.bfloat16)]
        ver = (self.basis_flat._version, self.coeff_flat._version, self.basis_flat.data_ptr(),
               self.coeff_flat.data_ptr())
        if self._bf16[0] != ver:
            with torch.no_grad():
                self._bf16[1].copy_(self.basis_flat.detach())
                self._bf16[2].copy_(self.coeff_flat.detach())
            self._bf16[0] = ver
        return self._bf16[1], self._bf16[2], N.FF_BF16

    def bf16_shadows(self):
        """{parameter: its BF16 read copy} for an optimizer that refreshes the copies itself
        (FusedAdam); empty for precision='fp32'."""
        if self.precision != "bf16":
            return {}
        self._read_buffers()
        return {self.basis_flat: self._bf16[1], self.coeff_flat: self._bf16[2]}

    def _coeff_scene(self, buf):
        n = self.layout.coeff_scene_numel
        return buf[self.scene_idx * n:(self.scene_idx + 1) * n]

    def _field(self, x, want):
        basis_r, coeff_r, dt = self._read_buffers()
        desc = self.descriptor(dt)
        coeff_param = self.coeff_flat
        if self.n_scene > 1:
            coeff_param = self._coeff_scene(self.coeff_flat)
            coeff_r = self._coeff_scene(coeff_r)
        return FN.FieldCoding.apply(x, self.basis_flat, coeff_param, basis_r, coeff_r, desc, want)

    # ---- reference methods --------------------------------------------------------------
    def get_coding(self, x):
        """models/FactorFields.py:523-527: (basis * coeff, coeff)."""
        feats, coeff, _ = self._field(x, (True, True, False))
        return feats, coeff

    def get_basis(self, x):
        """models/FactorFields.py:467-513 (grid basis)."""
        return self._field(x, (False, False, True))[2]

    def get_coeff(self, x):
        """models/FactorFields.py:425-434 (grid coefficients)."""
        return self._field(x, (False, True, False))[1]

    def field_mlp(self, x):
        """linear_mat(get_coding(x)[0]) through the fused kernel (one launch forward, one
        backward): BF16 tensor-core MLP with FP32 accumulation, grids read at self.precision."""
        basis_r, coeff_r, dt = self._read_buffers()
        desc = self.descriptor(dt)
        coeff_param = self.coeff_flat
        if self.n_scene > 1:
            coeff_param = self._coeff_scene(self.coeff_flat)
            coeff_r = self._coeff_scene(coeff_r)
        lm = self.linear_mat
        if lm.num_layers != 2:
            raise NotImplementedError("the fused path needs an MLPMixer with num_layers=2")
        l0, l1 = lm.backbone
        return FN.FusedFieldMLP.apply(x, self.basis_flat, coeff_param, l0.weight, l0.bias, l1.weight, basis_r,
                                      coeff_r, desc, (lm.in_dim, lm.hidden_dim, lm.out_dim))

    def n_parameters(self):
        """Logical parameter count (models/FactorFields.py:535-539), padding excluded."""
        basis = sum(c * r ** self.in_dim for c, r in zip(self.basis_dims, self.basis_reso))
        coeff = self.n_feat * self.layout.coeff_cells * self.n_scene
        rest = sum(p.numel() for n, p in self.named_parameters() if n not in ("basis_flat", "coeff_flat"))
        return basis + coeff + rest

    def get_optparam_groups(self, lr_small=0.001, lr_large=0.02):
        """models/FactorFields.py:541-554."""
        t = self.cfg.training or {}
        groups = []
        if t.get("linear_mat", True):
            groups.append({"params": self.linear_mat.parameters(), "lr": lr_small})
        if t.get("coeff", True):
            groups.append({"params": [self.coeff_flat], "lr": lr_large})
        if t.get("basis", True):
            groups.append({"params": [self.basis_flat], "lr": lr_large})
        if "reconstruction" in self.cfg.defaults.mode and t.get("renderModule", True):
            groups.append({"params": self.renderModule.parameters(), "lr": lr_small})
        return groups

    def set_optimizable(self, items, statue):
        """models/FactorFields.py:556-567, with the reference's effects kept as they are:
        'basis' and 'coeff' both switch requires_grad of the basis grids (the reference's
        'coeff' branch loops over self.basises), 'proj' and 'renderer' set a plain
        `requires_grad` attribute on linear_mat / renderModule (which leaves their parameters
        as they were)."""
        for item in items:
            if item in ("basis", "coeff"):
                self.basis_flat.requires_grad_(statue)
            elif item == "proj":
                self.linear_mat.requires_grad = statue
            elif item == "renderer":
                self.renderModule.requires_grad = statue

    def TV_loss(self, reg):
        """models/FactorFields.py:569-573: sum over the basis levels of reg(level) * 1e-2, the
        levels passed as the reference's [1, C, R..] tensors (views of basis_flat, so the
        gradient reaches it)."""
        total = 0
        for level in self.basises:
            total = total + reg(level) * 1e-2
        return total

    @torch.no_grad()
    def normalize_basis(self):
        """models/FactorFields.py:519-521: each level divided by its norm over dims (2, 3) of
        the [1, C, R, R(, R)] tensor, in place."""
        for level in self.basises:
            level.copy_(level / torch.norm(level, dim=(2, 3), keepdim=True))

    @torch.no_grad()
    def upsample_volume_grid(self, res_target):
        """models/FactorFields.py:701-707: new render parameters for res_target; for the
        google_objs dataset with one scene, the coefficient grid is also resampled by 1.3
        (trilinear, align_corners=True) and rebuilt at its new resolution, as a new
        parameter: build a new optimizer afterwards, as the reference's training loop does
        (train_per_scene.py:214-218)."""
        self.update_renderParams(res_target)
        if self.cfg.dataset.dataset_name == "google_objs" and self.n_scene == 1 and self.coeff_type == "grid":
            grid = F.interpolate(self.coeffs[0].detach().contiguous(), size=None, scale_factor=1.3,
                                 align_corners=True, mode="trilinear")
            self.coeff_reso = list(grid.shape[2:])
            self.geom.coeff_reso = self.coeff_reso
            self.layout = FieldLayout(self.basis_dims, self.basis_reso, self.in_dim, self.coeff_reso, self.n_scene)
            self.coeff_flat = torch.nn.Parameter(self.layout.coeff_from_reference([grid], device=self.device))
            self.T_coeff = self.n_feat * int(np.prod(self.coeff_reso))
            self._desc_cache = {}
            self._bf16 = None

    @torch.no_grad()
    def cal_mean_coef(self, state_dict):
        """models/FactorFields.py:645-667 for grid coefficients: the scenes' coefficient grids
        averaged into coeffs.0 (the others dropped)."""
        keys = [k for k in state_dict.keys() if "coeffs.0" in k]
        for key in keys:
            average = torch.zeros_like(state_dict[key])
            for i in range(self.n_scene):
                item = key.replace("0", f"{i}", 1)
                average += state_dict[item]
                state_dict.pop(item, None)
            state_dict[key] = average / self.n_scene
        return state_dict

    def normalize_coord(self, xyz):
        """models/FactorFields.py:635-637."""
        inv = 2.0 / (self.aabb[1] - self.aabb[0])
        return (xyz - self.aabb[0]) * inv - 1

    def basis2density(self, density_features):
        """models/FactorFields.py:639-643."""
        if self.cfg.renderer.fea2denseAct == "softplus":
            return F.softplus(density_features + self.cfg.renderer.density_shift)
        return F.relu(density_features + self.cfg.renderer.density_shift)

    def update_renderParams(self, gridSize):
        """models/FactorFields.py:693-699."""
        aabb = self.aabb.cpu()
        self.aabbSize = (aabb[1] - aabb[0]).to(self.device)
        self.gridSize = torch.tensor(gridSize, dtype=torch.long, device=self.device)
        step, n = render_step(aabb, gridSize, self.cfg.renderer.step_ratio)
        self.stepSize = step.to(self.device)
        self.nSamples = n
        # host copies for the render descriptor (valid while self.aabb is this tensor, unmodified)
        self._render_host = (self.aabb, self.aabb._version, aabb, float(step))

    def forward(self, rays_chunk, white_bg=True, is_train=False, ndc_ray=False, N_samples=-1, jitter=None,
                fused=None, static=False):
        """models/FactorFields.py:843-898 (bounded scenes): (rgb_map, depth_map, coeffs).
        fused=None picks the fused BF16 field kernel when precision == 'bf16'; static=True renders
        without host synchronisation (CUDA-graph capturable; fused path, SH-2 head)."""
        from .renderer import render_forward
        return render_forward(self, rays_chunk, white_bg=white_bg, is_train=is_train, ndc_ray=ndc_ray,
                              N_samples=N_samples, jitter=jitter, fused=fused, static=static)

    # ---- occupancy maintenance (models/FactorFields.py:710-793) ----------------------------
    @torch.no_grad()
    def density(self, xyz, chunk=1 << 20):
        """basis2density(linear_mat(get_coding(xyz))[:, 0]) (:639-643, :721-723), chunked."""
        out = torch.empty(xyz.shape[0], device=xyz.device)
        for s in range(0, xyz.shape[0], chunk):
            x = xyz[s:s + chunk].contiguous()
            if self.precision == "bf16":
                f0 = self.field_mlp(x)[:, 0]
            else:
                f0 = self.linear_mat(self.get_coding(x)[0])[:, 0]
            out[s:s + chunk] = self.basis2density(f0)
        return out

    @torch.no_grad()
    def compute_alpha(self, xyz_locs, length=1):
        """:710-727: alpha = 1 - exp(-sigma * length), zero where the current mask is empty."""
        sigma = torch.zeros(xyz_locs.shape[0], device=xyz_locs.device)
        if self.alphaMask is not None:
            keep = self.alphaMask.sample_alpha(xyz_locs) > 0
        else:
            keep = torch.ones_like(sigma, dtype=torch.bool)
        if keep.any():
            sigma[keep] = self.density(xyz_locs[keep])
        return 1 - torch.exp(-sigma * length)

    @torch.no_grad()
    def getDenseAlpha(self, gridSize=None, times=16, seed=None):
        """:729-755: alpha on the voxel centres of an (X, Y, Z) grid over inward_aabb, averaged
        over `times` passes jittered by up to 0.6 voxel; returns (alpha [Z, Y, X], xyz [Z, Y, X, 3])."""
        grid = self.gridSize.tolist() if gridSize is None else list(gridSize)
        a0, a1 = self.inward_aabb[0], self.inward_aabb[1]
        units = (a1 - a0) / (torch.tensor(grid, device=self.device) - 1)
        half = 1.0 / (torch.tensor(grid, dtype=torch.float32) - 1) * 0.5
        step = torch.mean(units)
        axes = [torch.linspace(float(half[k]), float(1 - half[k]), grid[k]) for k in range(3)]
        samples = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).to(self.device)
        dense_xyz = (a0 * (1 - samples) + a1 * samples).transpose(0, 2).contiguous()
        gen = torch.Generator(device=self.device)
        if seed is not None:
            gen.manual_seed(seed)
        alpha = torch.zeros(dense_xyz.shape[:-1], device=self.device)
        length = float(step) * float(self.cfg.renderer.distance_scale)
        flat = dense_xyz.view(-1, 3)
        for _ in range(times):
            shift = 0.0
            if times > 1:
                shift = (torch.rand(flat.shape, device=self.device, generator=gen) * 2 - 1) * (units / 2 * 1.2)
            alpha += self.compute_alpha(flat + shift, length).view(alpha.shape)
        return alpha / times, dense_xyz

    @torch.no_grad()
    def updateAlphaMask(self, gridSize=(200, 200, 200), is_update_alphaMask=False, times=16, seed=None):
        """:757-793: dense alpha -> ff_occupancy_mask (clamp, 3x3x3 max-pool, threshold, removal
        of 6-connected components smaller than the mean grid dimension like the reference's
        remove_small_objects, bit packing, bounding box) -> AlphaGridMask, and the padded
        bounding box of the occupied voxels as the new aabb."""
        from .renderer import AlphaGridMask
        alpha, dense_xyz = self.getDenseAlpha(gridSize, times=times, seed=seed)
        d, h, w = alpha.shape
        thres = float(self.cfg.renderer.alphaMask_thres) if is_update_alphaMask else 0.08
        min_size = int(math.ceil(float(np.mean(alpha.shape))))  # remove_small_objects keeps size >= min_size
        need = int(N.lib().ff_occupancy_workspace_bytes(d, h, w))
        N.check(0 if need >= 0 else need, "ff_occupancy_workspace_bytes")
        ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        bits = torch.empty((alpha.numel() + 31) // 32, dtype=torch.int32, device=self.device)
        vol = torch.empty(alpha.shape, dtype=torch.float32, device=self.device)
        bbox = torch.empty(6, dtype=torch.int32, device=self.device)
        alpha = alpha.contiguous()
        N.call("ff_occupancy_mask", N.ptr(alpha), d, h, w, thres, min_size, N.ptr(bits), N.ptr(vol), N.ptr(bbox),
               N.ptr(ws), need, N.stream_ptr(), kernels=5 if min_size > 1 else 3)
        x0, y0, z0, x1, y1, z1 = bbox.tolist()
        if x0 > x1:
            # nothing occupied yet (an untrained field): keep the current mask - an empty mask
            # would leave no live samples and so no gradients (the reference fails here on amin)
            return self.aabb.clone()
        if is_update_alphaMask:
            self.alphaMask = AlphaGridMask(self.device, self.inward_aabb, vol, bits=bits)
        lo = torch.stack((dense_xyz[0, 0, x0, 0], dense_xyz[0, y0, 0, 1], dense_xyz[z0, 0, 0, 2]))
        hi = torch.stack((dense_xyz[0, 0, x1, 0], dense_xyz[0, y1, 0, 1], dense_xyz[z1, 0, 0, 2]))
        pad = (hi - lo) / 20
        return torch.stack((lo - pad, hi + pad))

    @torch.no_grad()
    def shrink(self, new_aabb):
        """:795-809: the field is rebuilt for the new box (setup_params: coefficient / basis
        resolutions follow the box) and re-initialised; aabb and inward_aabb become new_aabb and
        the render parameters are recomputed. The parameters are new tensors: build a new
        optimizer afterwards, as the reference's training loop does."""
        new_aabb = torch.as_tensor(new_aabb, dtype=torch.float32)
        self.cfg.dataset.aabb = new_aabb.tolist()
        self._setup(self.cfg)
        self.aabb = self.inward_aabb = new_aabb.to(self.device)
        self.update_renderParams(self.gridSize.tolist())

    @torch.no_grad()
    def filtering_rays(self, all_rays, all_rgbs, N_samples=256, chunk=10240 * 5, bbox_only=False):
        """:825-841: the rays (and their colours) that meet the box (bbox_only) or have some of
        their N_samples un-jittered samples on an occupied voxel (ff_filter_rays), in their
        original order. Works chunk by chunk on the GPU; returns tensors on all_rays' device."""
        from .renderer import render_desc
        if not bbox_only and self.alphaMask is None:
            raise ValueError("filtering_rays needs an alpha mask (updateAlphaMask) unless bbox_only=True")
        rays = all_rays.reshape(-1, all_rays.shape[-1])
        rgbs = all_rgbs.reshape(-1, all_rgbs.shape[-1])
        desc = render_desc(self, N_samples, True)
        keep = []
        for s in range(0, rays.shape[0], chunk):
            r = rays[s:s + chunk].to(self.device, torch.float32).contiguous()
            k = torch.empty(r.shape[0], dtype=torch.uint8, device=self.device)
            N.call("ff_filter_rays", ctypes.byref(desc), N.ptr(r), r.shape[0], N_samples, int(bool(bbox_only)),
                   N.ptr(k), N.stream_ptr())
            keep.append(k)
        keep = torch.cat(keep).bool() if keep else torch.zeros(0, dtype=torch.bool, device=self.device)
        keep = keep.to(rays.device)
        return rays[keep], rgbs[keep]

    # ---- checkpoints (models/FactorFields.py:669-691) --------------------------------------
    def reference_state_dict(self):
        """state_dict with the reference's keys and layouts (basises.l, coeffs.s as [1,C,...])."""
        sd = {}
        for k, v in self.state_dict().items():
            if k not in ("basis_flat", "coeff_flat"):
                sd[k] = v.detach().clone()
        for l, b in enumerate(self.basises):
            sd[f"basises.{l}"] = b.detach().contiguous().clone()
        for s, c in enumerate(self.coeffs):
            sd[f"coeffs.{s}"] = c.detach().contiguous().clone()
        return sd

    @torch.no_grad()
    def load_reference_state_dict(self, sd):
        own = {k: v for k, v in sd.items() if not (k.startswith("basises.") or k.startswith("coeffs."))}
        missing, unexpected = self.load_state_dict(
            {**own, "basis_flat": self.basis_flat, "coeff_flat": self.coeff_flat}, strict=False)
        for l in range(len(self.basis_dims)):
            self.layout.basis_view(self.basis_flat, l).copy_(sd[f"basises.{l}"].to(self.device))
        for s in range(self.n_scene):
            key = f"coeffs.{s}" if f"coeffs.{s}" in sd else "coeffs.0"
            self.layout.coeff_view(self.coeff_flat, s).copy_(sd[key].to(self.device))
        return unexpected

    def save(self, path):
        """models/FactorFields.py:669-680: the reference's keys and layouts, the packbits alpha
        mask, and in the reconstruction modes the scenes' coefficients averaged into coeffs.0
        (cal_mean_coef)."""
        ckpt = {"state_dict": self.reference_state_dict(), "cfg": dict(self.cfg)}
        if self.alphaMask is not None:
            vol = self.alphaMask.alpha_volume.bool().cpu().numpy()
            ckpt.update({"alphaMask.shape": vol.shape, "alphaMask.mask": np.packbits(vol.reshape(-1)),
                         "alphaMask.aabb": self.alphaMask.aabb.cpu()})
        if "reconstruction" in self.cfg.defaults.mode:
            ckpt["state_dict"] = self.cal_mean_coef(ckpt["state_dict"])
        torch.save(ckpt, path)

    def load(self, ckpt):
        """models/FactorFields.py:682-691 (render parameters recomputed for volume_resoFinal,
        as the reference does, whatever the mode)."""
        if "alphaMask.aabb" in ckpt:
            from .renderer import AlphaGridMask
            length = int(np.prod(ckpt["alphaMask.shape"]))
            vol = torch.from_numpy(np.unpackbits(ckpt["alphaMask.mask"])[:length].reshape(ckpt["alphaMask.shape"]))
            self.alphaMask = AlphaGridMask(self.device, ckpt["alphaMask.aabb"].to(self.device), vol.float().to(self.device))
        self.load_reference_state_dict(ckpt["state_dict"])
        self.update_renderParams(n_to_reso(self.cfg.training.volume_resoFinal ** self.in_dim, self.aabb.cpu()))
