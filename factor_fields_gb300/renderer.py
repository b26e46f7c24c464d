"""Renderer surface: render_ray (renderer.py:8-27), the colour heads (MLPRender_Fea,
models/FactorFields.py:162-203, and the degree-2 SH head), the occupancy mask and
FactorFields.forward (models/FactorFields.py:843-898) for bounded scenes, on the native
march / compact / composite kernels.

Per chunk of rays: ff_march_count -> ff_scan_counts -> ff_march_emit give the live samples in
the reference's order (xyz_sampled[ray_valid]); the field + MLP head runs on them (drop-in
float32 kernels, or the fused BF16 kernel). With the SH head, ff_composite_forward evaluates the
colours and alpha-composites in one pass. With MLPRender_Fea, ff_composite_weights gives the
weights, ff_app_emit lists the samples above the weight threshold (app_mask), the colour head
runs on them and ff_composite_forward_rgb composites. The backward runs the same chain in
reverse. One host synchronisation per chunk reads the number of live samples (the reference
synchronises on ray_valid.any()), and one more the number of head samples (app_mask.any()).
"""
import ctypes
import math

import torch

from . import _native as N
from . import functional as FN
from .config import Cfg


class SHRender(torch.nn.Module):
    """Degree-2 spherical-harmonics colour head: rgb = sigmoid(eval_sh(2, feat.view(-1, 3, 9), dirs))
    (models/sh.py:34-64 composed as the reference's renderModule). No parameters."""

    def __init__(self, in_channels=27):
        super().__init__()
        # A field fitted without rendering (e.g. an SDF with out_dim = 1) still owns a head, as
        # in the reference; the channel count is checked when rays are rendered.
        self.in_channels = in_channels


class AlphaGridMask(torch.nn.Module):
    """models/FactorFields.py:91-110: a 0/1 occupancy volume [D, H, W] over an aabb, kept as
    the float volume (reference layout) and as a packed bitfield for the kernels."""

    def __init__(self, device, aabb, alpha_volume, bits=None):
        super().__init__()
        self.device = device
        self.aabb = aabb.to(device)
        self.aabbSize = self.aabb[1] - self.aabb[0]
        self.invgridSize = 1.0 / self.aabbSize * 2
        self.aabb_host = aabb.detach().cpu()  # host copies for the render descriptor
        self.inv_host = 1.0 / (self.aabb_host[1] - self.aabb_host[0]) * 2
        self.alpha_volume = alpha_volume.view(1, 1, *alpha_volume.shape[-3:]).to(device)
        self.gridSize = torch.tensor([alpha_volume.shape[-1], alpha_volume.shape[-2], alpha_volume.shape[-3]],
                                     dtype=torch.long, device=device)
        # bits: the packed volume when the caller has it (ff_occupancy_mask), else packed here
        self.bits = bits.to(device) if bits is not None else pack_bits(self.alpha_volume.reshape(-1) > 0)

    def sample_alpha(self, xyz_sampled):
        """The reference's trilinear lookup (:103-107) — used for inspection, not by the kernels."""
        import torch.nn.functional as F
        pts = (xyz_sampled - self.aabb[0]) * self.invgridSize - 1
        return F.grid_sample(self.alpha_volume, pts.view(1, -1, 1, 1, 3), align_corners=True).view(-1)


def pack_bits(flags):
    """Bool vector -> int32 words, bit k of word w = flags[32 w + k]."""
    n = flags.numel()
    pad = (-n) % 32
    f = torch.nn.functional.pad(flags.to(torch.int64), (0, pad)).view(-1, 32)
    words = (f << torch.arange(32, device=f.device, dtype=torch.int64)).sum(1)
    return words.to(torch.int32).contiguous()


class MLPRender_Fea(torch.nn.Module):
    """models/FactorFields.py:162-203: rgb = sigmoid(MLP([features, viewdirs, PE(features, feape),
    PE(viewdirs, viewpe)])), Linear + ReLU per hidden layer, the last Linear (to 3) without bias.
    Same parameter names (mlp.i.weight / bias) and initialisation as the reference; the math runs
    on the native kernels (float32 drop-in, or the tensor-core head on the fused BF16 path)."""

    def __init__(self, inChanel, num_layers=3, hidden_dim=64, viewpe=6, feape=2):
        super().__init__()
        self.in_mlpC = 3 + inChanel + 2 * viewpe * 3 + 2 * feape * inChanel
        self.in_channels, self.num_layers, self.hidden_dim = inChanel, num_layers, hidden_dim
        self.viewpe, self.feape = viewpe, feape
        layers = []
        for l in range(num_layers):
            din = self.in_mlpC if l == 0 else hidden_dim
            last = l == num_layers - 1
            layers.append(torch.nn.Linear(din, 3 if last else hidden_dim, bias=not last))
        self.mlp = torch.nn.ModuleList(layers)

    def params(self):
        return [l.weight for l in self.mlp], [l.bias for l in self.mlp]

    def forward(self, viewdirs, features):
        """Colours [N, 3] of N samples from their view directions [N, 3] and features [N, C]."""
        return HeadFunction.apply(features, viewdirs, self, *[p for p in self.parameters()])


def head_struct(head):
    """FFRenderMlp of an MLPRender_Fea module (float32 parameters, contiguous)."""
    h = N.FFRenderMlp()
    h.n_layers, h.in_channels, h.hidden_dim = head.num_layers, head.in_channels, head.hidden_dim
    h.view_pe, h.fea_pe, h.in_dim = head.viewpe, head.feape, head.in_mlpC
    ws, bs = head.params()
    for i, (w, b) in enumerate(zip(ws, bs)):
        h.weight[i] = w.data_ptr()
        h.bias[i] = b.data_ptr() if b is not None else None
    return h


def _head_workspace(h, n):
    need = int(N.lib().ff_render_head_workspace_bytes(ctypes.byref(h), n))
    N.check(0 if need >= 0 else need, "ff_render_head_workspace_bytes")
    return torch.empty(max(need, 256), dtype=torch.uint8, device="cuda"), need


def head_tc_supported(head):
    """The tensor-core head's shapes: 3 layers, 128 hidden, fea_pe 2, view_pe 6, C = 27 or 31."""
    return (head.num_layers == 3 and head.hidden_dim == 128 and head.feape == 2 and head.viewpe == 6
            and head.in_channels in (27, 31))


def head_forward(head, feat, rays, app_idx, app_ray, rgb_sample, tc=False, status=None):
    """rgb_sample[app_idx[i]] = colour of app sample i (features = feat[app_idx[i], 1:], direction =
    rays[app_ray[i], 3:6]): the float32 drop-in head, or with tc the tensor-core head (FP16
    operands with the BF16-rounded weights, FP32 accumulation; status: optional zeroed device
    int32 that reports a bounded-wait failure or an input outside the FP16 range)."""
    n = app_idx.shape[0]
    if n == 0:
        return
    h = head_struct(head)
    if tc:
        N.call("ff_render_head_forward_tc", ctypes.byref(h), N.ptr(feat), feat.shape[1], N.ptr(rays), N.ptr(app_idx),
               N.ptr(app_ray), n, N.ptr(rgb_sample), N.ptr(status), N.stream_ptr())
        return
    ws, need = _head_workspace(h, n)
    N.call("ff_render_head_forward", ctypes.byref(h), N.ptr(feat), feat.shape[1], N.ptr(rays), N.ptr(app_idx),
           N.ptr(app_ray), n, N.ptr(rgb_sample), N.ptr(ws), need, N.stream_ptr(), kernels=1 + head.num_layers)


def head_backward(head, feat, rays, app_idx, app_ray, g_rgb_sample, g_feat, direct=True, tc=False, status=None):
    """Backward of head_forward: g_feat rows app_idx, channels 1..C (overwritten); the head's
    parameter gradients accumulated into their .grad (direct) or returned as a list."""
    ws_, bs_ = head.params()
    if direct:
        gw = [_direct_grad(w) for w in ws_]
        gb = [_direct_grad(b) if b is not None else None for b in bs_]
    else:
        gw = [torch.zeros_like(w) for w in ws_]
        gb = [torch.zeros_like(b) if b is not None else None for b in bs_]
    n = app_idx.shape[0]
    if n:
        h = head_struct(head)
        g = N.FFMlpGrad()
        for i in range(len(gw)):
            g.weight[i] = gw[i].data_ptr()
            g.bias[i] = gb[i].data_ptr() if gb[i] is not None else None
        if tc:
            N.call("ff_render_head_backward_tc", ctypes.byref(h), N.ptr(feat), feat.shape[1], N.ptr(rays),
                   N.ptr(app_idx), N.ptr(app_ray), n, N.ptr(g_rgb_sample), N.ptr(g_feat), ctypes.byref(g),
                   N.ptr(status), N.stream_ptr())
            return gw, gb
        ws, need = _head_workspace(h, n)
        n_bias = sum(1 for b in bs_ if b is not None)
        N.call("ff_render_head_backward", ctypes.byref(h), N.ptr(feat), feat.shape[1], N.ptr(rays), N.ptr(app_idx),
               N.ptr(app_ray), n, N.ptr(g_rgb_sample), N.ptr(g_feat), ctypes.byref(g), N.ptr(ws), need,
               N.stream_ptr(), kernels=4 + head.num_layers * 3 + n_bias)
    return gw, gb


class HeadFunction(torch.autograd.Function):
    """MLPRender_Fea.forward(viewdirs, features) on its own (one app sample per row)."""

    @staticmethod
    def forward(ctx, features, viewdirs, head, *params):
        n, c = features.shape
        dev = features.device
        feat = torch.zeros(n, c + 1, device=dev)
        feat[:, 1:] = features.to(torch.float32)
        rays = torch.zeros(n, 6, device=dev)
        rays[:, 3:6] = viewdirs.to(torch.float32)
        idx = torch.arange(n, dtype=torch.int32, device=dev)
        rgb = torch.empty(n, 3, device=dev)
        head_forward(head, feat, rays, idx, idx, rgb)
        ctx.save_for_backward(feat, rays, idx)
        ctx.head = head
        return rgb

    @staticmethod
    def backward(ctx, g_rgb):
        feat, rays, idx = ctx.saved_tensors
        g_feat = torch.zeros_like(feat)
        gw, gb = head_backward(ctx.head, feat, rays, idx, idx, g_rgb.contiguous(), g_feat, direct=False)
        grads = []
        for w, b in zip(gw, gb):
            grads.append(w)
            if b is not None:
                grads.append(b)
        return (g_feat[:, 1:], None, None, *grads)


def make_render_module(cfg, in_channels):
    """The colour head: MLPRender_Fea (the reference's head, built whatever shadingMode says,
    :243-246) unless renderer.shadingMode is 'SH' (the degree-2 SH head)."""
    rc = cfg.renderer or Cfg()
    shading = rc.get("shadingMode") or "MLP_Fea"
    if shading == "SH":
        return SHRender(in_channels)
    return MLPRender_Fea(inChanel=in_channels, num_layers=int(rc.get("num_layers") or 3),
                         hidden_dim=int(rc.get("hidden_dim") or 128), viewpe=int(rc.get("view_pe", 6)),
                         feape=int(rc.get("fea_pe", 2)))


def render_desc(model, n_samples, white_bg):
    """FFRender for a FactorFields model (float32 constants computed as the reference does).
    Reads the host copies of aabb / stepSize that update_renderParams keeps (no device read, so a
    render can be captured in a CUDA graph) while model.aabb is the tensor they were taken from,
    unmodified; otherwise the device values."""
    r = N.FFRender()
    host = getattr(model, "_render_host", None)
    if host is not None and host[0] is model.aabb and host[1] == model.aabb._version:
        aabb, step = host[2], host[3]
    else:
        aabb, step = model.aabb.detach().cpu(), float(model.stepSize.detach().cpu())
    for k in range(3):
        r.aabb_min[k] = float(aabb[0, k])
        r.aabb_max[k] = float(aabb[1, k])
    r.step = step
    r.n_samples = int(n_samples)
    rc = model.cfg.renderer
    r.distance_scale = float(rc.distance_scale)
    r.density_shift = float(rc.density_shift)
    act = rc.fea2denseAct or "softplus"
    if act not in ("softplus", "relu"):
        raise NotImplementedError(f"fea2denseAct {act!r}")
    r.density_act = 0 if act == "softplus" else 1
    r.weight_thres = float(rc.rayMarch_weight_thres)
    r.white_bg = 1 if white_bg else 0
    mask = model.alphaMask
    if mask is not None:
        r.occ_bits = mask.bits.data_ptr()
        vol = mask.alpha_volume
        r.occ_reso[0], r.occ_reso[1], r.occ_reso[2] = vol.shape[-1], vol.shape[-2], vol.shape[-3]
        a0, inv = mask.aabb_host, mask.inv_host
        for k in range(3):
            r.occ_origin[k] = float(a0[0, k])
            r.occ_inv[k] = float(inv[k])
    return r


def march(model, rays, jitter, rdesc):
    """Live samples of a chunk: (offsets [R+1] int64, xyz [M, 3], sample_idx [M] int32)."""
    n = rays.shape[0]
    dev = rays.device
    st = N.stream_ptr()
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    N.call("ff_march_count", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(counts), None, st)
    offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
    wsb = N.lib().ff_scan_workspace_bytes(n)
    ws = torch.empty(max(wsb, 8), dtype=torch.uint8, device=dev)
    N.call("ff_scan_counts", N.ptr(counts), n, N.ptr(offsets), N.ptr(ws), wsb, st)
    m = int(offsets[-1].item())
    xyz = torch.empty(m, 3, device=dev)
    sidx = torch.empty(m, dtype=torch.int32, device=dev)
    if m > 0:
        N.call("ff_march_emit", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(offsets), N.ptr(xyz),
               N.ptr(sidx), st)
    return offsets, xyz, sidx


def march_static(model, rays, jitter, rdesc):
    """march() without the host read of the live-sample count: xyz / sample_idx sized for every
    sample slot (n_rays * n_samples rows, the first offsets[-1] of them written), the count left on
    the device in offsets[-1]. Returns (offsets, xyz, sample_idx)."""
    n = rays.shape[0]
    dev = rays.device
    st = N.stream_ptr()
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    N.call("ff_march_count", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(counts), None, st)
    offsets = scan_counts(counts)
    m_max = n * int(rdesc.n_samples)
    xyz = torch.empty(m_max, 3, device=dev)
    sidx = torch.empty(m_max, dtype=torch.int32, device=dev)
    if n:
        N.call("ff_march_emit", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(offsets), N.ptr(xyz),
               N.ptr(sidx), st)
    return offsets, xyz, sidx


def sh_render_forward(job, rays, jitter):
    """The SH-2 render forward on the native kernels: (rgb, depth, saved tensors for the
    backward). Static jobs (job['static']) make no host read."""
    m, rdesc = job["model"], job["rdesc"]
    if job.get("static"):  # no host synchronisation: capturable in a CUDA graph
        offsets, xyz, sidx = march_static(m, rays, jitter, rdesc)
        job["n_dev"] = offsets[rays.shape[0]:]
    else:
        offsets, xyz, sidx = march(m, rays, jitter, rdesc)
    feat = field_eval(m, job, xyz)
    n = rays.shape[0]
    rgb = torch.empty(n, 3, device=rays.device)
    depth = torch.empty(n, device=rays.device)
    N.call("ff_composite_forward", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(offsets),
           N.ptr(sidx), N.ptr(feat), feat.shape[1], None, N.ptr(rgb), N.ptr(depth), None, N.stream_ptr())
    job["xyz"] = xyz
    return rgb, depth, (rays, offsets, xyz, sidx, feat)


def sh_render_backward(job, jitter, saved, g_rgb):
    """Backward of sh_render_forward for dL/drgb: the compositing reverse scan, then the field
    and MLP backward (field_grad)."""
    rays, offsets, xyz, sidx, feat = saved
    rdesc = job["rdesc"]
    n = rays.shape[0]
    g_feat = torch.empty_like(feat)
    g_rgb = g_rgb.contiguous()
    N.call("ff_composite_backward", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(offsets),
           N.ptr(sidx), N.ptr(feat), feat.shape[1], None, N.ptr(g_rgb), N.ptr(g_feat), N.stream_ptr())
    return field_grad(job["model"], job, xyz, g_feat)


class RenderFunction(torch.autograd.Function):
    """rgb, depth = render(rays) with gradients to the grids and the MLP head.

    apply(rays, jitter, basis_param, coeff_param, w0, b0, w1, ctx_obj) where ctx_obj carries the
    model, its read buffers, descriptors and the path (fused or drop-in)."""

    @staticmethod
    def forward(ctx, rays, jitter, basis_param, coeff_param, w0, b0, w1, job):
        rgb, depth, saved = sh_render_forward(job, rays, jitter)
        ctx.save_for_backward(*saved)
        ctx.jitter, ctx.job = jitter, job
        ctx.mark_non_differentiable(depth)
        return rgb, depth

    @staticmethod
    def backward(ctx, g_rgb, g_depth):
        grads = sh_render_backward(ctx.job, ctx.jitter, ctx.saved_tensors, g_rgb)
        return (None, None) + grads + (None,)


def scan_counts(counts):
    """Exclusive scan of int32 counts -> int64 offsets [n + 1] (ff_scan_counts)."""
    n = counts.shape[0]
    offsets = torch.empty(n + 1, dtype=torch.int64, device=counts.device)
    wsb = N.lib().ff_scan_workspace_bytes(n)
    ws = torch.empty(max(wsb, 8), dtype=torch.uint8, device=counts.device)
    N.call("ff_scan_counts", N.ptr(counts), n, N.ptr(offsets), N.ptr(ws), wsb, N.stream_ptr())
    return offsets


class RenderFunctionMLP(torch.autograd.Function):
    """rgb, depth = render(rays) with the MLPRender_Fea colour head (models/FactorFields.py:
    862-898): march -> field + MLP -> compositing weights -> the samples above the weight
    threshold (app_mask) -> the colour head on them -> compositing. Gradients reach the grids,
    the field MLP and the head.

    apply(rays, jitter, basis_param, coeff_param, w0, b0, w1, job, *head_params)."""

    @staticmethod
    def forward(ctx, rays, jitter, basis_param, coeff_param, w0, b0, w1, job, *head_params):
        m, rdesc = job["model"], job["rdesc"]
        head = m.renderModule
        offsets, xyz, sidx = march(m, rays, jitter, rdesc)
        feat = field_eval(m, job, xyz)
        n, M = rays.shape[0], feat.shape[0]
        dev = rays.device
        st = N.stream_ptr()
        w = torch.empty(M, device=dev)
        app_counts = torch.empty(n, dtype=torch.int32, device=dev)
        N.call("ff_composite_weights", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(offsets), N.ptr(sidx),
               N.ptr(feat), feat.shape[1], N.ptr(w), N.ptr(app_counts), st)
        app_off = scan_counts(app_counts)
        n_app = int(app_off[-1].item())  # the reference synchronises on app_mask.any() (:883)
        app_idx = torch.empty(n_app, dtype=torch.int32, device=dev)
        app_ray = torch.empty(n_app, dtype=torch.int32, device=dev)
        if n_app:
            N.call("ff_app_emit", n, N.ptr(offsets), N.ptr(w), float(rdesc.weight_thres), N.ptr(app_off),
                   N.ptr(app_idx), N.ptr(app_ray), st)
        rgb_sample = torch.empty(M, 3, device=dev)
        job["head_tc"] = bool(job["fused"]) and head_tc_supported(head)
        head_forward(head, feat, rays, app_idx, app_ray, rgb_sample, tc=job["head_tc"])
        rgb = torch.empty(n, 3, device=dev)
        depth = torch.empty(n, device=dev)
        N.call("ff_composite_forward_rgb", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jitter), n, N.ptr(offsets),
               N.ptr(sidx), N.ptr(feat), feat.shape[1], N.ptr(rgb_sample), None, N.ptr(rgb), N.ptr(depth), None, st)
        ctx.save_for_backward(rays, offsets, xyz, sidx, feat, rgb_sample, app_idx, app_ray)
        ctx.jitter, ctx.job = jitter, job
        ctx.mark_non_differentiable(depth)
        job["xyz"] = xyz
        return rgb, depth

    @staticmethod
    def backward(ctx, g_rgb, g_depth):
        rays, offsets, xyz, sidx, feat, rgb_sample, app_idx, app_ray = ctx.saved_tensors
        job = ctx.job
        m, rdesc = job["model"], job["rdesc"]
        n = rays.shape[0]
        g_feat = torch.empty_like(feat)
        g_rgb_sample = torch.empty_like(rgb_sample)
        g_rgb = g_rgb.contiguous()
        N.call("ff_composite_backward_rgb", ctypes.byref(rdesc), N.ptr(rays), N.ptr(ctx.jitter), n, N.ptr(offsets),
               N.ptr(sidx), N.ptr(feat), feat.shape[1], N.ptr(rgb_sample), None, N.ptr(g_rgb), N.ptr(g_feat),
               N.ptr(g_rgb_sample), N.stream_ptr())
        direct = getattr(m, "accumulate_grad_directly", True)
        gw, gb = head_backward(m.renderModule, feat, rays, app_idx, app_ray, g_rgb_sample, g_feat, direct=direct,
                               tc=job["head_tc"])
        grads = field_grad(m, job, xyz, g_feat)
        head_grads = []
        for wg, bg in zip(gw, gb):
            head_grads.append(None if direct else wg)
            if bg is not None:
                head_grads.append(None if direct else bg)
        return (None, None) + grads + (None,) + tuple(head_grads)


def field_eval(m, job, xyz):
    """MLP output [M, out_dim] of the field at xyz (fused BF16 path or drop-in float32 path)."""
    n = xyz.shape[0]
    out_dim = m.linear_mat.out_dim
    out = torch.empty(n, out_dim, device=xyz.device)
    if n == 0:
        return out
    st = N.stream_ptr()
    lm = m.linear_mat
    ws, bs = lm.weights()
    mlp = FN.mlp_struct(ws, bs, lm.in_dim, lm.hidden_dim, lm.out_dim)
    if job["fused"] and job.get("n_dev") is not None:
        N.call("ff_field_mlp_forward_counted", ctypes.byref(job["fdesc"]), N.ptr(job["basis_r"]),
               N.ptr(job["coeff_r"]), ctypes.byref(mlp), N.ptr(xyz), n, N.ptr(job["n_dev"]), N.ptr(out), st)
    elif job["fused"]:
        N.call("ff_field_mlp_forward", ctypes.byref(job["fdesc"]), N.ptr(job["basis_r"]), N.ptr(job["coeff_r"]),
               ctypes.byref(mlp), N.ptr(xyz), n, N.ptr(out), st)
    else:
        feats = torch.empty(n, m.n_feat, device=xyz.device)
        N.call("ff_field_forward", ctypes.byref(job["fdesc"]), N.ptr(job["basis_r"]), N.ptr(job["coeff_r"]),
               N.ptr(xyz), n, N.ptr(feats), None, None, st)
        N.call("ff_mlp_forward", ctypes.byref(mlp), N.ptr(feats), n, N.ptr(out), st)
        job["feats"] = feats
    return out


def _direct_grad(p):
    """p.grad (zeros when missing) for the kernels to accumulate into."""
    if p.grad is None:
        p.grad = torch.zeros_like(p)
    return p.grad


def field_grad(m, job, xyz, g_out):
    """(grad_basis, grad_coeff, grad_w0, grad_b0, grad_w1) for dL/dout = g_out at xyz.

    With m.accumulate_grad_directly (the default) the kernels accumulate straight into the
    parameters' .grad buffers and None is returned for them: no per-step zeroed gradient
    buffers and no autograd additions of 40-70 MB grids (torch.autograd.grad does not see
    these gradients; set the attribute to False for that)."""
    lm = m.linear_mat
    ws, bs = lm.weights()
    direct = getattr(m, "accumulate_grad_directly", True)
    if direct:
        gb = _direct_grad(m.basis_flat)
        gc = _direct_grad(m.coeff_flat)
        if job["coeff_param"] is not m.coeff_flat:
            gc = m._coeff_scene(gc)
        gw = [_direct_grad(w) for w in ws]
        gbias = [_direct_grad(b) if b is not None else None for b in bs]
    else:
        gb = torch.zeros_like(m.basis_flat)
        gc = torch.zeros_like(job["coeff_param"])
        gw = [torch.zeros_like(w) for w in ws]
        gbias = [torch.zeros_like(b) if b is not None else None for b in bs]
    n = xyz.shape[0]
    if n:
        st = N.stream_ptr()
        mlp = FN.mlp_struct(ws, bs, lm.in_dim, lm.hidden_dim, lm.out_dim)
        g = N.FFMlpGrad()
        for i in range(len(ws)):
            g.weight[i] = gw[i].data_ptr()
            g.bias[i] = gbias[i].data_ptr() if gbias[i] is not None else None
        if job["fused"] and job.get("n_dev") is not None:
            N.call("ff_field_mlp_backward_counted", ctypes.byref(job["fdesc"]), N.ptr(job["basis_r"]),
                   N.ptr(job["coeff_r"]), ctypes.byref(mlp), N.ptr(xyz), n, N.ptr(job["n_dev"]), N.ptr(g_out),
                   N.ptr(gb), N.ptr(gc), ctypes.byref(g), st)
        elif job["fused"]:
            N.call("ff_field_mlp_backward", ctypes.byref(job["fdesc"]), N.ptr(job["basis_r"]),
                   N.ptr(job["coeff_r"]), ctypes.byref(mlp), N.ptr(xyz), n, N.ptr(g_out), N.ptr(gb), N.ptr(gc),
                   ctypes.byref(g), st)
        else:
            feats = job["feats"]
            g_feats = torch.empty_like(feats)
            N.call("ff_mlp_backward", ctypes.byref(mlp), N.ptr(feats), n, N.ptr(g_out), N.ptr(g_feats),
                   ctypes.byref(g), st)
            N.call("ff_field_backward", ctypes.byref(job["fdesc"]), N.ptr(job["basis_r"]), N.ptr(job["coeff_r"]),
                   N.ptr(xyz), n, N.ptr(g_feats), None, None, N.ptr(gb), N.ptr(gc), st)
    if direct:
        return (None, None, None, None, None)
    return (gb, gc, gw[0], gbias[0], gw[1] if len(gw) > 1 else None)


def render_job(model, rays, n_samples, white_bg, fused, static):
    """The descriptors and read buffers of one render call."""
    basis_r, coeff_r, dt = model._read_buffers()
    coeff_param = model.coeff_flat
    if model.n_scene > 1:
        coeff_param = model._coeff_scene(model.coeff_flat)
        coeff_r = model._coeff_scene(coeff_r)
    return {"model": model, "rdesc": render_desc(model, n_samples, white_bg), "fdesc": model.descriptor(dt),
            "basis_r": basis_r, "coeff_r": coeff_r, "coeff_param": coeff_param, "fused": fused, "static": static}


def render_forward(model, rays_chunk, white_bg=True, is_train=False, ndc_ray=False, N_samples=-1, fused=None,
                   jitter=None, static=False):
    """FactorFields.forward (models/FactorFields.py:843-898), bounded scenes, with the model's
    colour head (MLPRender_Fea or the SH-2 head): returns (rgb_map [R, 3], depth_map [R], coeffs).

    jitter: optional per-ray sample offsets [R] in [0, 1) (the reference draws them with
    torch.rand_like when is_train); given explicitly they make sampling reproducible.
    static: no host synchronisation (live-sample buffers sized for every sample slot, the
    live count read by the kernels on the device), so the call can be captured in a CUDA graph;
    the fused BF16 path with the SH-2 head only."""
    if ndc_ray:
        raise NotImplementedError("NDC rays (sample_point_ndc) are not on this path")
    mlp_head = isinstance(model.renderModule, MLPRender_Fea)
    if not mlp_head and model.linear_mat.out_dim < 28:
        raise NotImplementedError("the SH-2 colour head needs out_dim >= 28")
    if mlp_head and model.renderModule.in_channels != model.linear_mat.out_dim - 1:
        raise ValueError("MLPRender_Fea's inChanel must be out_dim - 1")
    lm = model.linear_mat
    if lm.num_layers != 2:
        raise NotImplementedError("rendering needs an MLPMixer with num_layers = 2")
    rays = rays_chunk.to(model.device, torch.float32).contiguous()
    n_samples = N_samples if N_samples > 0 else model.nSamples
    if jitter is not None:
        jitter = jitter.to(rays.device, torch.float32).reshape(-1).contiguous()
    elif is_train:
        jitter = torch.rand(rays.shape[0], device=rays.device)
    wb = bool(white_bg or (is_train and torch.rand((1,)) < 0.5))  # :890
    if fused is None:
        fused = model.precision == "bf16"
    job = render_job(model, rays, n_samples, wb, fused, static)
    coeff_param = job["coeff_param"]
    if static and (mlp_head or not fused):
        raise NotImplementedError("static (graph-capturable) rendering needs the fused BF16 path and the SH-2 head")
    l0, l1 = lm.backbone
    if mlp_head:
        rgb, depth = RenderFunctionMLP.apply(rays, jitter, model.basis_flat, coeff_param, l0.weight, l0.bias,
                                             l1.weight, job, *list(model.renderModule.parameters()))
    else:
        rgb, depth = RenderFunction.apply(rays, jitter, model.basis_flat, coeff_param, l0.weight, l0.bias, l1.weight,
                                          job)
    coeffs = torch.zeros((1, model.n_feat), device=rays.device)
    if getattr(model, "return_coeffs", False) and not static and job["xyz"].shape[0]:
        with torch.no_grad():
            coeffs = model.get_coeff(job["xyz"])
    return rgb, depth, coeffs


def render_ray(rays, factor_fields, chunk=4096, N_samples=-1, ndc_ray=False, white_bg=True, is_train=False,
               device="cuda"):
    """renderer.py:8-27: render rays in chunks; returns (rgb, depth) or, when training,
    (rgb, depth, coeffs)."""
    rgbs, depths, coeffs = [], [], []
    n = rays.shape[0]
    for c in range(n // chunk + int(n % chunk > 0)):
        rc = rays[c * chunk:(c + 1) * chunk].to(device)
        rgb, depth, coeff = factor_fields(rc, is_train=is_train, white_bg=white_bg, ndc_ray=ndc_ray,
                                          N_samples=N_samples)
        rgbs.append(rgb)
        depths.append(depth)
        if is_train:
            coeffs.append(coeff)
    if is_train:
        return torch.cat(rgbs), torch.cat(depths), torch.cat(coeffs)
    return torch.cat(rgbs), torch.cat(depths)


def image_metrics(img0, img1, max_val=1.0):
    """(mse, ssim) of two [H, W, C] float32 device images (ff_image_metrics: the reference's
    rgb_ssim, utils.py:110-156, and the MSE behind its PSNR, renderer.py:64)."""
    a = img0.to(torch.float32).contiguous()
    b = img1.to(device=a.device, dtype=torch.float32).contiguous()
    h, w, c = a.shape
    need = int(N.lib().ff_image_metrics_workspace_bytes(h, w, c))
    N.check(0 if need >= 0 else need, "ff_image_metrics_workspace_bytes")
    ws = torch.empty(need, dtype=torch.uint8, device=a.device)
    out = (ctypes.c_double * 2)()
    N.call("ff_image_metrics", N.ptr(a), N.ptr(b), h, w, c, float(max_val), out, N.ptr(ws), need, N.stream_ptr())
    return float(out[0]), float(out[1])


@torch.no_grad()
def evaluation(test_dataset, factor_fields, renderer=None, savePath=None, N_vis=5, prtx="", N_samples=-1,
               white_bg=False, ndc_ray=False, compute_extra_metrics=True, device="cuda", chunk=None,
               sampler=None):
    """renderer.py:30-98: render every (N_vis-spaced) test image and return its PSNRs.

    The image's rays are rendered in one pass (chunk=None: H*W rays; the reference uses
    chunks of 1,024), with the plain sampler through `renderer` (default render_ray) or, if
    `sampler` is given, with the learned proposal sampler. Metrics run on the GPU
    (ff_image_metrics): PSNR from the MSE and, with compute_extra_metrics, SSIM as the
    reference's rgb_ssim. LPIPS is not computed: it needs the lpips package and its pretrained
    AlexNet/VGG weights, which are not available. With savePath, each rendered image is saved
    as <prtx><idx>.npy (uint8 [H, W, 3]) and <prtx>mean.txt holds (psnr[, ssim], n_params);
    the reference's PNG/MP4 writers and the colour-mapped depth image are left out.
    Returns (PSNRs, extras) with extras = {"ssim": [...], "ms_per_image": [...]}."""
    import os
    import time
    renderer = renderer or render_ray
    W, H = test_dataset.img_wh
    all_rays, all_rgbs = test_dataset.all_rays, test_dataset.all_rgbs
    n_img = all_rays.shape[0]
    step = 1 if N_vis < 0 else max(n_img // N_vis, 1)
    idxs = list(range(0, n_img, step))
    psnrs, ssims, times = [], [], []
    if savePath is not None:
        os.makedirs(savePath, exist_ok=True)
    for idx in idxs:
        rays = all_rays[idx].reshape(-1, all_rays.shape[-1]).to(device, torch.float32)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if sampler is not None:
            rgb, depth = sampler.render(rays, is_train=False, white_bg=white_bg)
        else:
            rgb, depth = renderer(rays, factor_fields, chunk=chunk or rays.shape[0], N_samples=N_samples,
                                  ndc_ray=ndc_ray, white_bg=white_bg, device=device)
        rgb = rgb.clamp(0.0, 1.0).reshape(H, W, 3)
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t0) * 1e3)
        if all_rgbs is not None and len(all_rgbs):
            gt = all_rgbs[idx].reshape(H, W, 3).to(device, torch.float32)
            mse, ssim = image_metrics(rgb, gt, 1.0)
            psnrs.append(-10.0 * math.log10(mse))
            if compute_extra_metrics:
                ssims.append(ssim)
        if savePath is not None:
            import numpy as np
            np.save(os.path.join(savePath, f"{prtx}{idx:03d}.npy"), (rgb.cpu().numpy() * 255).astype("uint8"))
    if savePath is not None and psnrs:
        import numpy as np
        vals = [float(np.mean(psnrs))] + ([float(np.mean(ssims))] if ssims else []) + [factor_fields.n_parameters()]
        np.savetxt(os.path.join(savePath, f"{prtx}mean.txt"), np.asarray(vals))
    return psnrs, {"ssim": ssims, "ms_per_image": times}
