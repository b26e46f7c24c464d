"""torch.autograd.Function wrappers around the native kernels (drop-in float32 path).

Each Function saves only its inputs; the backward launches recompute interpolation weights
and gathered values instead of storing them.
"""
import ctypes

import torch

from . import _native as N


def _contig_f32(t, name):
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if not t.is_cuda:
        raise N.NativeError(f"{name} must be a CUDA tensor (no CPU fallback)")
    return t.contiguous()


class FieldCoding(torch.autograd.Function):
    """(feats, coeff, basis) = get_coding / get_basis outputs for points x.

    Inputs: x [N, coord_dim]; basis_param / coeff_param: the float32 master parameters that
    receive gradients; basis_read / coeff_read: the buffers the kernel reads (the parameters
    themselves, or their BF16 copies); desc: the FFField; want: tuple of three bools selecting
    which outputs to produce (feats, coeff, basis) — unselected outputs are returned as None."""

    @staticmethod
    def forward(ctx, x, basis_param, coeff_param, basis_read, coeff_read, desc, want):
        x = _contig_f32(x, "points")
        n, f = x.shape[0], desc.n_feat
        outs = [torch.empty(n, f, device=x.device, dtype=torch.float32) if w else None for w in want]
        N.call("ff_field_forward", ctypes.byref(desc), N.ptr(basis_read), N.ptr(coeff_read), N.ptr(x), n,
               N.ptr(outs[0]), N.ptr(outs[1]), N.ptr(outs[2]), N.stream_ptr())
        ctx.save_for_backward(x, basis_read, coeff_read)
        ctx.desc = desc
        ctx.shapes = (basis_param.shape, coeff_param.shape)
        ctx.want = want
        return tuple(outs)

    @staticmethod
    def backward(ctx, g_feats, g_coeff, g_basis):
        x, basis_read, coeff_read = ctx.saved_tensors
        need_b, need_c = ctx.needs_input_grad[1], ctx.needs_input_grad[2]
        gb = torch.zeros(ctx.shapes[0], device=x.device, dtype=torch.float32) if need_b else None
        gc = torch.zeros(ctx.shapes[1], device=x.device, dtype=torch.float32) if need_c else None
        if need_b or need_c:
            gs = [g.contiguous() if g is not None else None for g in (g_feats, g_coeff, g_basis)]
            N.call("ff_field_backward", ctypes.byref(ctx.desc), N.ptr(basis_read), N.ptr(coeff_read), N.ptr(x),
                   x.shape[0], N.ptr(gs[0]), N.ptr(gs[1]), N.ptr(gs[2]), N.ptr(gb), N.ptr(gc), N.stream_ptr())
        return None, gb, gc, None, None, None, None


def mlp_struct(weights, biases, in_dim, hidden_dim, out_dim):
    m = N.FFMlp()
    m.n_layers = len(weights)
    if m.n_layers > N.FF_MAX_MLP_LAYERS:
        raise NotImplementedError(f"at most {N.FF_MAX_MLP_LAYERS} MLP layers are supported")
    m.in_dim, m.hidden_dim, m.out_dim = in_dim, hidden_dim, out_dim
    for i, (w, b) in enumerate(zip(weights, biases)):
        m.weight[i] = w.data_ptr()
        m.bias[i] = b.data_ptr() if b is not None else None
    return m


class MLPFunction(torch.autograd.Function):
    """MLPMixer forward (Linear+ReLU ..., last layer without bias) on the native float32 kernels.

    Call as MLPFunction.apply(x, dims, n_layers, *weights, *biases) with biases given as
    tensors or None (None entries are replaced by empty placeholders)."""

    @staticmethod
    def forward(ctx, x, dims, n_layers, *params):
        x = _contig_f32(x, "MLP input")
        weights = [p.contiguous() for p in params[:n_layers]]
        biases = [p.contiguous() if p is not None and p.numel() else None for p in params[n_layers:]]
        in_dim, hidden_dim, out_dim = dims
        m = mlp_struct(weights, biases, in_dim, hidden_dim, out_dim)
        out = torch.empty(x.shape[0], out_dim, device=x.device, dtype=torch.float32)
        N.call("ff_mlp_forward", ctypes.byref(m), N.ptr(x), x.shape[0], N.ptr(out), N.stream_ptr())
        ctx.save_for_backward(x, *weights, *[b if b is not None else torch.empty(0) for b in biases])
        ctx.dims, ctx.n_layers = dims, n_layers
        ctx.has_bias = [b is not None for b in biases]
        return out

    @staticmethod
    def backward(ctx, g_out):
        saved = ctx.saved_tensors
        L = ctx.n_layers
        x, weights = saved[0], list(saved[1:1 + L])
        biases = [b if h else None for b, h in zip(saved[1 + L:], ctx.has_bias)]
        m = mlp_struct(weights, biases, *ctx.dims)
        gw = [torch.zeros_like(w) if ctx.needs_input_grad[3 + i] else None for i, w in enumerate(weights)]
        gbias = [torch.zeros_like(b) if (b is not None and ctx.needs_input_grad[3 + L + i]) else None
                 for i, b in enumerate(biases)]
        g = N.FFMlpGrad()
        for i in range(L):
            g.weight[i] = gw[i].data_ptr() if gw[i] is not None else None
            g.bias[i] = gbias[i].data_ptr() if gbias[i] is not None else None
        gx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        g_out = g_out.contiguous()  # a named tensor stays alive until the launch is enqueued
        N.call("ff_mlp_backward", ctypes.byref(m), N.ptr(x), x.shape[0], N.ptr(g_out), N.ptr(gx),
               ctypes.byref(g), N.stream_ptr())
        return (gx, None, None, *gw, *gbias)


class FusedFieldMLP(torch.autograd.Function):
    """linear_mat(get_coding(x)[0]) in one fused launch (BF16 tensor-core MLP, FP32 accumulation).

    apply(x, basis_param, coeff_param, w0, b0, w1, basis_read, coeff_read, desc, dims)."""

    @staticmethod
    def forward(ctx, x, basis_param, coeff_param, w0, b0, w1, basis_read, coeff_read, desc, dims):
        x = _contig_f32(x, "points")
        w0, b0, w1 = w0.contiguous(), b0.contiguous(), w1.contiguous()
        m = mlp_struct([w0, w1], [b0, None], *dims)
        out = torch.empty(x.shape[0], dims[2], device=x.device, dtype=torch.float32)
        N.call("ff_field_mlp_forward", ctypes.byref(desc), N.ptr(basis_read), N.ptr(coeff_read), ctypes.byref(m),
               N.ptr(x), x.shape[0], N.ptr(out), N.stream_ptr())
        ctx.save_for_backward(x, w0, b0, w1, basis_read, coeff_read)
        ctx.desc, ctx.dims = desc, dims
        ctx.shapes = (basis_param.shape, coeff_param.shape)
        return out

    @staticmethod
    def backward(ctx, g_out):
        x, w0, b0, w1, basis_read, coeff_read = ctx.saved_tensors
        m = mlp_struct([w0, w1], [b0, None], *ctx.dims)
        gb = torch.zeros(ctx.shapes[0], device=x.device)
        gc = torch.zeros(ctx.shapes[1], device=x.device)
        gw0, gb0, gw1 = torch.zeros_like(w0), torch.zeros_like(b0), torch.zeros_like(w1)
        g = N.FFMlpGrad()
        g.weight[0], g.bias[0], g.weight[1] = gw0.data_ptr(), gb0.data_ptr(), gw1.data_ptr()
        g_out = g_out.contiguous()
        N.call("ff_field_mlp_backward", ctypes.byref(ctx.desc), N.ptr(basis_read), N.ptr(coeff_read),
               ctypes.byref(m), N.ptr(x), x.shape[0], N.ptr(g_out), N.ptr(gb), N.ptr(gc),
               ctypes.byref(g), N.stream_ptr())
        return None, gb, gc, gw0, gb0, gw1, None, None, None, None


def mlp(x, weights, biases, in_dim, hidden_dim, out_dim):
    L = len(weights)
    return MLPFunction.apply(x, (in_dim, hidden_dim, out_dim), L, *weights, *biases)
