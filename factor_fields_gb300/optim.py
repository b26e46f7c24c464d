"""FusedAdam: torch.optim.Adam (amsgrad=False, weight_decay=0) as one native pass per step.

The reference trains with torch.optim.Adam over get_optparam_groups (train_per_scene.py:132,
betas (0.9, 0.99)) and zero_grad() before each backward (:160). FusedAdam runs ff_adam_step:
for every parameter of every group the moment updates and the parameter update in torch's
operation order, plus, in the same pass, the BF16 copy the field kernels read (the model's
read buffers) and, by default, the gradient zeroing of the next step. State layout
(state[p] = {step, exp_avg, exp_avg_sq}) and param groups are torch's, so checkpoints and
learning-rate schedules written for torch.optim.Adam work unchanged.

The update writes parameters through their device pointers: torch's version counters do not
move. The BF16 copies registered through `shadows` are written by the same pass, so a model
whose read buffers are keyed on those counters stays consistent.
"""
import ctypes

import torch

from . import _native as N


class FusedAdam(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, zero_grad=True, shadows=None):
        if not 0.0 <= betas[0] < 1.0 or not 0.0 <= betas[1] < 1.0:
            raise ValueError(f"invalid betas {betas}")
        super().__init__(params, dict(lr=lr, betas=tuple(betas), eps=eps))
        self.fused_zero_grad = bool(zero_grad)
        self._shadows = {}
        for p, s in (shadows or {}).items():
            self.set_shadow(p, s)

    def set_shadow(self, param, shadow):
        """Register the BF16 copy of `param` that each step refreshes (None: stop)."""
        if shadow is None:
            self._shadows.pop(param, None)
            return
        if shadow.dtype != torch.bfloat16 or shadow.numel() != param.numel() or not shadow.is_contiguous():
            raise ValueError("a shadow is a contiguous BF16 tensor with the parameter's size")
        self._shadows[param] = shadow

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        by_hyper = {}
        for group in self.param_groups:
            b1, b2 = group["betas"]
            key = (float(b1), float(b2), float(group["eps"]))
            for p in group["params"]:
                if p.grad is None:
                    continue
                if p.dtype != torch.float32 or not p.is_contiguous() or not p.grad.is_contiguous():
                    raise ValueError("FusedAdam needs contiguous float32 parameters and gradients")
                st = self.state[p]
                if not st:
                    st["step"] = torch.tensor(0.0)
                    st["exp_avg"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                    st["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                st["step"] += 1
                e = N.FFAdamParam()
                e.param, e.grad = p.data_ptr(), p.grad.data_ptr()
                e.exp_avg, e.exp_avg_sq = st["exp_avg"].data_ptr(), st["exp_avg_sq"].data_ptr()
                sh = self._shadows.get(p)
                e.param_bf16 = sh.data_ptr() if sh is not None else None
                e.n, e.step, e.lr = p.numel(), int(st["step"].item()), float(group["lr"])
                by_hyper.setdefault(key, []).append(e)
        flags = N.FF_ADAM_ZERO_GRAD if self.fused_zero_grad else 0
        for (b1, b2, eps), entries in by_hyper.items():
            arr = (N.FFAdamParam * len(entries))(*entries)
            N.call("ff_adam_step", ctypes.cast(arr, ctypes.c_void_p), len(entries), b1, b2, eps, flags,
                   N.stream_ptr(), kernels=-(-len(entries) // 8))
        return loss

    def zero_grad(self, set_to_none=False):
        """With zero_grad=True the step already zeroed every gradient it updated."""
        if self.fused_zero_grad:
            return
        super().zero_grad(set_to_none=set_to_none)


def zero_grads(params):
    """Zero the gradients of `params` (those that have one; contiguous float32) in one
    ff_zero_f32 launch per 8 buffers instead of one fill per tensor."""
    bufs = [p.grad for p in params if p.grad is not None]
    if not bufs:
        return
    for b in bufs:
        if b.dtype != torch.float32 or not b.is_contiguous():
            raise ValueError("gradient buffers must be contiguous float32")
    ptrs = (ctypes.c_void_p * len(bufs))(*[b.data_ptr() for b in bufs])
    counts = (ctypes.c_int64 * len(bufs))(*[b.numel() for b in bufs])
    N.call("ff_zero_f32", ptrs, counts, len(bufs), N.stream_ptr(), kernels=-(-len(bufs) // 8))
