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

Device schedule (enable_device_schedule): the step count and the learning rates move to device
memory and step() runs ff_adam_step_scheduled, so that a training step including the update
can be captured in a CUDA graph and replayed with the current step and learning rates.
decay_lr() scales the learning rates on the device; sync_host() (also run by state_dict())
writes them and the step counts back into param_groups and state.
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

    def enable_device_schedule(self):
        """Move the step count and learning rates to device memory (creating the Adam state of
        every parameter that has a gradient). All those parameters must be at the same step.
        The parameter set is fixed from here on."""
        if getattr(self, "_dev", None) is not None:
            return
        entries, lrs, steps, dev = {}, [], set(), None
        for gi, group in enumerate(self.param_groups):
            b1, b2 = group["betas"]
            key = (float(b1), float(b2), float(group["eps"]))
            for p in group["params"]:
                if p.grad is None:
                    continue
                if p.dtype != torch.float32 or not p.is_contiguous() or not p.grad.is_contiguous():
                    raise ValueError("FusedAdam needs contiguous float32 parameters and gradients")
                dev = p.device
                st = self.state[p]
                if not st:
                    st["step"] = torch.tensor(0.0)
                    st["exp_avg"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                    st["exp_avg_sq"] = torch.zeros_like(p, memory_format=torch.preserve_format)
                steps.add(int(st["step"].item()))
                e = N.FFAdamParam()
                e.param, e.grad = p.data_ptr(), p.grad.data_ptr()
                e.exp_avg, e.exp_avg_sq = st["exp_avg"].data_ptr(), st["exp_avg_sq"].data_ptr()
                sh = self._shadows.get(p)
                e.param_bf16 = sh.data_ptr() if sh is not None else None
                e.n = p.numel()
                entries.setdefault(key, []).append((e, float(group["lr"]), gi, p))
        if len(steps) > 1:
            raise ValueError("the device schedule needs every parameter at the same step")
        if dev is None:
            raise ValueError("no parameter has a gradient")
        t = torch.tensor(steps.pop() if steps else 0, dtype=torch.int64, device=dev)
        calls = []
        for (b1, b2, eps), es in entries.items():
            lr = torch.tensor([lr_ for _, lr_, _, _ in es], dtype=torch.float64, device=dev)
            arr = (N.FFAdamParam * len(es))(*[e for e, _, _, _ in es])
            calls.append((arr, len(es), b1, b2, eps, lr, [(gi, p) for _, _, gi, p in es]))
        # every group's learning rate (groups without a gradient too), for sync_host
        glr = torch.tensor([float(g["lr"]) for g in self.param_groups], dtype=torch.float64, device=dev)
        self._dev = {"t": t, "calls": calls, "glr": glr}

    @property
    def device_schedule(self):
        return getattr(self, "_dev", None) is not None

    def decay_lr(self, factor):
        """lr *= factor in every group (on the device under the device schedule, in float64 as
        the host's Python floats)."""
        if self.device_schedule:
            for call in self._dev["calls"]:
                call[5].mul_(factor)
            self._dev["glr"].mul_(factor)
            return
        for g in self.param_groups:
            g["lr"] = g["lr"] * factor

    def sync_host(self):
        """Device schedule: copy the step count and learning rates into state and param_groups."""
        if not self.device_schedule:
            return
        t = int(self._dev["t"].item())
        for g, v in zip(self.param_groups, self._dev["glr"].cpu().tolist()):
            g["lr"] = v
        for arr, k, b1, b2, eps, lr, owners in self._dev["calls"]:
            for gi, p in owners:
                self.state[p]["step"] = torch.tensor(float(t))

    def state_dict(self):
        self.sync_host()
        return super().state_dict()

    def load_state_dict(self, state_dict):
        """Loads as torch's optimizers do; a device schedule is dropped (its step count and learning
        rates would be stale) and must be enabled again, which rebuilds it from the loaded state."""
        super().load_state_dict(state_dict)
        self._dev = None

    @torch.no_grad()
    def step(self, closure=None):
        loss = None
        if closure is not None:
            with torch.enable_grad():
                loss = closure()
        if self.device_schedule:  # no host reads: capturable
            d = self._dev
            d["t"].add_(1)
            flags = N.FF_ADAM_ZERO_GRAD if self.fused_zero_grad else 0
            for arr, k, b1, b2, eps, lr, _ in d["calls"]:
                N.call("ff_adam_step_scheduled", ctypes.cast(arr, ctypes.c_void_p), k, b1, b2, eps, flags,
                       N.ptr(lr), N.ptr(d["t"]), N.stream_ptr(), kernels=-(-k // 8))
            return loss
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
