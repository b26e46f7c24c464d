"""Field-fit training steps (the notebooks' regression loop, scripts/2D_regression.ipynb cell 4,
scripts/sdf_regression.ipynb cell 2) without autograd: explicit native launches per step."""
import ctypes
from collections import OrderedDict

import torch

from . import _native as N
from . import functional as FN


class RadianceFieldTrainer:
    """The per-scene radiance-field training loop (train_per_scene.py:147-175): render a batch of
    rays, MSE against the targets, backward, Adam with the reference's parameter groups
    (get_optparam_groups, lr_small / lr_large) and exponential lr decay to `decay_ratio` over
    n_iters (train_per_scene.py:118-125, 171-172)."""

    def __init__(self, model, n_samples=1024, lr_small=1e-3, lr_large=2e-2, n_iters=1000, decay_ratio=0.1,
                 white_bg=True, sampler=None, fused_adam=True):
        self.m, self.n_samples, self.white_bg = model, n_samples, white_bg
        groups = model.get_optparam_groups(lr_small, lr_large)
        if fused_adam:  # update + BF16 read copies + next step's zero_grad in one pass
            from .optim import FusedAdam
            self.opt = FusedAdam(groups, betas=(0.9, 0.99), shadows=model.bf16_shadows())
        else:
            self.opt = torch.optim.Adam(groups, betas=(0.9, 0.99))
        self.fused_adam = fused_adam
        self._grads_clean = False  # every gradient is known to be zero (a fused step zeroed them)
        self.lr_factor = decay_ratio ** (1.0 / max(n_iters, 1))
        self.sampler = sampler  # None: the plain uniform sampler; else a ProposalSampler
        self.jitter = None  # fixed per-ray sample jitter [R] for training renders; None: random per step

    def render(self, rays, is_train, static=False):
        if self.sampler is not None:
            return self.sampler.render(rays, is_train=is_train, white_bg=self.white_bg,
                                       jitter=self.jitter if is_train else None)
        rgb, depth, _ = self.m(rays, white_bg=self.white_bg, is_train=is_train, N_samples=self.n_samples,
                               jitter=self.jitter if is_train else None, static=static)
        return rgb, depth

    def _side_stream(self):
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream(device=self.m.basis_flat.device)
        return self._side

    def _zero_grads(self):
        """Every gradient of the field and the sampler, in one ff_zero_f32 launch."""
        from .optim import zero_grads
        params = [p for g in self.opt.param_groups for p in g["params"]]
        if self.sampler is not None:
            params += self.sampler.params
        zero_grads(params)

    def step(self, rays, rgb_gt, optimize=True, static=False):
        rgb, _ = self.render(rays, is_train=True, static=static)
        loss = torch.mean((rgb - rgb_gt) ** 2)
        if not self._grads_clean:
            self._zero_grads()
        self._grads_clean = False
        side = None
        if self.sampler is not None:
            # the proposal's loss and backward need only the forward's outputs: they run on a
            # second stream beside the field's backward (the field backward leaves room for them
            # on the SMs) and are joined before the update
            main = torch.cuda.current_stream()
            side = self._side_stream()
            side.wait_stream(main)
            with torch.cuda.stream(side):
                self.sampler.backward()
        loss.backward()
        if side is not None:
            torch.cuda.current_stream().wait_stream(side)
        if optimize:
            self._update()
        return loss.detach()

    def _update(self):
        """Adam on the field (lr decayed by lr_factor per step) and the proposal network."""
        self.opt.step()
        if self.fused_adam:
            self.opt.decay_lr(self.lr_factor)
        else:
            for g in self.opt.param_groups:
                g["lr"] = g["lr"] * self.lr_factor
        if self.sampler is not None:
            self.sampler.step()
        self._grads_clean = self.fused_adam and (self.sampler is None or self.sampler.fused_adam)

    def _schedules(self):
        """The optimizers' device schedules (what a captured update step reads; compared by identity)."""
        return (getattr(self.opt, "_dev", None),
                getattr(self.sampler.opt, "_dev", None) if self.sampler is not None else None)

    def _plain_step_static(self, rays, rgb_gt):
        """The plain sampler's fwd+bwd training step without autograd and without host reads
        (the body of its CUDA graph): gradients zeroed, static render forward, MSE, its gradient
        2 (rgb - gt) / (3 R), render backward into the .grad buffers. Returns the loss (device)."""
        from .renderer import render_job, sh_render_backward, sh_render_forward
        m = self.m
        if not self._grads_clean:
            self._zero_grads()
        self._grads_clean = False
        jitter = self.jitter if self.jitter is not None else torch.rand(rays.shape[0], device=rays.device)
        job = render_job(m, rays, self.n_samples, self.white_bg, True, True)
        rgb, _, saved = sh_render_forward(job, rays, jitter)
        diff = rgb - rgb_gt
        loss = torch.mean(diff * diff)
        sh_render_backward(job, jitter, saved, diff * (2.0 / diff.numel()))
        return loss

    def graph_step(self, rays, rgb_gt, optimize=False):
        """step(optimize) replayed from a CUDA graph. The batch is copied into static buffers;
        the capture covers the gradient zeroing, rendering, loss, the field backward and
        (proposal sampler) the proposal loss/backward, and with optimize=True the fused Adam
        updates of the field (with its learning-rate decay) and the proposal network. The plain
        sampler's step is captured as the explicit _plain_step_static (no autograd, no host reads:
        live-sample buffers sized for all n_rays * n_samples slots, the live count read on the
        device; fused BF16 path, SH-2 head). The per-ray jitter is drawn inside the graph (or
        self.jitter). Re-captured when the batch shape changes.

        optimize=True needs FusedAdam for the field and the proposal network (fused_adam=True):
        the optimizers switch to their device schedule (step counts and learning rates in device
        memory, FusedAdam.enable_device_schedule) at the first capture, and the update zeroes the
        gradients for the next replay. A load_state_dict of either optimizer (which drops its
        device schedule and replaces the moment buffers) makes the next call capture again. The
        captured decay multiplies by the lr_factor of capture time: after changing lr_factor, drop
        self._rgraphs."""
        static = self.sampler is None
        if optimize and not (self.fused_adam and (self.sampler is None or self.sampler.fused_adam)):
            raise ValueError("graph_step(optimize=True) needs fused_adam=True")
        key = (tuple(rays.shape), tuple(rgb_gt.shape), bool(optimize))
        graphs = self.__dict__.setdefault("_rgraphs", {})
        ent = graphs.get(key)
        if ent is not None and optimize and any(a is not b for a, b in zip(ent["sched"], self._schedules())):
            ent = None  # an optimizer dropped its device schedule (load_state_dict): capture again
        if ent is None:
            dev = self.m.basis_flat.device
            gr = torch.empty(rays.shape, dtype=torch.float32, device=dev)
            gg = torch.empty(rgb_gt.shape, dtype=torch.float32, device=dev)
            gr.copy_(rays)
            gg.copy_(rgb_gt)
            fwd_bwd = (lambda: self._plain_step_static(gr, gg)) if static else \
                (lambda: self.step(gr, gg, optimize=False))
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):  # warm-up (kernel attributes, workspaces) without updates
                for _ in range(2):
                    fwd_bwd()
            torch.cuda.current_stream().wait_stream(side)
            if optimize:
                self.opt.enable_device_schedule()
                if self.sampler is not None:
                    self.sampler.opt.enable_device_schedule()
                self._zero_grads()  # the warm-up's gradients; each replay's update zeroes its own
                self._grads_clean = True

                def body():
                    loss = fwd_bwd()
                    self._update()
                    return loss
            else:
                body = fwd_bwd
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                loss = body()
            # the captured body zeroes the gradients first unless an update leaves them clean
            ent = {"graph": graph, "loss": loss, "rays": gr, "gt": gg, "clean_after": bool(optimize),
                   "sched": self._schedules() if optimize else None}
            graphs[key] = ent
        self.m._read_buffers()
        if self.sampler is not None:
            self.sampler.grid_read()
        if optimize and not self._grads_clean:  # the captured update step does not zero first
            self._zero_grads()
        ent["rays"].copy_(rays, non_blocking=True)
        ent["gt"].copy_(rgb_gt, non_blocking=True)
        ent["graph"].replay()
        self._grads_clean = ent["clean_after"]
        return ent["loss"]

    @torch.no_grad()
    def psnr(self, rays, rgb_gt, chunk=16384):
        """Mean-squared-error PSNR (renderer.py:60) of the rendered rays against the targets."""
        err = 0.0
        for s in range(0, rays.shape[0], chunk):
            rgb, _ = self.render(rays[s:s + chunk], is_train=False)
            err += float(((rgb - rgb_gt[s:s + chunk]) ** 2).sum())
        mse = err / (rays.shape[0] * 3)
        return -10.0 * torch.log10(torch.tensor(mse)).item()


class FieldFitRunner:
    """One fwd+bwd regression step of a FactorFields model on (points, targets).

    fused=True: ONE ff_field_fit_step launch (gathers, BF16 tensor-core MLP, loss, backward,
    scatter) after zeroing the gradient buffers; binned=True (the default with fused) runs
    ff_field_fit_step_binned instead: the batch is binned by coefficient cell first so that the
    coefficient gradients of points sharing a cell are summed on chip. fused=False: the drop-in
    kernels launched one after the other (field fwd, MLP fwd, MLP bwd, field bwd) with the loss
    in PyTorch. Gradients land in the model's .grad buffers; step() returns the mean loss as a
    0-d device tensor (no host synchronisation).

    optimizer: a FusedAdam over the model's parameters (the notebooks' torch.optim.Adam), run by
    step(..., optimize=True) and graph_step(..., optimize=True) after the backward. With the
    binned path, FusedAdam(zero_grad=False) avoids a second zeroing: the step zeroes first."""

    def __init__(self, model, loss="l1", fused=True, binned=None, level0_shared=False, optimizer=None):
        if loss not in N.FF_LOSS:
            raise ValueError("loss must be 'l1' or 'mse'")
        self.m, self.loss, self.fused = model, loss, fused
        self.binned = fused if binned is None else bool(binned)
        if self.binned and not fused:
            raise ValueError("binned=True needs fused=True")
        # binned 2-D fits: level-0 basis gradients summed per block in shared memory
        # (FF_FIT_LEVEL0_SHARED; no effect where the kernel does not support it)
        self.level0_shared = bool(level0_shared)
        self._l0 = N.FF_FIT_LEVEL0_SHARED if self.level0_shared else 0
        self.opt = optimizer
        self._ws = None
        self._ws_gen = 0
        # the fused kernel's template arguments: mode, basis dim, coordinate dim, 8-wide output tiles
        out = model.linear_mat.out_dim
        dims = f"{model.in_dim},{model.geom.coord_dim},{1 if out == 1 else (2 if out <= 16 else 4)}"
        if fused and self.binned:
            self.path_name = ("fused, binned: one ff_field_fit_step_binned call per step (bin by coefficient cell "
                              "with the gradient zeroing, allocate cell ranges, permute, fit)")
            self.dominant_kernel = f"fused_field_mlp_kernel<3,{dims},bf16> (binned fit)"
            self.dominant_call = "ff_field_fit_step_binned"
            self.gathers_per_point = 1
        elif fused:
            self.path_name = "fused: one ff_field_fit_step launch per step (+ gradient zeroing)"
            self.dominant_kernel = f"fused_field_mlp_kernel<2,{dims},bf16> (fit)"
            self.dominant_call = "ff_field_fit_step"
            self.gathers_per_point = 1
        else:
            self.path_name = "explicit drop-in kernels (field fwd, MLP fwd, MLP bwd, field bwd)"
            self.dominant_kernel = "ff_field_backward"
            self.dominant_call = "ff_field_backward"
            self.gathers_per_point = 2
        for p in self._params():
            if p.grad is None:
                p.grad = torch.zeros_like(p)
        self.loss_buf = torch.zeros(1, device=model.basis_flat.device)

    def _params(self):
        ws, bs = self.m.linear_mat.weights()
        return [self.m.basis_flat, self.m.coeff_flat] + ws + [b for b in bs if b is not None]

    def _grad_struct(self):
        ws, bs = self.m.linear_mat.weights()
        g = N.FFMlpGrad()
        for i, (w, b) in enumerate(zip(ws, bs)):
            g.weight[i] = w.grad.data_ptr()
            g.bias[i] = b.grad.data_ptr() if b is not None else None
        return g

    def zero_grad(self, loss_buf=None):
        """Zero the parameters' gradients and the loss accumulator in one ff_zero_f32 launch."""
        bufs = [p.grad for p in self._params()] + [self.loss_buf if loss_buf is None else loss_buf]
        key = tuple(b.data_ptr() for b in bufs)
        if getattr(self, "_zero_key", None) != key:
            for b in bufs:
                if b.dtype != torch.float32 or not b.is_contiguous():
                    raise ValueError("gradient buffers must be contiguous float32")
            self._zero_ptrs = (ctypes.c_void_p * len(bufs))(*key)
            self._zero_counts = (ctypes.c_int64 * len(bufs))(*[b.numel() for b in bufs])
            self._zero_key = key
        N.call("ff_zero_f32", self._zero_ptrs, self._zero_counts, len(bufs), N.stream_ptr(),
               kernels=-(-len(bufs) // 8))

    _GRAPHS_KEPT = 8  # graphs per kind of input pair read in place (device, host; least recently used first out)

    def graph_step(self, x, y, optimize=False):
        """step() replayed from a CUDA graph, one host call for all its launches (the binning with
        the gradient zeroing, the fit kernel; the loss is the mean, accumulated by the kernel;
        with optimize=True the optimizer's update too, its step count and learning rates moved to
        device memory at the first capture: FusedAdam.enable_device_schedule).

        Device batches (contiguous float32 on the model's device) are read in place: a graph is
        captured per input buffer pair and kept (up to 8), so that a ring of batches resident in
        HBM replays without copies. Page-locked host batches (contiguous float32, pin_memory())
        get a graph per buffer pair too (up to 8), which holds the step's own host-to-device
        copies (FF_FIT_HOST_BATCH): the replay reads the host buffers' contents at that time. Any
        other batch (pageable host memory, other dtypes or strides) is copied into static
        buffers whose graph then replays. Graphs are re-captured when the batch shape, a parameter
        buffer or the binning workspace changes. The returned 0-d loss belongs to the replayed
        graph: the next replay of the same graph overwrites it."""
        key, kind = self._graph_key(x, y, optimize)
        graphs = self.__dict__.setdefault("_graphs", OrderedDict())
        ent = graphs.get(key)
        if ent is not None and (ent["ws_gen"] != self._ws_gen  # captured with a workspace since freed
                                or (optimize and ent["sched"] is not getattr(self.opt, "_dev", None))):
            del graphs[key]
            ent = None
        if ent is None:
            ent = self._capture(x, y, kind, optimize)
            graphs[key] = ent
            for k in [k for k, e in graphs.items() if e["ws_gen"] != self._ws_gen]:
                del graphs[k]
            self._evict(graphs, kind)
        graphs.move_to_end(key)
        self.m._read_buffers()  # refresh the BF16 grid copies in place if the masters changed
        if kind == "static":
            ent["x"].copy_(x, non_blocking=True)
            ent["y"].copy_(y, non_blocking=True)
        ent["graph"].replay()
        return ent["loss"]

    def capture_graphs(self, batches, optimize=False):
        """Capture (without replaying) the graphs graph_step will use for these (x, y) batches,
        e.g. a ring of batches resident in HBM, so that no step pays for a capture."""
        graphs = self.__dict__.setdefault("_graphs", OrderedDict())
        if len(batches) > self._GRAPHS_KEPT:
            raise ValueError(f"at most {self._GRAPHS_KEPT} batches keep their graphs")
        kinds = set()
        for x, y in batches:
            key, kind = self._graph_key(x, y, optimize)
            kinds.add(kind)
            if key not in graphs or graphs[key]["ws_gen"] != self._ws_gen:
                graphs[key] = self._capture(x, y, kind, optimize)
            graphs.move_to_end(key)
        for k in [k for k, e in graphs.items() if e["ws_gen"] != self._ws_gen]:
            del graphs[k]
        for kind in kinds:
            self._evict(graphs, kind)

    def _evict(self, graphs, kind):
        """Keep at most _GRAPHS_KEPT graphs of this kind (one for "static"), oldest out first."""
        cap = 1 if kind == "static" else self._GRAPHS_KEPT
        same = [k for k, e in graphs.items() if e["kind"] == kind]
        for k in same[:max(0, len(same) - cap)]:
            del graphs[k]

    def _host_batch(self, x, y):
        """FF_FIT_HOST_BATCH for a page-locked float32 host batch on the binned path, else 0
        (device batches; anything else on the host is refused)."""
        if x.device.type != "cpu" and y.device.type != "cpu":
            return 0
        if not (self.fused and self.binned):
            raise ValueError("host batches need the binned fused path; copy the batch to the device first")
        if not (x.device.type == y.device.type == "cpu" and x.dtype == y.dtype == torch.float32
                and x.is_contiguous() and y.is_contiguous() and x.is_pinned() and y.is_pinned()):
            raise ValueError("a host batch must be contiguous float32 in page-locked memory (tensor.pin_memory())")
        return N.FF_FIT_HOST_BATCH

    def _graph_key(self, x, y, optimize=False):
        """(key, kind): kind "device" reads a device batch in place, "host" copies a pinned host
        batch inside the graph (FF_FIT_HOST_BATCH), "static" copies anything else into static
        device buffers before the replay."""
        dev = self.m.basis_flat.device
        if (x.device == dev and y.device == dev and x.dtype == torch.float32 and y.dtype == torch.float32
                and x.is_contiguous() and y.is_contiguous()):
            kind, tag = "device", (x.data_ptr(), y.data_ptr())
        elif (self.fused and self.binned and x.device.type == y.device.type == "cpu"
              and x.dtype == y.dtype == torch.float32 and x.is_contiguous() and y.is_contiguous()
              and x.is_pinned() and y.is_pinned()):
            kind, tag = "host", ("host", x.data_ptr(), y.data_ptr())
        else:
            kind, tag = "static", ("static",)
        key = (tuple(x.shape), tuple(y.shape), self.m.basis_flat.data_ptr(), self.m.coeff_flat.data_ptr(),
               self.m.precision, bool(optimize)) + tag
        return key, kind

    def _capture(self, x, y, kind, optimize=False):
        dev = self.m.basis_flat.device
        if kind != "static":  # read in place: the device batch, or the host batch by the call's own copies
            xs, ys = x, y
        else:
            xs = torch.empty(x.shape, dtype=torch.float32, device=dev)
            ys = torch.empty(y.shape, dtype=torch.float32, device=dev)
            xs.copy_(x)
            ys.copy_(y)
        loss_buf = torch.zeros(1, device=dev)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.step(xs, ys, _loss_buf=loss_buf)  # warm-up outside the capture (kernel attributes, workspace)
        torch.cuda.current_stream().wait_stream(side)
        if optimize:
            if self.opt is None or not hasattr(self.opt, "enable_device_schedule"):
                raise ValueError("graph_step(optimize=True) needs FieldFitRunner(..., optimizer=FusedAdam(...))")
            self.opt.enable_device_schedule()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            loss = self.step(xs, ys, _loss_buf=loss_buf, optimize=optimize)
        return {"graph": graph, "loss": loss, "x": xs, "y": ys, "buf": loss_buf, "ws_gen": self._ws_gen,
                "kind": kind, "sched": getattr(self.opt, "_dev", None) if optimize else None}

    def _workspace(self, desc, n):
        """Device workspace of ff_field_fit_step_binned for n points, kept across steps."""
        need = int(N.lib().ff_field_fit_binned_workspace_bytes(ctypes.byref(desc), n, self.m.linear_mat.out_dim))
        if need < 0:
            N.check(need, "ff_field_fit_binned_workspace_bytes")
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.m.basis_flat.device)
            self._ws_gen += 1
        return self._ws

    def step(self, x, y, kernel_events=False, _loss_buf=None, optimize=False):
        """One step on (x, y): device tensors, or (binned path) page-locked host tensors that the
        call copies into its workspace itself (FF_FIT_HOST_BATCH). optimize=True: then the
        optimizer's update (not with kernel_events)."""
        if optimize and self.opt is None:
            raise ValueError("optimize=True needs FieldFitRunner(..., optimizer=FusedAdam(...))")
        loss = self._fwd_bwd(x, y, kernel_events, _loss_buf)
        if optimize and not kernel_events:
            self.opt.step()
        return loss

    def _fwd_bwd(self, x, y, kernel_events, _loss_buf):
        m = self.m
        host = self._host_batch(x, y)
        if not (self.fused and self.binned):  # the binned call zeroes them in its binning pass
            self.zero_grad(_loss_buf)
        basis_r, coeff_r, dt = m._read_buffers()
        desc = m.descriptor(dt)
        n = x.shape[0]
        ws, bs = m.linear_mat.weights()
        mlp = FN.mlp_struct(ws, bs, m.linear_mat.in_dim, m.linear_mat.hidden_dim, m.linear_mat.out_dim)
        st = N.stream_ptr()
        g = self._grad_struct()
        # kernel_events: CUDA events around the dominant kernel alone ("kernel": the fit kernel,
        # the binned call issued as its two halves; the drop-in path's field backward) and
        # around the whole call ("call"); kernel_events="call": one combined call, its events only
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)] if kernel_events else None
        split = bool(kernel_events) and kernel_events != "call"
        if self.fused:
            if self.binned:
                ws = self._workspace(desc, n)
            if ev:
                ev[0].record()
            lbuf = self.loss_buf if _loss_buf is None else _loss_buf
            scale = 1.0 / max(n * m.linear_mat.out_dim, 1)
            gb, gc = N.ptr(m.basis_flat.grad), N.ptr(m.coeff_flat.grad)
            xp, yp = (N.host_ptr(x), N.host_ptr(y)) if host else (N.ptr(x), N.ptr(y))
            if self.binned and split:  # the same launches as one ff_field_fit_step_binned call, in two calls
                N.call("ff_field_fit_bin", ctypes.byref(desc), ctypes.byref(mlp), xp, yp, n, N.ptr(lbuf),
                       gb, gc, ctypes.byref(g), N.FF_FIT_ZERO_GRADS | host, N.ptr(ws), ws.numel(), st)
                ev[1].record()
                N.call("ff_field_fit_step_on_bins", ctypes.byref(desc), N.ptr(basis_r), N.ptr(coeff_r),
                       ctypes.byref(mlp), n, N.FF_LOSS[self.loss], scale, N.ptr(lbuf), gb, gc, ctypes.byref(g),
                       N.FF_FIT_MEAN_LOSS | self._l0, N.ptr(ws), ws.numel(), st)
            else:
                if ev:
                    ev[1].record()
                common = (ctypes.byref(desc), N.ptr(basis_r), N.ptr(coeff_r), ctypes.byref(mlp), xp, yp,
                          n, N.FF_LOSS[self.loss], scale, N.ptr(lbuf), gb, gc, ctypes.byref(g))
                if self.binned:  # kernels: bin (+ gradient and loss zeroing), alloc, permute, fit (mean loss)
                    N.call("ff_field_fit_step_binned", *common,
                           N.FF_FIT_ZERO_GRADS | N.FF_FIT_MEAN_LOSS | self._l0 | host, N.ptr(ws), ws.numel(), st,
                           kernels=4)
                else:
                    N.call("ff_field_fit_step", *common, st)
            if ev:
                ev[2].record()
                return {"call": (ev[0], ev[2]), "kernel": (ev[1], ev[2]) if split else None}
            if self.binned:
                # the kernel accumulated the mean; a captured step returns its own buffer
                return lbuf[0] if _loss_buf is not None else lbuf[0].clone()
            return lbuf[0] / max(n * m.linear_mat.out_dim, 1)
        feats = torch.empty(n, m.n_feat, device=x.device)
        N.call("ff_field_forward", ctypes.byref(desc), N.ptr(basis_r), N.ptr(coeff_r), N.ptr(x), n, N.ptr(feats),
               None, None, st)
        pred = torch.empty(n, m.linear_mat.out_dim, device=x.device)
        N.call("ff_mlp_forward", ctypes.byref(mlp), N.ptr(feats), n, N.ptr(pred), st)
        err = pred - y
        if self.loss == "l1":
            loss = err.abs().mean()
            g_out = torch.sign(err) / err.numel()
        else:
            loss = (err * err).mean()
            g_out = 2 * err / err.numel()
        g_feats = torch.empty_like(feats)
        N.call("ff_mlp_backward", ctypes.byref(mlp), N.ptr(feats), n, N.ptr(g_out), N.ptr(g_feats), ctypes.byref(g), st)
        if ev:
            ev[0].record()
        N.call("ff_field_backward", ctypes.byref(desc), N.ptr(basis_r), N.ptr(coeff_r), N.ptr(x), n, N.ptr(g_feats),
               None, None, N.ptr(m.basis_flat.grad), N.ptr(m.coeff_flat.grad), st)
        if ev:
            ev[1].record()
            return {"call": (ev[0], ev[1]), "kernel": (ev[0], ev[1])}
        return loss
