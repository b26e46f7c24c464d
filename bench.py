"""Benchmark: fwd+bwd field samples/s on the 3-D SDF regression workload (262,144 points/step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

One step = one fwd+bwd pass of the field hot path over one batch: gradients zeroed, field
forward (mapping, basis + coefficient gathers, product, MLP head), L1 loss gradient, MLP
backward and the scatter of the grid gradients. Inputs (262,144 points + SDF targets) are
resident in HBM for `value`; `e2e` times the public API from pinned host buffers (H2D copy of
the batch and D2H of the loss inside the timed region). L2 is flushed (256 MB write) before
every timed step and each step is timed alone with CUDA events.

--impl reference times the reference's own CPU PyTorch op sequence (oracle/ref_torch.py) on
all host cores, on the same workload (262,144-point batches, K steps after W warm-up steps). Under torchrun each rank runs an
independent replica on its own GPU (the path shards by points: no collective on the data
path); `value` is the sum over ranks of points / max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "cfg1: 3-D SDF fit, 6-level grid basis [4,4,4,2,2,2] @ [32..128]^3, coeff 18x32^3, 2x64 ReLU head, L1"
N_POINTS = 262144
METRIC = "fwd+bwd field samples/s"


def bench_config(ws):
    """The workload both arms run (native and --impl reference): one dict, so the two JSON lines
    carry the same config."""
    return {"workload": WORKLOAD, "points_per_step": N_POINTS, "loss": "l1",
            "l2": "flushed (256 MB write) before every timed step (native arm)", "parallelism": f"replicas x{ws}"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) > 8:
                for nm, v in zip(names, r[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(buf):
    buf.zero_()


# The field-fit workloads measured (configurations 0, 1 and 4): points per step, loss, workload.
FIELD_CONFIGS = {
    "cfg1": {"points": 262144, "loss": "l1",
             "workload": WORKLOAD},
    "cfg0": {"points": 65536, "loss": "mse",
             "workload": "cfg0: 2-D image fit, 512x512x3 procedural image, 6-level grid basis [4,4,4,2,2,2] @ "
                         "[32..128]^2, coeff 18x271^2, 2x64 ReLU head to RGB, MSE"},
    "cfg4": {"points": 262144, "loss": "mse",
             "workload": "cfg4: image set, 256 procedural 256x256x3 images, shared 6-level 2-D basis, "
                         "per-image coeff 18x32^2 ([1,18,256,32,32]), 2x64 head, MSE"},
}


def field_batches(key, seed0, nb):
    """nb seeded batches (points, targets) of configuration `key`, generated on the host."""
    from factor_fields_gb300 import workloads as W
    n = FIELD_CONFIGS[key]["points"]
    if key == "cfg1":
        return [W.sdf_batch(seed0 + i, n) for i in range(nb)]
    if key == "cfg0":
        img = W.ProceduralImage(0, 512, 512)
        return [W.image_batch(seed0 + i, n, img=img) for i in range(nb)]
    return [W.image_set_batch(seed0 + i, n) for i in range(nb)]


def make_model(precision, key="cfg1"):
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    torch.manual_seed(0)
    m = FactorFields(W.field_cfg(key), device="cuda", precision=precision)
    if key == "cfg0":
        m.freq_bands = W.FREQ6
    g = torch.Generator(device="cpu").manual_seed(1)
    with torch.no_grad():  # a mid-training-like state: random coefficients
        for c in m.coeffs:
            c.copy_(torch.rand(c.shape, generator=g) * 2 - 1)
    return m


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one full-size launch of the fit
# kernel from the ncu captures summarised in profiles/fused_fit_kernel_cfg1_ncu.md.
NCU_TRAFFIC = {"fused_field_mlp_kernel<3,3,3,1,bf16> (binned fit)": 69.600256e6 + 1.299968e6,
               "fused_field_mlp_kernel<2,3,3,1,bf16> (fit)": 69.626112e6 + 1.560832e6}
# The binned fit kernel's L2-side work per 262,144-point launch (same capture): warp-level
# global red instructions (l1tex__t_requests_pipe_lsu_mem_global_op_red.sum) and L2 red requests
# (lts__t_requests_srcunit_tex_op_red.sum); and the rate of warp-wide float4 reds with one line
# per lane that a standalone probe sustained on this GPU, the ceiling those reds run against.
NCU_FIT_REDS = {"warp_reds": 791374, "l2_red_requests": 11301333}
PROBE_WARP_REDS_PER_S = 6.5e9


def bytes_per_point(m, gathers, param_bytes):
    """Algorithmic bytes per point: `gathers` passes over K corners x (sum C + C_coeff)
    channels at param_bytes, one float32 scatter of the same, coords + targets (4 B each).
    The fwd+bwd algorithm gathers twice (the backward re-reads the grid values it multiplies
    by): 2 G + S + IO = 2,320 B for the 3-D BF16 point (1,172 B for a 2-D point, 1,176 B for the
    image set's (x, y, image) point); the fused kernel keeps the values in registers and reads
    them once (1 G + S + IO = 1,744 B in 3-D)."""
    k = 2 ** m.in_dim
    ch = m.n_feat * 2
    return gathers * k * ch * param_bytes + k * ch * 4 + 4 * m.geom.coord_dim + 4 * m.linear_mat.out_dim


def max_over_ranks(vals):
    """Element-wise maximum of per-rank values over the process group (each rank's timed
    region; the slowest rank sets the job's time). Identity without a process group."""
    import torch.distributed as dist
    vals = [float(v) for v in vals]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vals
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor(vals, dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def whole_job_rate(points_per_rank_step, steps, world_size, ms_max):
    """Points of all ranks over the max-over-ranks time (points/s): every rank processes its
    own batches (replicas), so the job's rate is the sum of the ranks' work over the slowest
    rank's time."""
    return points_per_rank_step * steps * world_size / (ms_max / 1e3)


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def measure_field(key, args, ws, rank, local, flush, with_dropin):
    """One field-fit configuration (FIELD_CONFIGS): the fused BF16 binned step replayed from CUDA
    graphs over resident batches (value), the fit kernel alone under CUDA events (roofline), the
    public API from pinned host memory (e2e) and optionally the float32 drop-in path."""
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300 import train as T
    dev = torch.device("cuda", local)
    fc = FIELD_CONFIGS[key]
    n = fc["points"]
    nb = 8 if key != "cfg4" else 4  # distinct batches cycled through (seeded, generated on the host)
    batches = field_batches(key, 1000 * rank, nb)
    host = [(torch.from_numpy(x).pin_memory(), torch.from_numpy(y).pin_memory()) for x, y in batches]
    devb = [(x.to(dev), y.to(dev)) for x, y in host]
    m = make_model("bf16", key)
    runner = T.FieldFitRunner(m, loss=fc["loss"])
    stream = torch.cuda.current_stream()

    def timed(step_fn, k, with_kernel_events):
        times, ktimes = [], []
        for i in range(k):
            if with_kernel_events and ws == 1:
                # no host sync after the flush: the GPU is still busy (a ~1 ms spin, then the
                # 256 MB flush) while the host enqueues the step, so the kernel events see device
                # time, not enqueue gaps (on a slow host the flush alone did not cover the Python
                # between the two halves of the call)
                torch.cuda.synchronize()
                torch.cuda._sleep(2_000_000)
                flush_l2(flush)
            else:
                flush_l2(flush)
                torch.cuda.synchronize()
            if ws > 1:
                torch.distributed.barrier()
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            kev = step_fn(i)
            s1.record(stream)
            torch.cuda.synchronize()
            times.append(s0.elapsed_time(s1))
            if with_kernel_events and kev is not None:
                ktimes.append(kev[with_kernel_events][0].elapsed_time(kev[with_kernel_events][1]))
        return times, ktimes

    # launches of this library per step (the captured graph replays exactly these)
    N.reset_launch_count()
    runner.step(*devb[0])
    per_step = N.launch_count()
    # setup: one CUDA graph per resident batch (graph_step reads device batches in place)
    runner.capture_graphs(devb)
    for i in range(args.warmup):
        runner.graph_step(*devb[i % nb])
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    t_fast, _ = timed(lambda i: runner.graph_step(*devb[i % nb]), args.steps, False)
    # the dominant kernel alone, CUDA events around its launch on the launching stream
    _, k_fast = timed(lambda i: runner.step(*devb[i % nb], kernel_events=True), args.steps, "kernel")
    ck = clocks.stop()
    ms = float(np.sum(t_fast))

    # end to end through the public API from pinned host memory
    loss_host = torch.empty(1, pin_memory=True)

    def e2e_step(i):
        x, y = host[i % nb]
        # one replay per step: the captured call copies the pinned host batch into its workspace
        # (FF_FIT_HOST_BATCH) before the binning; then the loss is read back to pinned host memory
        loss = runner.graph_step(x, y)
        loss_host.copy_(loss.reshape(1), non_blocking=True)
        return None

    runner.capture_graphs(host)  # setup: one graph per pinned host batch, as for the device ring
    for i in range(args.warmup):
        e2e_step(i)
    t_e2e, _ = timed(e2e_step, args.steps, False)

    # the notebooks' whole training step: the same graph-replayed fit with the fused Adam update
    # (lr 1e-2) captured after it (FusedAdam's device schedule; it moves the parameters)
    from factor_fields_gb300.optim import FusedAdam
    opt = FusedAdam(m.parameters(), lr=1e-2, zero_grad=False, shadows=m.bf16_shadows())
    trainer = T.FieldFitRunner(m, loss=fc["loss"], optimizer=opt)
    trainer.capture_graphs(devb, optimize=True)
    for i in range(args.warmup):
        trainer.graph_step(*devb[i % nb], optimize=True)
    t_adam, _ = timed(lambda i: trainer.graph_step(*devb[i % nb], optimize=True), args.steps, False)

    ms_drop = None
    if with_dropin:  # the float32 drop-in path (autograd through get_coding / linear_mat)
        md = make_model("fp32", key)

        def dropin_step(i):
            x, y = devb[i % nb]
            md.zero_grad(set_to_none=True)
            feats, _ = md.get_coding(x)
            pred = md.linear_mat(feats)
            err = pred - y
            (err.abs().mean() if fc["loss"] == "l1" else (err * err).mean()).backward()
            return None

        for i in range(args.warmup):
            dropin_step(i)
        t_drop, _ = timed(dropin_step, args.steps, False)
        ms_drop = float(np.sum(t_drop))

    vals = max_over_ranks([ms, float(np.sum(t_e2e)), float(np.sum(t_adam))] + ([ms_drop] if with_dropin else []))
    ms, ms_e2e, ms_adam = vals[0], vals[1], vals[2]
    pts = n * args.steps * ws
    kern_ms = float(np.mean(k_fast)) if k_fast else None  # the fit kernel alone
    # the whole ff_field_fit_step_binned call (binning with the gradient zeroing + the fit kernel):
    # the graph-replayed step is exactly that call, so its time is the step's
    call_ms = ms / args.steps
    bpp = bytes_per_point(m, 2, 2)  # the fwd+bwd algorithm's bytes (BF16 grids)
    bpp_read_once = bytes_per_point(m, 1, 2)  # what the fused kernel reads and writes
    peaks = load_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = (bpp * n) / (kern_ms / 1e3) / 1e9 if kern_ms else None
    achieved_call = (bpp * n) / (call_ms / 1e3) / 1e9 if call_ms else None
    xin, yin = host[0]
    out = {
        "workload": fc["workload"], "points_per_step": n, "loss": fc["loss"],
        "value": whole_job_rate(n, args.steps, ws, ms), "unit": "samples/s", "ms_per_step": ms / args.steps,
        "path": runner.path_name,
        "e2e": {"value": pts / (ms_e2e / 1e3), "unit": "samples/s",
                "h2d_bytes_per_step": int(xin.numel() * 4 + yin.numel() * 4), "d2h_bytes_per_step": 4},
        "roofline": {"bound": "hbm", "kernel": runner.dominant_kernel, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "bytes_per_point": bpp, "bytes_per_point_read_once": bpp_read_once,
                     "frac_read_once": (achieved * bpp_read_once / bpp / peak) if achieved else None,
                     "kernel_ms": kern_ms, "call": runner.dominant_call, "call_ms": call_ms,
                     "call_frac": (achieved_call / peak) if achieved_call else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback"},
        "gpu_launches": per_step * args.steps,
        "clocks": ck,
        # the notebooks' training step (fit + Adam), resident batches, L2 flushed per step as above
        "train_with_adam": {"mode": "CUDA graph replay: binned fit + fused Adam (lr 1e-2, device schedule)",
                            "value": pts / (ms_adam / 1e3), "unit": "samples/s", "ms_per_step": ms_adam / args.steps},
    }
    if with_dropin:
        out["fp32_dropin"] = {"value": pts / (vals[3] / 1e3), "unit": "samples/s", "ms_per_step": vals[3] / args.steps}
    return out, m


def run_native(args, ws, rank, local):
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    r1, _ = measure_field("cfg1", args, ws, rank, local, flush, with_dropin=True)
    roof = dict(r1["roofline"])
    roof["traffic"] = NCU_TRAFFIC.get(roof["kernel"])
    roof["traffic_source"] = ("ncu dram read+write of the fit kernel, one 262,144-point launch "
                              "(profiles/fused_fit_kernel_cfg1_ncu.md)")
    if roof.get("kernel_ms") and roof["kernel"] in NCU_TRAFFIC and "<3,3,3,1" in roof["kernel"]:
        # the L2-side fraction: warp-level gradient reds per second against the probe's rate
        rate = NCU_FIT_REDS["warp_reds"] / (roof["kernel_ms"] / 1e3)
        roof["l2_reds"] = {"warp_reds_per_launch": NCU_FIT_REDS["warp_reds"],
                           "l2_red_requests_per_point": NCU_FIT_REDS["l2_red_requests"] / N_POINTS,
                           "achieved_warp_reds_per_s": rate, "peak_warp_reds_per_s": PROBE_WARP_REDS_PER_S,
                           "frac": rate / PROBE_WARP_REDS_PER_S,
                           "source": "ncu counts of one launch (profiles/fused_fit_kernel_cfg1_ncu.md) over the "
                                     "event time of the kernel; peak = a warp-wide float4 red probe, one line "
                                     "per lane"}
    res = {
        "metric": METRIC, "value": r1["value"], "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r1["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 storage, fp32 accumulation",
        "data": "synthetic (seeded analytic SDF: 16 spheres + 8 boxes)",
        "config": bench_config(ws), "path": r1["path"],
        "e2e": r1["e2e"], "fp32_dropin": r1["fp32_dropin"], "roofline": roof,
        "gpu_launches": r1["gpu_launches"], "clocks": r1["clocks"], "train_with_adam": r1["train_with_adam"],
    }
    if not args.no_field_configs:
        # the 2-D configurations: the image fit and the image set (shared basis, per-image coefficients)
        res["field_configs"] = {}
        for key in ("cfg0", "cfg4"):
            r, mk = measure_field(key, args, ws, rank, local, flush, with_dropin=True)
            if rank == 0 and not args.no_cpu_baseline:
                r["cpu_baseline"] = run_cpu_baseline_model(mk, key, 3)
            res["field_configs"][key] = r
    return res


def _train_radiance(kind, seed, iters, pool, gt, dev):
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.proposal import ProposalSampler
    from factor_fields_gb300.train import RadianceFieldTrainer
    torch.manual_seed(seed)
    m = FactorFields(W.field_cfg("cfg2"), device=dev, precision="bf16")
    sampler = ProposalSampler(m, seed=seed) if kind == "cfg3_proposal" else None
    tr = RadianceFieldTrainer(m, n_samples=1024, n_iters=iters, sampler=sampler)
    g = torch.Generator(device=dev).manual_seed(seed)
    for it in range(iters):
        idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
        tr.step(pool[idx], gt[idx])
        if sampler is None and it in (iters // 5, iters // 2):
            m.updateAlphaMask((128, 128, 128), is_update_alphaMask=True, times=1)
    return m, sampler, tr, g


def measure_radiance_field_kernels(m, rays, dev, flush, steps, warmup, seed=3):
    """The fused field + 18->64->28 head kernels alone (ff_field_mlp_forward / _backward) and the
    compositing kernels (ff_composite_forward / _backward) on the live samples of one 4,096-ray
    plain-sampler batch (ray order, as the render calls them), each launch bracketed by CUDA events
    on its stream after an L2 flush. The backward's contract bytes
    per sample are those of the field backward (two BF16 gathers of the 8 corners x 36 channels,
    one float32 scatter, coordinates and dL/dout: 2,428 B); the forward's one gather plus the
    coordinates and outputs (700 B)."""
    import ctypes
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300 import functional as FN
    from factor_fields_gb300.renderer import march, render_desc
    g = torch.Generator(device=dev).manual_seed(seed)
    jit = torch.rand(rays.shape[0], device=dev, generator=g)
    rdesc = render_desc(m, 1024, True)
    with torch.no_grad():
        offs, xyz, sidx = march(m, rays, jit, rdesc)
    n = xyz.shape[0]
    lm = m.linear_mat
    ws, bs = lm.weights()
    mlp = FN.mlp_struct(ws, bs, lm.in_dim, lm.hidden_dim, lm.out_dim)
    basis_r, coeff_r, dt = m._read_buffers()
    fdesc = m.descriptor(dt)
    out = torch.empty(n, lm.out_dim, device=dev)
    g_out = torch.randn(n, lm.out_dim, device=dev, generator=g) * 1e-3
    gb, gc = torch.zeros_like(m.basis_flat), torch.zeros_like(m.coeff_flat)  # scratch gradients
    gw = [torch.zeros_like(w) for w in ws]
    gbias = [torch.zeros_like(b) if b is not None else None for b in bs]
    grad = N.FFMlpGrad()
    for i in range(len(ws)):
        grad.weight[i] = gw[i].data_ptr()
        grad.bias[i] = gbias[i].data_ptr() if gbias[i] is not None else None
    stream = torch.cuda.current_stream()
    st = N.stream_ptr()

    def fwd():
        N.call("ff_field_mlp_forward", ctypes.byref(fdesc), N.ptr(basis_r), N.ptr(coeff_r), ctypes.byref(mlp),
               N.ptr(xyz), n, N.ptr(out), st)

    def bwd():
        N.call("ff_field_mlp_backward", ctypes.byref(fdesc), N.ptr(basis_r), N.ptr(coeff_r), ctypes.byref(mlp),
               N.ptr(xyz), n, N.ptr(g_out), N.ptr(gb), N.ptr(gc), ctypes.byref(grad), st)

    def timed(fn):
        for _ in range(warmup):
            fn()
        ts = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            torch.cuda._sleep(2_000_000)  # the GPU spins (~1 ms) while the host enqueues: no launch gap timed
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    fwd_ms, bwd_ms = timed(fwd), timed(bwd)
    # the compositing kernels on the same samples (the field's outputs as their feature rows)
    fwd()
    n_rays = rays.shape[0]
    rgb = torch.empty(n_rays, 3, device=dev)
    depth = torch.empty(n_rays, device=dev)
    g_rgb = torch.randn(n_rays, 3, device=dev, generator=g) * 1e-3
    g_feat = torch.empty_like(out)

    def comp_fwd():
        N.call("ff_composite_forward", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jit), n_rays, N.ptr(offs),
               N.ptr(sidx), N.ptr(out), out.shape[1], None, N.ptr(rgb), N.ptr(depth), None, st)

    def comp_bwd():
        N.call("ff_composite_backward", ctypes.byref(rdesc), N.ptr(rays), N.ptr(jit), n_rays, N.ptr(offs),
               N.ptr(sidx), N.ptr(out), out.shape[1], None, N.ptr(g_rgb), N.ptr(g_feat), st)

    cf_ms, cb_ms = timed(comp_fwd), timed(comp_bwd)
    k, ch = 2 ** m.in_dim, m.n_feat * 2
    io = 4 * m.geom.coord_dim + 4 * lm.out_dim
    b_bwd = bytes_per_point(m, 2, 2)
    b_fwd = k * ch * 2 + io
    peaks = load_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    ach = b_bwd * n / (bwd_ms / 1e3) / 1e9
    ach_f = b_fwd * n / (fwd_ms / 1e3) / 1e9
    counts = (offs[1:] - offs[:-1]).float()
    return {"samples": n, "fwd_ms": fwd_ms, "bwd_ms": bwd_ms,
            "composite": {"fwd_ms": cf_ms, "bwd_ms": cb_ms, "rays": n_rays,
                          "live_samples_per_ray": {"mean": float(counts.mean()), "max": float(counts.max())},
                          # forward: the 28-float row + the sample index; backward: the row and the
                          # index, 8 parked floats written and read back, the 28-float gradient row
                          "bytes_per_sample": {"fwd": 28 * 4 + 4, "bwd": 28 * 4 + 4 + 2 * 32 + 28 * 4}},
            "roofline": {"bound": "hbm", "kernel": "fused_field_mlp_kernel<1,3,3,4,bf16> (field backward, 28-wide head)",
                         "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "bytes_per_sample": b_bwd,
                         "fwd_kernel": "fused_field_mlp_kernel<0,3,3,4,bf16>", "fwd_achieved": ach_f,
                         "fwd_frac": ach_f / peak, "fwd_bytes_per_sample": b_fwd,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback",
                         "l2": "flushed (256 MB write) before every timed launch"}}


def measure_adam(opt, steps, warmup):
    """The fused Adam update (ff_adam_step) over an optimizer's parameters alone: CUDA events
    around 5 back-to-back updates (entries built beforehand; the ~0.5 GB working set of the
    configuration-2 model is larger than L2), against the HBM roofline with 32 algorithmic bytes
    per element (param, grad, both moments: read and written; the gradient zeroed) + 2 for each
    element with a BF16 read copy."""
    import ctypes
    from factor_fields_gb300 import _native as N
    opt.step()  # the moments exist
    by_hyper, n, n_sh = {}, 0, 0
    for group in opt.param_groups:
        b1, b2 = group["betas"]
        for p in group["params"]:
            if p.grad is None:
                continue
            st = opt.state[p]
            e = N.FFAdamParam()
            e.param, e.grad = p.data_ptr(), p.grad.data_ptr()
            e.exp_avg, e.exp_avg_sq = st["exp_avg"].data_ptr(), st["exp_avg_sq"].data_ptr()
            sh = getattr(opt, "_shadows", {}).get(p)
            e.param_bf16 = sh.data_ptr() if sh is not None else None
            e.n, e.step, e.lr = p.numel(), int(st["step"].item()) + 1, float(group["lr"])
            by_hyper.setdefault((float(b1), float(b2), float(group["eps"])), []).append(e)
            n += p.numel()
            n_sh += p.numel() if sh is not None else 0
    calls = [((N.FFAdamParam * len(es))(*es), len(es), hyper) for hyper, es in by_hyper.items()]

    def launch():
        for arr, k, (b1, b2, eps) in calls:
            N.call("ff_adam_step", ctypes.cast(arr, ctypes.c_void_p), k, b1, b2, eps, N.FF_ADAM_ZERO_GRAD,
                   N.stream_ptr(), kernels=-(-k // 8))

    for _ in range(warmup):
        launch()
    ts = []
    for _ in range(steps):
        torch.cuda.synchronize()
        torch.cuda._sleep(2_000_000)  # the GPU stays busy while the host enqueues the five updates
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            launch()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 5)
    ms = float(np.median(ts))
    nbytes = 32 * n + 2 * n_sh
    peaks = load_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = nbytes / (ms / 1e3) / 1e9
    return {"ms": ms, "elements": n, "elements_with_bf16_copy": n_sh, "bytes_per_step": nbytes,
            "roofline": {"bound": "hbm", "kernel": "adam_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "l2": "working set larger than L2 (not flushed)",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback"}}


def run_radiance(args, dev):
    """Configurations 2 and 3 on the synthetic blob scene: rays/s of one fwd+bwd training step
    (plain sampler: 4,096 rays x up to 1,024 samples with 128^3 occupancy-bitfield pruning;
    proposal sampler: 8,192 rays x 48 stratified training samples + the proposal network's
    training), and PSNR / depth error against the FP64 quadrature ground truth after equal
    training (iters x 4,096 rays, Adam; the proposal configuration renders with 48 samples
    drawn from the network). The PSNR comparison is repeated on seeds 1 and 2 (training alone)
    because single runs differ by up to ~0.5 dB, more for an unlucky seed."""
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.renderer import march, render_desc
    scene = W.BlobScene(0)
    pool = torch.from_numpy(scene.ray_pool(1 << 18, 5)).float()
    gt = scene.render_gt(pool.double().numpy(), n_steps=512).to(dev)
    test = torch.from_numpy(scene.ray_pool(1 << 14, 6, views=[0, 1, 2])).float()
    gtt, gtd = scene.render_gt(test.double().numpy(), n_steps=512, with_depth=True)
    pool, test, gtt, gtd = pool.to(dev), test.to(dev), gtt.to(dev), gtd.to(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    eval_ds = scene.test_dataset([7], width=400, height=400, n_steps=512)  # one full 400x400 test view
    iters = args.render_iters
    out = {}
    for kind, batch in (("cfg2_plain", 4096), ("cfg3_proposal", 8192)):
        m, sampler, tr, g = _train_radiance(kind, 0, iters, pool, gt, dev)
        psnr = tr.psnr(test, gtt)
        with torch.no_grad():
            dep = torch.cat([tr.render(test[s:s + 16384], is_train=False)[1] for s in range(0, test.shape[0], 16384)])
        depth_err = float((dep - gtd).abs().mean())
        # timed fwd+bwd steps (no optimizer step), both samplers replayed from CUDA graphs: the
        # proposal path has a fixed sample count; the plain sampler renders without host
        # synchronisation (live-sample buffers for every sample slot, the count on the device)

        def timed_steps(b):
            for _ in range(args.warmup):
                idx = torch.randint(0, pool.shape[0], (b,), device=dev, generator=g)
                tr.graph_step(pool[idx], gt[idx])
            times = []
            for _ in range(args.steps):
                idx = torch.randint(0, pool.shape[0], (b,), device=dev, generator=g)
                rb, gb = pool[idx], gt[idx]
                flush.zero_()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                tr.graph_step(rb, gb)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            return float(np.mean(times))

        ms = timed_steps(batch)
        ms_8192 = timed_steps(8192) if batch != 8192 else ms
        # a whole training step (fwd + bwd + the fused Adam update of field and proposal) at the
        # training batch, after the measurements above
        ttimes = []
        for i in range(args.steps):
            idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
            rb, gb = pool[idx], gt[idx]
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            tr.step(rb, gb)
            e1.record()
            torch.cuda.synchronize()
            ttimes.append(e0.elapsed_time(e1))
        tms = float(np.mean(ttimes))
        # the evaluation renderer on a whole 400x400 image (one pass, metrics on the GPU)
        from factor_fields_gb300.renderer import evaluation
        evaluation(eval_ds, m, N_vis=-1, N_samples=1024, white_bg=True, sampler=sampler)  # warm-up
        e_psnr, e_extra = evaluation(eval_ds, m, N_vis=-1, N_samples=1024, white_bg=True, sampler=sampler)
        rec = {"rays_per_s": batch / (ms / 1e3), "ms_per_step": ms, "rays_per_step": batch,
               "rays_per_s_at_8192": 8192 / (ms_8192 / 1e3), "mode": "CUDA graph replay, fwd+bwd",
               "psnr_db": psnr, "depth_mae": depth_err, "train_steps": iters, "train_rays_per_step": 4096,
               "train_step_ms_with_adam": tms, "train_rays_per_s_with_adam": 4096 / (tms / 1e3),
               "eval_400x400": {"ms_per_image": e_extra["ms_per_image"][0], "psnr_db": e_psnr[0],
                                "ssim": e_extra["ssim"][0],
                                "rays_per_s": 400 * 400 / (e_extra["ms_per_image"][0] / 1e3)}}
        if sampler is not None:
            # the same with 32 render samples per ray (the configuration resamples 48)
            sampler.render_fine = 32
            evaluation(eval_ds, m, N_vis=-1, N_samples=1024, white_bg=True, sampler=sampler)  # warm-up
            p32, x32 = evaluation(eval_ds, m, N_vis=-1, N_samples=1024, white_bg=True, sampler=sampler)
            with torch.no_grad():
                dep32 = torch.cat([tr.render(test[s0:s0 + 16384], is_train=False)[1]
                                   for s0 in range(0, test.shape[0], 16384)])
            rec["render_32"] = {"psnr_db": tr.psnr(test, gtt), "samples_per_ray": 32,
                                "depth_mae": float((dep32 - gtd).abs().mean()),
                                "eval_400x400": {"ms_per_image": x32["ms_per_image"][0], "psnr_db": p32[0],
                                                 "ssim": x32["ssim"][0],
                                                 "rays_per_s": 400 * 400 / (x32["ms_per_image"][0] / 1e3)}}
            sampler.render_fine = sampler.n_fine
        # the whole training step (fwd + bwd + the fused Adam updates) replayed from one CUDA
        # graph (FusedAdam's device schedule), at the training batch: the eager step above is
        # bound by the host issuing its launches
        gtimes = []
        for i in range(max(args.warmup, 3) + args.steps):
            idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
            rb, gb = pool[idx], gt[idx]
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            tr.graph_step(rb, gb, optimize=True)
            e1.record()
            torch.cuda.synchronize()
            if i >= max(args.warmup, 3):
                gtimes.append(e0.elapsed_time(e1))
        gms = float(np.mean(gtimes))
        rec["train_step_ms_with_adam_graph"] = gms
        rec["train_rays_per_s_with_adam_graph"] = 4096 / (gms / 1e3)
        if sampler is None and not args.no_cpu_baseline:
            rec["cpu_baseline"] = run_cpu_baseline_render(m, pool, gt)
            rec["rays_per_s_vs_cpu_baseline"] = rec["rays_per_s"] / rec["cpu_baseline"]["value"]
        if sampler is None:
            offs, _, _ = march(m, test, None, render_desc(m, 1024, True))
            rec["live_samples_per_ray"] = float(offs[-1]) / test.shape[0]
            rec["max_samples_per_ray"] = 1024
            idx = torch.randint(0, pool.shape[0], (batch,), device=dev, generator=g)
            rec["field_kernels"] = measure_radiance_field_kernels(m, pool[idx], dev, flush, args.steps,
                                                                  max(args.warmup, 3))
            # the optimizer update of the same model (last: it moves the parameters one step)
            rec["adam"] = measure_adam(tr.opt, args.steps, max(args.warmup, 3))
        else:
            rec["samples_per_ray"] = sampler.n_fine
        out[kind] = rec
    out["proposal_rays_per_s_vs_plain"] = out["cfg3_proposal"]["rays_per_s"] / out["cfg2_plain"]["rays_per_s"]
    # whole training steps with the optimizer, both from CUDA graphs, 4,096 rays each
    out["proposal_train_rays_per_s_vs_plain_with_adam_graph"] = (
        out["cfg3_proposal"]["train_rays_per_s_with_adam_graph"] / out["cfg2_plain"]["train_rays_per_s_with_adam_graph"])
    # like for like: both samplers at 8,192 rays per step, both replayed from CUDA graphs
    out["proposal_rays_per_s_vs_plain_same_batch"] = (out["cfg3_proposal"]["rays_per_s_at_8192"] /
                                                      out["cfg2_plain"]["rays_per_s_at_8192"])
    # rendering alone (the evaluation renderer, no backward): 48 proposal samples per ray
    # against the plain sampler's ~125 live samples after occupancy pruning
    out["proposal_eval_rays_per_s_vs_plain"] = (out["cfg3_proposal"]["eval_400x400"]["rays_per_s"] /
                                                out["cfg2_plain"]["eval_400x400"]["rays_per_s"])
    out["proposal_eval_rays_per_s_vs_plain_32"] = (out["cfg3_proposal"]["render_32"]["eval_400x400"]["rays_per_s"] /
                                                   out["cfg2_plain"]["eval_400x400"]["rays_per_s"])
    seeds = {0: {"cfg2_plain": out["cfg2_plain"]["psnr_db"], "cfg3_proposal": out["cfg3_proposal"]["psnr_db"],
                 "cfg3_proposal_32": out["cfg3_proposal"]["render_32"]["psnr_db"]}}
    if args.psnr_seeds > 1:
        for seed in range(1, args.psnr_seeds):
            seeds[seed] = {"cfg2_plain": _train_radiance("cfg2_plain", seed, iters, pool, gt, dev)[2].psnr(test, gtt)}
            _, sam, trp, _ = _train_radiance("cfg3_proposal", seed, iters, pool, gt, dev)
            seeds[seed]["cfg3_proposal"] = trp.psnr(test, gtt)
            sam.render_fine = 32
            seeds[seed]["cfg3_proposal_32"] = trp.psnr(test, gtt)
    diffs = [v["cfg3_proposal"] - v["cfg2_plain"] for v in seeds.values()]
    diffs32 = [v["cfg3_proposal_32"] - v["cfg2_plain"] for v in seeds.values()]
    out["psnr_db_by_seed"] = {str(k): v for k, v in seeds.items()}
    out["proposal_psnr_minus_plain_db"] = float(np.mean(diffs))
    out["proposal_psnr_minus_plain_db_by_seed"] = diffs
    out["proposal_32_psnr_minus_plain_db_by_seed"] = diffs32
    # the target for the learned sampler: rendering within 0.1 dB of the plain sampler's PSNR (3-view
    # test set, each seed) at >= 3x its rays/s (a full 400x400 image through the evaluation renderer)
    r32, r48 = out["proposal_eval_rays_per_s_vs_plain_32"], out["proposal_eval_rays_per_s_vs_plain"]
    out["proposal_target"] = {
        "target": "PSNR within 0.1 dB of the plain sampler at >= 3x its rays/s",
        "render_samples_32": {"rays_per_s_vs_plain": r32, "psnr_minus_plain_db_by_seed": diffs32,
                              "depth_mae": out["cfg3_proposal"]["render_32"]["depth_mae"],
                              "met": bool(r32 >= 3.0 and min(diffs32) >= -0.1)},
        "render_samples_48": {"rays_per_s_vs_plain": r48, "psnr_minus_plain_db_by_seed": diffs,
                              "depth_mae": out["cfg3_proposal"]["depth_mae"],
                              "met": bool(r48 >= 3.0 and min(diffs) >= -0.1)},
        "plain_depth_mae": out["cfg2_plain"]["depth_mae"],
    }
    out["scene"] = "seeded 32 Gaussian density blobs in [-1.5,1.5]^3, 100 views 400x400 focal 555, white bg"
    return out


def _cpu_reference_field():
    """The reference's CPU op sequence (oracle/ref_torch.py) holding configuration 1's initial
    state (DCT basis, seeded random coefficients, a seeded MLP head) and all host threads."""
    from factor_fields_gb300 import workloads as W
    from oracle.ref_torch import RefField
    from factor_fields_gb300.config import FieldGeometry
    from factor_fields_gb300.field import dct_dict
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    cfg = W.field_cfg("cfg1")
    g = FieldGeometry(cfg)
    levels = [dct_dict(int(np.power(c, 1.0 / 3) + 1), r, c, 3).reshape([1, c] + [r] * 3)
              for c, r in zip(g.basis_dims, g.basis_reso)]
    gen = torch.Generator().manual_seed(1)
    coeff = torch.rand([1, 18] + g.coeff_reso, generator=gen) * 2 - 1
    torch.manual_seed(0)
    l0, l1 = torch.nn.Linear(18, 64), torch.nn.Linear(64, 1, bias=False)
    r = RefField("reconstruction", cfg.dataset.aabb, levels, coeff, [l0.weight.detach(), l1.weight.detach()],
                 [l0.bias.detach(), None], g.freq_bands, "sawtooth")
    return r, cores


CPU_KIND = "port"
CPU_DESC = ("torch CPU restatement of the reference's grid_sample/MLPMixer op sequence (oracle/ref_torch.py, "
            "pinned to outputs of the reference itself)")


def run_cpu_baseline(n_points, steps, warmup=1):
    """The reference's CPU op sequence on a bounded sample of the workload: samples/s (best step)."""
    from factor_fields_gb300 import workloads as W
    r, cores = _cpu_reference_field()
    x, y = W.sdf_batch(7, n_points)
    x, y = torch.from_numpy(x), torch.from_numpy(y)
    for _ in range(warmup):
        r.fit_step(x, y)
    best = []
    for _ in range(steps):
        t0 = time.perf_counter()
        r.fit_step(x, y)
        best.append(time.perf_counter() - t0)
    t = min(best)
    return {"value": n_points / t, "unit": "samples/s", "cores": cores, "kind": CPU_KIND,
            "sample": f"{n_points} points of the same workload per step, best of {steps} after {warmup} warm-up "
                      f"({CPU_DESC})"}


def head_flops_per_sample(c, hidden=128, view_pe=6, fea_pe=2):
    """Algorithmic FLOPs of MLPRender_Fea per head sample (models/FactorFields.py:162-203), forward
    and backward as autograd computes them (no recomputation counted): forward 2 (in H + H H + 3 H);
    backward dW0, dX (2 in H each), dW1, dH0 (2 H H each), dW2, dH1 (2 3 H each)."""
    i = 3 + c + 6 * view_pe + 2 * fea_pe * c
    fwd = 2 * (i * hidden + hidden * hidden + hidden * 3)
    bwd = 2 * (2 * i * hidden + 2 * hidden * hidden + 2 * 3 * hidden)
    return fwd, bwd


def measure_mlp_head(args, dev, flush):
    """The MLPRender_Fea colour head (the reference's head, nerf.yaml sizes with model.out_dim 28:
    27 feature channels, 174 inputs, 128 hidden): the tcgen05 kernels timed alone on 262,144 head
    samples (CUDA events, forward and backward), as TFLOP/s of the algorithmic FLOPs against the
    measured BF16 tensor peak; and a configuration-2 fwd+bwd step (4,096 rays) with this head."""
    from factor_fields_gb300 import FactorFields
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300.renderer import MLPRender_Fea, head_backward, head_forward
    torch.manual_seed(0)
    head = MLPRender_Fea(27, num_layers=3, hidden_dim=128, viewpe=6, feape=2).to(dev)
    n = 262144
    g = torch.Generator(device="cpu").manual_seed(3)
    feat = (torch.randn(n, 28, generator=g) * 0.5).to(dev)
    rays = torch.randn(n, 6, generator=g).to(dev)
    idx = torch.arange(n, dtype=torch.int32, device=dev)
    rgb = torch.empty(n, 3, device=dev)
    g_rgb = torch.randn(n, 3, generator=g).to(dev)
    g_feat = torch.empty_like(feat)
    for p in head.parameters():
        p.grad = torch.zeros_like(p)

    def run(fn, k):
        ts = []
        for _ in range(k):
            torch.cuda.synchronize()
            torch.cuda._sleep(2_000_000)  # the GPU stays busy while the host enqueues the timed launch
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    # the descriptors are built before the timed region, so the events see the kernels alone
    import ctypes
    from factor_fields_gb300 import _native as N
    from factor_fields_gb300.renderer import head_struct
    h = head_struct(head)
    gs = N.FFMlpGrad()
    ws_, bs_ = head.params()
    for i in range(3):
        gs.weight[i] = ws_[i].grad.data_ptr()
        gs.bias[i] = bs_[i].grad.data_ptr() if bs_[i] is not None else None
    fl = N.lib().ff_render_head_forward_tc
    bl = N.lib().ff_render_head_backward_tc
    fargs = (ctypes.byref(h), N.ptr(feat), 28, N.ptr(rays), N.ptr(idx), N.ptr(idx), n, N.ptr(rgb), None)
    bargs = (ctypes.byref(h), N.ptr(feat), 28, N.ptr(rays), N.ptr(idx), N.ptr(idx), n, N.ptr(g_rgb), N.ptr(g_feat),
             ctypes.byref(gs), None)
    st = N.stream_ptr()
    fwd = lambda: N.check(fl(*fargs, st), "ff_render_head_forward_tc")  # noqa: E731
    bwd = lambda: N.check(bl(*bargs, st), "ff_render_head_backward_tc")  # noqa: E731
    for _ in range(args.warmup):
        fwd()
        bwd()
    t_f, t_b = run(fwd, args.steps), run(bwd, args.steps)
    ff, fb = head_flops_per_sample(27)
    peaks = load_peaks()
    peak = peaks.get("bf16_tflops", 1900.0)
    ach_f, ach_b = ff * n / (t_f / 1e3) / 1e12, (ff + fb) * n / (t_b / 1e3) / 1e12
    out = {"head": "MLPRender_Fea, in 174 (27 features + PE 2, dirs + PE 6) -> 128 -> 128 -> 3, tcgen05 BF16 / FP32",
           "samples": n, "fwd_ms": t_f, "bwd_ms": t_b, "fwd_samples_per_s": n / (t_f / 1e3),
           "flops_per_sample": {"fwd": ff, "bwd": fb},
           "roofline": {"bound": "tensor", "kernel": "head_tc_kernel<27,2,6,bwd>",
                        "achieved": ach_b, "peak": peak, "unit": "TFLOP/s", "frac": ach_b / peak,
                        "fwd_achieved": ach_f, "fwd_frac": ach_f / peak,
                        "note": "algorithmic FLOPs (the backward launch recomputes the forward and is counted "
                                "as fwd + bwd); the kernel also runs the split-BF16 second MMA of layers 0 and 1",
                        "peak_source": ("MEASURED_PEAKS.json bf16_tflops (measured burst)" if "bf16_tflops" in peaks
                                        else "fallback")}}
    cfg = W.field_cfg("cfg2")
    cfg.renderer["shadingMode"] = "MLP_Fea"
    torch.manual_seed(0)
    m = FactorFields(cfg, device=dev, precision="bf16")
    pool = torch.from_numpy(W.BlobScene(0).ray_pool(1 << 16, 5)).float().to(dev)
    gen = torch.Generator(device=dev).manual_seed(0)
    ts = []
    for i in range(args.warmup + args.steps):
        r = pool[torch.randint(0, pool.shape[0], (4096,), device=dev, generator=gen)]
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rgb_r, _, _ = m(r, white_bg=True, is_train=True, N_samples=1024)
        (rgb_r * rgb_r).sum().backward()
        e1.record()
        torch.cuda.synchronize()
        if i >= args.warmup:
            ts.append(e0.elapsed_time(e1))
    out["cfg2_step_with_mlp_head"] = {"rays_per_step": 4096, "ms_per_step": float(np.mean(ts)),
                                     "rays_per_s": 4096 / (float(np.mean(ts)) / 1e3),
                                     "note": "untrained field (random-init), fwd+bwd, no optimizer"}
    return out


def run_cpu_baseline_render(m, pool, gt, n_rays=1024, steps=3, warmup=1):
    """The reference's render path on the host cores (oracle/ref_torch.py RefRender: sample_point,
    the alpha mask, get_coding + MLPMixer on the live samples, raw2alpha, the SH-2 colour head,
    compositing; fwd+bwd with the MSE loss) holding the trained configuration-2 model's parameters
    and occupancy volume, on a bounded sample of its training rays: rays/s, best step."""
    from oracle.ref_torch import RefRender, from_model
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    r = m.cfg.renderer
    vol = m.alphaMask.alpha_volume[0, 0].cpu() if m.alphaMask is not None else None
    rr = RefRender(from_model(m), float(m.stepSize), 1024, vol, r.density_shift, r.distance_scale,
                   r.rayMarch_weight_thres, r.fea2denseAct or "softplus")
    g = torch.Generator().manual_seed(5)
    idx = torch.randint(0, pool.shape[0], (n_rays,), generator=g)
    rays, rgb = pool[idx.to(pool.device)].cpu(), gt[idx.to(gt.device)].cpu().float()
    jit = torch.rand(n_rays, 1, generator=g)
    for _ in range(warmup):
        rr.train_step(rays, rgb, jit)
    best = []
    for _ in range(steps):
        t0 = time.perf_counter()
        rr.train_step(rays, rgb, jit)
        best.append(time.perf_counter() - t0)
    return {"value": n_rays / min(best), "unit": "rays/s", "cores": cores, "kind": CPU_KIND,
            "sample": f"{n_rays} training rays x up to 1024 samples with the trained model's occupancy volume, "
                      f"fwd+bwd (MSE), best of {steps} after {warmup} warm-up (torch CPU restatement of the "
                      "reference's FactorFields.forward render path with the SH-2 head (oracle/ref_torch.py "
                      "RefRender, pinned to renders of the reference itself))"}


def run_cpu_baseline_model(m, key, steps, warmup=1):
    """The reference's CPU op sequence (oracle/ref_torch.py) holding model m's parameters, on one
    batch of configuration `key` (all host threads): samples/s, best step."""
    from oracle.ref_torch import from_model
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    r = from_model(m)
    x, y = (torch.from_numpy(a) for a in field_batches(key, 7, 1)[0])
    loss = FIELD_CONFIGS[key]["loss"]
    for _ in range(warmup):
        r.fit_step(x, y, loss)
    best = []
    for _ in range(steps):
        t0 = time.perf_counter()
        r.fit_step(x, y, loss)
        best.append(time.perf_counter() - t0)
    n = x.shape[0]
    return {"value": n / min(best), "unit": "samples/s", "cores": cores, "kind": CPU_KIND,
            "sample": f"{n} points of the same workload per step, best of {steps} after {warmup} warm-up ({CPU_DESC})"}


def run_reference_arm(args, ws):
    """--impl reference: the reference's CPU op sequence on the native arm's workload (the same
    262,144-point batches of configuration 1, one batch per step), W warm-up steps then K timed
    steps on all host cores; value = points of the K steps / their total time."""
    from factor_fields_gb300 import workloads as W
    r, cores = _cpu_reference_field()
    nb = 8
    batches = [tuple(torch.from_numpy(a) for a in W.sdf_batch(i, N_POINTS)) for i in range(nb)]
    for i in range(args.warmup):
        r.fit_step(*batches[i % nb])
    t0 = time.perf_counter()
    for i in range(args.steps):
        r.fit_step(*batches[i % nb])
    dt = time.perf_counter() - t0
    value = N_POINTS * args.steps / dt
    return {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded analytic SDF: 16 spheres + 8 boxes)", "config": bench_config(ws),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": CPU_KIND,
                             "sample": f"the whole workload: {args.steps} steps of {N_POINTS} points after "
                                       f"{args.warmup} warm-up steps ({CPU_DESC})"},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_profile_case(case, level0_shared, dev):
    """One small workload for an ncu capture (ncu --profile-from-start off): the launches to capture
    run between torch.cuda.profiler.start() and stop(), after warm-up launches outside them.
      fit:cfg0 / fit:cfg1 / fit:cfg4  one binned fit step of the configuration (its batch size)
      radiance_fwd    the 28-wide field forward on a 4,096-ray batch's live samples (plain sampler,
                      300 training steps, occupancy volume updated at step 100)
      radiance_bwd    the 28-wide field backward on the same samples
      proposal_render the proposal head and resampling of a 400x400 view (160,000 rays, 32 samples)
      train:plain / train:proposal  two whole training steps (4,096 rays, fwd + bwd + the fused
                      Adam updates) replayed from their CUDA graph after 300 eager training steps"""
    from factor_fields_gb300 import workloads as W
    from factor_fields_gb300 import train as T
    if case.startswith("fit:"):
        key = case[4:]
        fc = FIELD_CONFIGS[key]
        x, y = field_batches(key, 0, 1)[0]
        x, y = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
        r = T.FieldFitRunner(make_model("bf16", key), loss=fc["loss"], level0_shared=level0_shared)
        for _ in range(3):
            r.step(x, y)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        r.step(x, y)
    elif case in ("radiance_fwd", "radiance_bwd"):
        import ctypes
        from factor_fields_gb300 import FactorFields
        from factor_fields_gb300 import _native as N
        from factor_fields_gb300 import functional as FN
        from factor_fields_gb300.renderer import field_eval, march, render_desc
        scene = W.BlobScene(0)
        pool = torch.from_numpy(scene.ray_pool(1 << 16, 5)).float()
        gt = scene.render_gt(pool.double().numpy(), n_steps=256).to(dev)
        pool = pool.to(dev)
        torch.manual_seed(0)
        m = FactorFields(W.field_cfg("cfg2"), device=dev, precision="bf16")
        tr = T.RadianceFieldTrainer(m, n_samples=1024, n_iters=300)
        g = torch.Generator(device=dev).manual_seed(0)
        for it in range(300):
            idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
            tr.step(pool[idx], gt[idx])
            if it == 100:
                m.updateAlphaMask((128, 128, 128), is_update_alphaMask=True, times=1)
        idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
        _, xyz, _ = march(m, pool[idx], None, render_desc(m, 1024, True))
        basis_r, coeff_r, dt = m._read_buffers()
        job = {"fused": True, "fdesc": m.descriptor(dt), "basis_r": basis_r, "coeff_r": coeff_r}
        if case == "radiance_fwd":
            run = lambda: field_eval(m, job, xyz)  # noqa: E731
        else:  # the field backward (ff_field_mlp_backward) on the same samples, scratch gradients
            lm = m.linear_mat
            ws_, bs_ = lm.weights()
            mlp = FN.mlp_struct(ws_, bs_, lm.in_dim, lm.hidden_dim, lm.out_dim)
            n = xyz.shape[0]
            g_out = torch.randn(n, lm.out_dim, device=dev, generator=g) * 1e-3
            gbas, gcoef = torch.zeros_like(m.basis_flat), torch.zeros_like(m.coeff_flat)
            gw = [torch.zeros_like(w) for w in ws_]
            gbias = [torch.zeros_like(b) if b is not None else None for b in bs_]
            grad = N.FFMlpGrad()
            for i in range(len(ws_)):
                grad.weight[i] = gw[i].data_ptr()
                grad.bias[i] = gbias[i].data_ptr() if gbias[i] is not None else None
            run = lambda: N.call("ff_field_mlp_backward", ctypes.byref(job["fdesc"]), N.ptr(basis_r),  # noqa: E731
                                 N.ptr(coeff_r), ctypes.byref(mlp), N.ptr(xyz), n, N.ptr(g_out), N.ptr(gbas),
                                 N.ptr(gcoef), ctypes.byref(grad), N.stream_ptr())
        for _ in range(3):
            run()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        run()
    elif case == "proposal_render":
        from factor_fields_gb300 import FactorFields
        from factor_fields_gb300.proposal import ProposalSampler
        torch.manual_seed(0)
        m = FactorFields(W.field_cfg("cfg2"), device=dev, precision="bf16")
        s = ProposalSampler(m, seed=0, render_fine=32)
        rays = torch.from_numpy(W.BlobScene(0).ray_pool(160000, 6, views=[7])).float().to(dev)
        with torch.no_grad():
            for _ in range(3):
                s.render(rays, is_train=False)
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
            s.render(rays, is_train=False)
    elif case in ("train:plain", "train:proposal"):
        from factor_fields_gb300 import FactorFields
        from factor_fields_gb300.proposal import ProposalSampler
        scene = W.BlobScene(0)
        pool = torch.from_numpy(scene.ray_pool(1 << 16, 5)).float()
        gt = scene.render_gt(pool.double().numpy(), n_steps=256).to(dev)
        pool = pool.to(dev)
        torch.manual_seed(0)
        m = FactorFields(W.field_cfg("cfg2"), device=dev, precision="bf16")
        sampler = ProposalSampler(m, seed=0) if case == "train:proposal" else None
        tr = T.RadianceFieldTrainer(m, n_samples=1024, n_iters=300, sampler=sampler)
        g = torch.Generator(device=dev).manual_seed(0)
        for it in range(300):
            idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
            tr.step(pool[idx], gt[idx])
            if it == 100 and sampler is None:
                m.updateAlphaMask((128, 128, 128), is_update_alphaMask=True, times=1)
        for it in range(5):
            idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
            tr.graph_step(pool[idx], gt[idx], optimize=True)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for it in range(2):
            idx = torch.randint(0, pool.shape[0], (4096,), device=dev, generator=g)
            tr.graph_step(pool[idx], gt[idx], optimize=True)
    else:
        raise SystemExit(f"unknown --profile-case {case!r}")
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile_case": case, "level0_shared": level0_shared, "ok": True}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--cpu-points", type=int, default=N_POINTS,
                    help="points per step of the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-render", action="store_true", help="skip the radiance-field configurations")
    ap.add_argument("--no-field-configs", action="store_true", help="skip the 2-D field configurations (0 and 4)")
    ap.add_argument("--head-only", action="store_true",
                    help="measure the MLPRender_Fea tensor-core head alone (prints its JSON record)")
    ap.add_argument("--render-iters", type=int, default=1500)
    ap.add_argument("--psnr-seeds", type=int, default=3, help="training seeds of the PSNR comparison")
    ap.add_argument("--profile-case", default=None,
                    help="run one small workload for an ncu capture and exit (see run_profile_case)")
    ap.add_argument("--level0-shared", action="store_true", help="--profile-case fit:*: FF_FIT_LEVEL0_SHARED")
    args = ap.parse_args()
    if args.profile_case:
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        run_profile_case(args.profile_case, args.level0_shared, dev)
        return 0
    ws, rank, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference_arm(args, ws)))
        return 0
    if args.head_only:
        dev = torch.device("cuda", local)
        torch.cuda.set_device(dev)
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
        print(json.dumps(measure_mlp_head(args, dev, flush)))
        return 0
    if ws > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    res = run_native(args, ws, rank, local)
    if not args.no_render:
        res["radiance_field"] = run_radiance(args, torch.device("cuda", local))
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=torch.device("cuda", local))
        res["radiance_field"]["mlp_fea_head"] = measure_mlp_head(args, torch.device("cuda", local), flush)
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = run_cpu_baseline(args.cpu_points, 3)
        print(json.dumps(res))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
