"""Benchmark: ray-updates/s of projection + projection_t (the autograd pair) on
the fan equal-distance workload 16 x 512^2, 1152 views, 736 bins.

One step = A x followed by A^T y for the whole batch (one launch of each
operator for all 16 slices). A ray-update is one (slice, view, detector bin,
image line); one step is 2 * 16 * 1152 * 736 * 512 = 1.39e10 ray-updates.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py [--impl ours|reference] --operators   # each operator alone

Prints one JSON line (rank 0). Timing: CUDA events on the launching stream around
each step, L2 flushed (256 MB write) before every timed step, max over ranks.
Under torchrun each rank runs an independent replica of the workload (the
operators need no exchange between slices): weak scaling.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = "fan_ed_512"
METRIC = "ray-updates/s proj+adjoint 512² fan-ED B=16, batched vs plain, rel-L2≤1e-5"
UNIT = "ray-updates/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, val in zip(names, p[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _cpu_step(w, step_seconds: float):
    """One step of the CPU arm: the OpenMP oracle port (fp32, reference type
    promotions) running projection then projection_t on a bounded sample of the
    workload, one slice and a contiguous subset of its views sized to about
    `step_seconds`, on all host threads. Returns (step, ray-updates per step,
    sample description, threads)."""
    import oracle
    from ctlib_gb300.workloads import ellipse_phantom
    s = w.slices[0]
    o = list(s.options)
    V, D, W, H = (int(o[i]) for i in range(4))
    threads = oracle.max_threads()
    img = ellipse_phantom(H, W, o[4], s.seed)[None, None]
    sub = list(o)

    def step():
        sino = oracle.run("projection", img, sub, oracle.MODE_F32, threads)
        oracle.run("projection_t", sino, sub, oracle.MODE_F32, threads)

    nv = 16
    while True:
        sub[0] = float(nv)
        t0 = time.perf_counter()
        step()
        dt = time.perf_counter() - t0
        if dt > step_seconds / 2 or nv >= V:
            break
        nv = min(V, int(nv * max(2.0, step_seconds / max(dt, 1e-3))))
    ru = 2 * nv * D * max(W, H)
    return step, ru, f"1 slice of {w.name}, views 0..{nv - 1} of {V}, projection + projection_t", threads


def _cpu_baseline(w, seconds_target: float = 15.0) -> dict:
    """The CPU arm timed over about `seconds_target` seconds of repeated steps,
    in ray-updates/s."""
    step, ru, sample, threads = _cpu_step(w, 1.0)
    t0 = time.perf_counter()
    step()
    one = time.perf_counter() - t0
    reps = max(1, int(round(seconds_target / max(one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(reps):
        step()
    dt = (time.perf_counter() - t0) / reps
    return {"value": ru / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample}, {reps} rep(s) of {dt:.2f} s"}


def run_reference(args):
    """Reference arm: the reference has no CPU path; its distance-driven loops
    run as the OpenMP oracle port on the host cores (all threads), each step a
    bounded sample of the workload (about 2 s), W warm-up and K timed steps."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from ctlib_gb300.workloads import WORKLOADS
    from oracle import build as obuild
    obuild.build_oracle()
    w = WORKLOADS[args.workload]()
    step, ru, sample, threads = _cpu_step(w, 2.0)
    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = ru / (ms / 1e3)
    cb = {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": f"{sample}, per step"}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic ellipse phantoms (seeded)",
            "config": {"workload": w.name, "global_batch": len(w.slices), "cpu_sample": sample,
                       "ray_updates_per_step": ru},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    rc = _reference_cuda(w, args)
    if rc is not None:
        line["reference_cuda"] = rc
    print(json.dumps(line), flush=True)
    return 0


LAPLACIAN_CASE = {"points": 16384, "dim": 64, "k": 16}


def _laplacian_timing(fn, timed, dev):
    """Mean time of one laplacian call (fp32 Gaussian points, seed 1) with its
    FP32 FMA count n^2 * dim."""
    import torch
    c = LAPLACIAN_CASE
    x = torch.from_numpy(np.random.default_rng(1).standard_normal((c["points"], c["dim"])).astype(np.float32)).to(dev)
    ms = timed(lambda: fn(x, c["k"]))
    fma = float(c["points"]) ** 2 * c["dim"]
    return {"case": dict(c), "ms": ms, "fma_per_s": fma / (ms / 1e3),
            "note": "kNN graph adjacency of n points: distances, top-k, median, weights, COO output"}


def run_laplacian_only(args):
    """One JSON line with the laplacian case alone (W warm-up, K timed calls)."""
    import torch
    import ctlib_gb300 as ctlib
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ts = []
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    print(json.dumps({"only_laplacian": True, **_laplacian_timing(lambda x, k: ctlib.laplacian(x, k), timed, dev)}),
          flush=True)
    return 0


OPERATORS = ("projection", "projection_t", "backprojection", "backprojection_t", "fbp", "backprojection_sv",
             "backprojection_sv_1")


def run_operators(args):
    """One JSON line: each operator of the public API alone on the workload's
    batch, mean ms over K calls after W warm-up calls, L2 flushed before every
    timed call, CUDA events on the launching stream. backprojection_sv (equal-
    distance fans only) writes one image per view: it runs on the whole batch
    when that output fits in 24 GB, and as backprojection_sv_1 on one slice.
    --impl reference times the reference's own CUDA kernels through
    oracle/ref_cuda.py instead (fbp: its weighting, taps, torch conv2d and
    backprojection kernel)."""
    import torch
    from ctlib_gb300.workloads import WORKLOADS, phantoms
    w = WORKLOADS[args.workload]()
    if not w.uniform:
        raise SystemExit("--operators needs a uniform workload")
    if args.batch:
        w.slices = w.slices[:1] * args.batch
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    dt = torch.float64 if args.dtype == "f64" else torch.float32
    img = torch.from_numpy(np.stack(phantoms(w))[:, None]).to(dt).contiguous().to(dev)
    opts = torch.tensor(w.slices[0].options, dtype=dt, device=dev)
    if args.impl == "reference":
        from oracle import ref_cuda
        if not ref_cuda.available():
            print(json.dumps({"impl": "reference", "operators": None,
                              "unavailable": "reference cubins not built"}), flush=True)
            return 0
        ref = ref_cuda.get()
        sino = ref.run(0, img, opts)
        calls = {"projection": lambda: ref.run(0, img, opts), "projection_t": lambda: ref.run(1, sino, opts),
                 "backprojection": lambda: ref.run(2, sino, opts), "backprojection_t": lambda: ref.run(3, img, opts),
                 "fbp": lambda: ref.fbp(sino, opts), "backprojection_sv": lambda: ref.run(5, sino, opts),
                 "backprojection_sv_1": lambda: ref.run(5, sino[:1], opts)}
    else:
        import ctlib_gb300 as ctlib
        from ctlib_gb300 import _native as N
        sino = ctlib.projection(img, opts)
        if not args.no_tune:
            from ctlib_gb300 import tune
            plan = ctlib.get_plan(opts, dt, dev)
            ops = [N.OP_PROJECTION, N.OP_PROJECTION_T, N.OP_BACKPROJECTION, N.OP_BACKPROJECTION_T, N.OP_FBP]
            if w.slices[0].scan_type == 0:
                ops.append(N.OP_BACKPROJECTION_SV)
            for op in ops:
                tune.tune(plan, op, img.shape[0])
                if op == N.OP_BACKPROJECTION_SV:
                    tune.tune(plan, op, 1)
        calls = {"projection": lambda: ctlib.projection(img, opts),
                 "projection_t": lambda: ctlib.projection_t(sino, opts),
                 "backprojection": lambda: ctlib.backprojection(sino, opts),
                 "backprojection_t": lambda: ctlib.backprojection_t(img, opts), "fbp": lambda: ctlib.fbp(sino, opts),
                 "backprojection_sv": lambda: ctlib.backprojection_sv(sino, opts),
                 "backprojection_sv_1": lambda: ctlib.backprojection_sv(sino[:1], opts)}
    res = {}
    # backprojection_sv exists for equal-distance fans only (src/fan_ed_kernel.cu:946-1161)
    names = list(OPERATORS if w.slices[0].scan_type == 0 else OPERATORS[:-2])
    if args.op:
        if args.op not in names:
            raise SystemExit(f"--op must be one of {names}")
        names = [args.op]
    if "backprojection_sv" in names and img.numel() * sino.shape[-2] * img.element_size() > 24e9:  # B x V x H x W
        names.remove("backprojection_sv")
    for name in names:
        fn = calls[name]
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        slices = 1 if name == "backprojection_sv_1" else img.shape[0]
        ms = statistics.mean(ts)
        res[name] = {"ms": ms, "slices": slices,
                     "ray_updates_per_s": w.ray_updates() * slices / img.shape[0] / (ms / 1e3)}
    print(json.dumps({"impl": args.impl, "workload": args.workload, "batch": img.shape[0], "dtype": args.dtype,
                      "operators": res,
                      "timing": "mean of K calls, L2 flushed before each, CUDA events on the launching stream"}),
          flush=True)
    return 0


def _reference_cuda(w, args):
    """The reference's own CUDA kernels (src/fan_ed_kernel.cu prj_fan_ed and
    prj_t_fan_ed, compiled unchanged for sm_103a, oracle/ref_cuda.py) on the full
    workload: one step = projection then projection_t of the whole batch, each
    call allocating its output as the reference's wrapper does, L2 flushed
    before every step, CUDA events on the launching stream. None when there is
    no GPU or the cubins were not built."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        from oracle import ref_cuda
        if not ref_cuda.available():
            return None
    except Exception:
        return None
    from ctlib_gb300.workloads import phantoms
    ref = ref_cuda.get()
    dev = ref.device
    stream = torch.cuda.current_stream(dev)
    opts = torch.tensor(w.slices[0].options, dtype=torch.float32, device=dev)
    img_h = torch.from_numpy(np.stack(phantoms(w))[:, None]).contiguous()
    img = img_h.to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(max(1, args.warmup)):
        ref.run(1, ref.run(0, img, opts), opts)
    torch.cuda.synchronize()
    t_a, t_at = [], []
    for i in range(args.steps):
        flush.fill_(float(i))
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        s = ref.run(0, img, opts)
        e1.record(stream)
        ref.run(1, s, opts)
        e2.record(stream)
        torch.cuda.synchronize()
        t_a.append(e0.elapsed_time(e1))
        t_at.append(e1.elapsed_time(e2))
    ms = statistics.mean(a + b for a, b in zip(t_a, t_at))
    ru = 2 * w.ray_updates()
    # end to end: host image in, host image out, as a reference user would call it
    img_pin = img_h.pin_memory()
    out_h = torch.empty_like(img_h).pin_memory()
    e2e = []
    for i in range(args.steps):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        x = img_pin.to(dev, non_blocking=True)
        out_h.copy_(ref.run(1, ref.run(0, x, opts), opts), non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        e2e.append(a.elapsed_time(b))
    e2e_ms = statistics.mean(e2e)

    def timed(fn):
        for _ in range(2):
            fn()
        ts = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    lap = _laplacian_timing(lambda x, k: ref.laplacian(x, k), timed, dev) if ref_cuda.laplacian_available() else None
    return {"value": ru / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "ms_projection": statistics.mean(t_a), "ms_projection_t": statistics.mean(t_at),
            "e2e": {"value": ru / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": img_h.numel() * 4, "d2h_bytes_per_step": img_h.numel() * 4},
            "kind": "reference CUDA kernels (src/fan_ed_kernel.cu) compiled for sm_103a, launched with the "
                    "reference wrappers' grids and output allocations",
            "dtype": "f32", "gpu_launches_per_step": 2, "laplacian": lap}


def _fp32_peak(device) -> dict:
    """Measured FFMA throughput of this GPU (lane-FMAs/s) from a short
    register-resident FMA kernel in libctgb (see csrc/peak_fp32.cu)."""
    from ctlib_gb300 import _peak
    return _peak.measure(device)


def run_ours(args):
    import torch
    import torch.distributed as dist

    import ctlib_gb300 as ctlib
    from ctlib_gb300 import autograd as ag
    from ctlib_gb300.workloads import WORKLOADS, phantoms

    ws, rank, local = _dist()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = WORKLOADS[args.workload]()
    B = len(w.slices)
    opts = torch.tensor(w.slices[0].options, dtype=torch.float32)
    V, D, W, H = (int(w.slices[0].options[i]) for i in range(4))
    img_h = torch.from_numpy(np.stack(phantoms(w))[:, None]).contiguous()
    img = img_h.to(dev)
    ru_step = 2 * w.ray_updates()
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        s = ctlib.projection(img, opts)
        return ctlib.projection_t(s, opts)

    plan = ctlib.get_plan(opts, torch.float32, dev)
    # schedules picked by the autotuner (outside the timed region, like any
    # one-time plan set-up); --no-tune keeps the default schedule
    tuned = {}
    if not args.no_tune:
        from ctlib_gb300 import tune
        from ctlib_gb300 import _native as N
        for op, name in ((N.OP_PROJECTION, "projection"), (N.OP_PROJECTION_T, "projection_t")):
            r = tune.tune(plan, op, B)
            tuned[name] = {"slices_per_thread": r["slices_per_thread"], "warps_per_cta": r["warps_per_cta"],
                           "unroll": r["unroll"]}
            tune.tune(plan, op, 1)  # schedule of the one-slice-per-call path
    # warm-up (builds plans, workspace, caches)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # -- device-resident timing, per-op events -----------------------------
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clk = ClockSampler(local)
    clk.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.fill_(float(i))
        e0, e1, e2 = ev[i]
        e0.record(stream)
        s = ctlib.projection(img, opts)
        e1.record(stream)
        ctlib.projection_t(s, opts)
        e2.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    t_a = [ev[i][0].elapsed_time(ev[i][1]) for i in range(args.steps)]
    t_at = [ev[i][1].elapsed_time(ev[i][2]) for i in range(args.steps)]
    step_ms = sum(a + b for a, b in zip(t_a, t_at)) / args.steps
    if args.only_step:
        if rank == 0:
            print(json.dumps({"only_step": True, "ms_per_step": step_ms, "ms_projection": statistics.mean(t_a),
                              "ms_projection_t": statistics.mean(t_at),
                              "value": ws * ru_step / (step_ms / 1e3), "unit": UNIT, "clocks": clocks}),
                  flush=True)
        if ws > 1:
            dist.destroy_process_group()
        return 0
    if ws > 1:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    value = ws * ru_step / (step_ms / 1e3)

    # -- plain per-slice path (one call per slice) ---------------------------
    torch.cuda.synchronize()
    plain_ms = []
    for i in range(max(2, args.steps // 2)):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for k in range(B):
            s = ctlib.projection(img[k:k + 1], opts)
            ctlib.projection_t(s, opts)
        b.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(a.elapsed_time(b))
    plain_value = ru_step / (statistics.median(plain_ms) / 1e3)

    # -- end to end through the autograd API with host buffers ---------------
    y_meas = ctlib.projection(img, opts)
    img_pin = img_h.pin_memory()
    grad_h = torch.empty_like(img_h).pin_memory()
    loss_h = torch.empty((), dtype=torch.float32).pin_memory()
    op = ag.Projector(opts)

    def e2e_step():
        x = img_pin.to(dev, non_blocking=True).requires_grad_(True)
        r = op(x) - y_meas
        loss = 0.5 * (r * r).sum()
        loss.backward()
        grad_h.copy_(x.grad, non_blocking=True)
        loss_h.copy_(loss.detach(), non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = []
    for i in range(args.steps):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e2e_step()
        b.record(stream)
        torch.cuda.synchronize()
        e2e_ms.append(a.elapsed_time(b))
    e2e_mean = sum(e2e_ms) / len(e2e_ms)
    if ws > 1:
        t = torch.tensor([e2e_mean], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_mean = float(t.item())
    e2e_value = ws * ru_step / (e2e_mean / 1e3)

    # -- data-term gradient A^T(Ax - y): fused call vs composed operators -----
    from ctlib_gb300.ops import data_gradient

    def timed(fn):
        for _ in range(2):
            fn()
        ts = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    grad_fused = timed(lambda: data_gradient(img, y_meas, opts))
    grad_composed = timed(lambda: ctlib.projection_t(ctlib.projection(img, opts) - y_meas, opts))

    # -- kNN graph adjacency (laplacian) on its own synthetic points ----------
    lap = _laplacian_timing(lambda x, k: ctlib.laplacian(x, k), timed, dev)

    # -- parity of the timed operator pair vs the FP64 oracle (1 slice) -------
    parity = None
    if rank == 0:
        import oracle
        x0 = img_h[:1].numpy()
        a_ref = oracle.run("projection", x0, w.slices[0].options, oracle.MODE_F64_ON_F32)
        a_got = ctlib.projection(img[:1], opts).cpu().numpy()
        at_ref = oracle.run("projection_t", a_got, w.slices[0].options, oracle.MODE_F64_ON_F32)
        at_got = ctlib.projection_t(torch.from_numpy(a_got).to(dev), opts).cpu().numpy()
        parity = {"projection_rel_l2_vs_fp64": oracle.rel_l2(a_got, a_ref),
                  "projection_t_rel_l2_vs_fp64": oracle.rel_l2(at_got, at_ref)}

    # kernels of this package per timed step: image layout + detector gather,
    # sinogram layout + image gather, and the sum of the image gather's view
    # parts when it splits the views
    launches_per_step = 4 + (1 if _view_split(V, W * H) > 1 else 0)

    # -- roofline of the dominant kernel -------------------------------------
    ta, tat = statistics.mean(t_a), statistics.mean(t_at)
    ka, kat = _kernel_times(plan, args.steps, flush, stream, lambda: ctlib.projection(img, opts),
                            lambda s: ctlib.projection_t(s, opts))
    dom = "k_det_gather (projection)" if ka >= kat else "k_pix_gather (projection_t)"
    dom_ms = max(ka, kat)
    # algorithmic bytes of one launch: read input + write output once
    alg_bytes = (B * H * W + B * V * D) * 4
    hbm_peak = _measured("hbm_gbs", 6790.7)
    achieved_gbs = alg_bytes / (dom_ms / 1e3) / 1e9
    peak = _fp32_peak(dev) if rank == 0 else None
    traffic = _ncu_traffic(dom.split()[0], args.workload)
    roof = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak[0], "unit": "GB/s",
            "frac": achieved_gbs / hbm_peak[0], "traffic": traffic,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm_peak[1] == "measured" else "fallback 6790.7 GB/s",
            "traffic_source": ("committed ncu summary profiles/dram_traffic.json (dram__bytes_read.sum + "
                               "dram__bytes_write.sum of one capture of this workload), not measured in this run"
                               if traffic is not None else "no ncu capture of this workload"),
            "kernel": dom, "kernel_ms": dom_ms, "algorithmic_bytes": alg_bytes,
            "timing": "CUDA events recorded by the library right around the kernel, mean of the timed steps"}
    roof_fp32 = None
    if peak:
        # model: 8 FP32 lane-ops per ray-update (two overlap segments of min, max,
        # subtract and FMA each) at the measured FFMA rate
        model_peak = peak["lane_ops_per_s"] / 8.0
        ru_dom = w.ray_updates()
        ach = ru_dom / (dom_ms / 1e3)
        roof_fp32 = {"achieved": ach, "peak": model_peak, "unit": "ray-updates/s", "frac": ach / model_peak,
                     "model": "8 FP32 lane-ops per ray-update at measured FFMA lane-op rate",
                     "peak_source": "builder-measured: FFMA lane-op rate of this GPU timed in this run by "
                                    "ctlib_gb300/csrc/peak_fp32.cu (MEASURED_PEAKS.json has no FP32 figure)",
                     "measured_fp32": peak}

    if rank == 0:
        # the CPU baseline is timed at N = 1 only (a replica run would only add
        # the same host measurement to every line)
        cb = _cpu_baseline(w) if ws == 1 else None
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic ellipse phantoms (seeded)",
                "config": {"workload": w.name, "global_batch": B * ws, "per_gpu_batch": B, "views": V,
                           "dets": D, "image": [H, W], "parallelism": f"replicas{ws}",
                           "l2": "flushed (256 MB write) before every timed step",
                           "schedule": tuned or "default",
                           "ray_updates_per_step": ru_step},
                "plain": {"value": plain_value, "unit": UNIT, "ms_per_step": statistics.median(plain_ms),
                          "note": "one projection + projection_t call per slice"},
                "batched_over_plain": value / ws / plain_value,
                "ms_projection": ta, "ms_projection_t": tat,
                "kernel_ms": {"k_det_gather": ka, "k_pix_gather": kat},
                "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_mean,
                        "h2d_bytes_per_step": int(img_h.numel() * 4),
                        "d2h_bytes_per_step": int(img_h.numel() * 4 + 4),
                        "path": "ctlib_gb300.autograd.Projector: H2D image, A, loss, backward (A^T), D2H grad+loss"},
                "data_gradient": {"ms_fused": grad_fused, "ms_composed": grad_composed,
                                  "note": "A^T(Ax - y) for the same batch: ctgb_data_gradient vs projection, "
                                          "subtraction, projection_t"},
                "laplacian": lap,
                "gpu_launches": args.steps * launches_per_step,
                "clocks": clocks, "roofline": roof, "roofline_fp32": roof_fp32, "parity": parity,
                "cpu_baseline": cb}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_ragged(args):
    """Ragged workload: projection then fbp over slices of mixed geometry, as one
    CUDA-graph replay in the form the autotuner picks for this batch (one
    launch per stage over all slices, or the slices' own launches on parallel
    graph branches; tuned outside the timed region), against the same work as
    per-slice calls, with the one-launch-per-stage form timed beside it.
    Ray-updates counted for both operators."""
    import torch

    import ctlib_gb300 as ctlib
    from ctlib_gb300 import tune
    from ctlib_gb300.batched import RaggedBatch
    from ctlib_gb300.workloads import WORKLOADS, phantoms

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = WORKLOADS[args.workload]()
    opts = [s.options for s in w.slices]
    imgs = [torch.from_numpy(x[None, None]).to(dev) for x in phantoms(w)]
    ru_step = 2 * w.ray_updates()
    rb = RaggedBatch(opts, dev)
    chain = ("projection", "fbp")
    tuned = tune.tune_ragged(rb, chain, imgs)
    replay_t, _, outs_t = rb.graphed(chain, imgs, branches=tuned["branches"])
    replay_p, _, outs_p = rb.graphed(chain, imgs, branches=0)
    topts = [torch.tensor(o, dtype=torch.float32) for o in opts]
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def plain():
        for x, o in zip(imgs, topts):
            ctlib.fbp(ctlib.projection(x, o), o)

    for _ in range(args.warmup):
        replay_t()
        replay_p()
        plain()
    torch.cuda.synchronize()

    def timed(fn):
        ms = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return sum(ms) / len(ms)

    clk = ClockSampler(local)
    clk.start()
    t_ms = timed(replay_t)
    g_ms = timed(replay_p)
    p_ms = timed(plain)
    clocks = clk.stop()
    # parity of the graph replays against the per-slice calls
    same_t = all(torch.equal(y, ctlib.fbp(ctlib.projection(x, o), o)) for x, o, y in zip(imgs, topts, outs_t))
    same_p = all(torch.equal(y, z) for y, z in zip(outs_p, outs_t))
    form = ("one launch per stage over all slices" if tuned["branches"] == 0 else
            f"the slices' own launches on {tuned['branches']} parallel CUDA-graph branches")
    line = {"metric": f"ray-updates/s projection+fbp {w.name}", "value": ru_step / (t_ms / 1e3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic ellipse phantoms (seeded)",
            "config": {"workload": w.name, "slices": len(opts), "ray_updates_per_step": ru_step,
                       "path": f"RaggedBatch.graphed(('projection','fbp')), autotuned form: {form}",
                       "tuning": tuned, "l2": "flushed before every timed step"},
            "plain": {"value": ru_step / (p_ms / 1e3), "unit": UNIT, "ms_per_step": p_ms,
                      "note": "per-slice ctlib.projection + ctlib.fbp calls"},
            "ragged_over_plain": p_ms / t_ms, "identical_to_per_slice_calls": bool(same_t),
            "one_launch_per_stage": {"value": ru_step / (g_ms / 1e3), "unit": UNIT, "ms_per_step": g_ms,
                                     "over_plain": p_ms / g_ms, "identical": bool(same_p),
                                     "path": "RaggedBatch.graphed(..., branches=0)"},
            "clocks": clocks}
    print(json.dumps(line), flush=True)
    return 0


def run_unrolled(args):
    """Unrolled reconstruction: one step = K gradient-descent iterations
    x <- x - a A^T(A x - y) from x = 0 on the whole batch, each iteration
    checkpointed, then backpropagation of 0.5 ||x_K - x_true||^2 to the
    measured sinogram y (y.grad). y is Poisson log data of the phantoms
    (I0 = 1e5, counts clamped >= 1, seed 11) and a = 1 / lambda_max(A^T A).
    Ray-updates are counted over the operator launches one step actually makes
    (counted on an untimed step). Our arm runs ctlib_gb300.recon.unrolled_gd;
    --impl reference runs the same recursion through torch autograd on the
    reference's own kernels (oracle/ref_cuda.py), and the CPU port's rate on a
    bounded sample."""
    import torch

    import ctlib_gb300 as ctlib
    from ctlib_gb300 import autograd as ag
    from ctlib_gb300 import recon
    from ctlib_gb300.workloads import WORKLOADS, phantoms

    ws, rank, local = _dist()
    if args.impl == "reference" and rank != 0:
        return 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = WORKLOADS[args.workload]()
    B = len(w.slices)
    o = w.slices[0].options
    V, D, W, H = (int(o[i]) for i in range(4))
    opts = torch.tensor(o, dtype=torch.float32)
    x_true_h = torch.from_numpy(np.stack(phantoms(w))[:, None]).contiguous()
    xt = x_true_h.to(dev)
    y_h = torch.from_numpy(recon.poisson_log_sinogram(ctlib.projection(xt, opts).cpu().numpy(), 1e5, 11))
    y_dev = y_h.to(dev)
    step_a = recon.gd_step_size(opts, H, W, dev)
    K = args.unrolled
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    if args.impl == "reference":
        from oracle import ref_cuda
        if not ref_cuda.available():
            print(json.dumps({"impl": "reference", "unavailable": "reference cubins not built"}), flush=True)
            return 0
        ref = ref_cuda.get()
        od = torch.tensor(o, dtype=torch.float32, device=dev)

        class _RefLinear(torch.autograd.Function):
            @staticmethod
            def forward(ctx, x, fwd, bwd):
                ctx.bwd = bwd
                return ref.run(fwd, x.detach().contiguous(), od)

            @staticmethod
            def backward(ctx, g):
                return ref.run(ctx.bwd, g.contiguous(), od), None, None

        A = lambda x: _RefLinear.apply(x, 0, 1)
        At = lambda s: _RefLinear.apply(s, 1, 0)
        counted = ref_cuda.RefCuda.run
    else:
        A = lambda x: ag.projection(x, opts)
        At = lambda s: ag.projection_t(s, opts)
        counted = None

    from torch.utils.checkpoint import checkpoint

    def one_iter(x, y):
        return x - step_a * At(A(x) - y)

    def forward_backward(y):
        y = y.detach().requires_grad_(True)
        if args.impl == "reference":
            x = torch.zeros_like(xt)
            for _ in range(K):
                x = checkpoint(one_iter, x, y, use_reentrant=False)
        else:
            x = recon.unrolled_gd(y, opts, K, step_a)
        loss = 0.5 * ((x - xt) ** 2).sum()
        loss.backward()
        return loss.detach(), y.grad

    # operator launches per step, counted on one untimed step
    calls = [0]
    image_gathers = [0]  # calls whose kernel is the image gather (A^T, B, fbp)
    if counted is None:
        orig = ag._run

        def counting(op, x, plan):
            calls[0] += 1
            if op in (ag.N.OP_PROJECTION_T, ag.N.OP_BACKPROJECTION, ag.N.OP_FBP):
                image_gathers[0] += 1
            return orig(op, x, plan)
        ag._run = counting
        try:
            forward_backward(y_dev)
        finally:
            ag._run = orig
    else:
        orig = ref_cuda.RefCuda.run

        def counting(self, op, *a, **k):
            calls[0] += 1
            return orig(self, op, *a, **k)
        ref_cuda.RefCuda.run = counting
        try:
            forward_backward(y_dev)
        finally:
            ref_cuda.RefCuda.run = orig
    ops_per_step = calls[0]
    ru_step = ops_per_step * w.ray_updates()

    for _ in range(args.warmup):
        forward_backward(y_dev)
    torch.cuda.synchronize()

    def timed(fn):
        ts = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    clk = ClockSampler(local)
    clk.start()
    ms = timed(lambda: forward_backward(y_dev))
    clocks = clk.stop()
    # end to end: measured sinogram from pinned host memory, gradient and loss back
    y_pin = y_h.pin_memory()
    g_h = torch.empty_like(y_h).pin_memory()
    l_h = torch.empty((), dtype=torch.float32).pin_memory()

    def e2e():
        loss, g = forward_backward(y_pin.to(dev, non_blocking=True))
        g_h.copy_(g, non_blocking=True)
        l_h.copy_(loss, non_blocking=True)

    e2e()
    e2e_ms = timed(e2e)
    value = ru_step / (ms / 1e3)
    line = {"metric": f"ray-updates/s unrolled GD ({K} it, checkpointed) fwd+bwd {w.name}", "value": value,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic ellipse phantoms (seeded), Poisson log data I0=1e5 seed 11",
            "config": {"workload": w.name, "global_batch": B, "views": V, "dets": D, "image": [H, W],
                       "iterations": K, "step_size": step_a, "operator_launches_per_step": ops_per_step,
                       "ray_updates_per_step": ru_step, "l2": "flushed (256 MB write) before every timed step"},
            "e2e": {"value": ru_step / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": int(y_h.numel() * 4), "d2h_bytes_per_step": int(y_h.numel() * 4 + 4)},
            "clocks": clocks}
    if args.impl == "reference":
        line["impl"] = "reference"
        line["path"] = ("torch autograd over the reference's prj_fan_ea / prj_t_fan_ea kernels compiled for "
                        "sm_103a (oracle/ref_cuda.py), the same checkpointed recursion")
    else:
        line["path"] = "ctlib_gb300.recon.unrolled_gd through ctlib_gb300.autograd (projection <-> projection_t)"
        # each operator call launches a layout kernel and a gather kernel, and an
        # image gather that splits its views also the sum of the parts
        split = _view_split(V, W * H) > 1
        line["gpu_launches"] = (2 * ops_per_step + (image_gathers[0] if split else 0)) * args.steps
        peak = _fp32_peak(dev)
        model_peak = peak["lane_ops_per_s"] / 8.0
        line["roofline_fp32"] = {"achieved": value, "peak": model_peak, "unit": "ray-updates/s",
                                 "frac": value / model_peak, "scope": "whole step (all operator launches)",
                                 "model": "8 FP32 lane-ops per ray-update at measured FFMA lane-op rate",
                                 "peak_source": "builder-measured FFMA rate (ctlib_gb300/csrc/peak_fp32.cu)"}
        line["cpu_baseline"] = _cpu_baseline(w)
    print(json.dumps(line), flush=True)
    return 0


def _view_split(views: int, pixels: int) -> int:
    """View parts of the image gather (view_split in csrc/ctgb_kernels.cu)."""
    if pixels <= (1 << 17):
        return 1 if views < 80 else min(8, views // 40)
    return 1 if views < 256 else (8 if views >= 1024 else views // 128)


def _kernel_times(plan, steps, flush, stream, run_a, run_at):
    """Mean durations (ms) of the gather kernel of projection and of
    projection_t alone: the library records caller events right around each
    gather launch (ctgb_plan_set_kernel_events), on the launching stream."""
    import torch
    from ctlib_gb300 import _native as N
    evs = []
    for _ in range(steps):
        pair = []
        for _ in range(2):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)  # creates the CUDA events behind the handles
            b.record(stream)
            pair.append((a, b))
        evs.append(pair)
    torch.cuda.synchronize()
    lib = N.lib()
    try:
        for i in range(steps):
            flush.fill_(float(i))
            (a0, b0), (a1, b1) = evs[i]
            N.check(lib.ctgb_plan_set_kernel_events(plan.handle, a0.cuda_event, b0.cuda_event), "kernel events")
            s = run_a()
            N.check(lib.ctgb_plan_set_kernel_events(plan.handle, a1.cuda_event, b1.cuda_event), "kernel events")
            run_at(s)
    finally:
        lib.ctgb_plan_set_kernel_events(plan.handle, None, None)
    torch.cuda.synchronize()
    ka = statistics.mean(evs[i][0][0].elapsed_time(evs[i][0][1]) for i in range(steps))
    kt = statistics.mean(evs[i][1][0].elapsed_time(evs[i][1][1]) for i in range(steps))
    return ka, kt


def _measured(key, fallback):
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)[key]), "measured"
    except (OSError, KeyError, ValueError):
        return fallback, "fallback"


def _ncu_traffic(kernel: str, workload: str):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu
    summary (profiles/dram_traffic.json, written from an ncu capture of one
    workload and its tuned schedule), or None when that summary covers another
    workload."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(path) as f:
            summary = json.load(f)
    except (OSError, ValueError):
        return None
    if summary.get("workload_key") != workload:
        return None
    entry = summary.get("kernels", {}).get(kernel)
    return None if entry is None else entry.get("bytes_per_launch")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch schedules")
    ap.add_argument("--only-step", action="store_true",
                    help="time only the batched projection + projection_t step (for profiler runs)")
    ap.add_argument("--only-laplacian", action="store_true",
                    help="time only the laplacian case (16384 points, dimension 64, k = 16; for profiler runs)")
    ap.add_argument("--operators", action="store_true",
                    help="time each operator of the API alone on the workload (both arms)")
    ap.add_argument("--batch", type=int, default=0, help="with --operators: slices per call (default: the workload's)")
    ap.add_argument("--dtype", default="f32", choices=["f32", "f64"], help="with --operators: element type")
    ap.add_argument("--op", default="", help="with --operators: time this operator only (for profiler runs)")
    ap.add_argument("--unrolled", type=int, default=0,
                    help="time K checkpointed gradient-descent iterations forward + backward (both arms)")
    args = ap.parse_args()
    if args.warmup < 1:
        args.warmup = 1
    if args.only_laplacian:
        return run_laplacian_only(args)
    if args.operators:
        return run_operators(args)
    if args.unrolled:
        return run_unrolled(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload.startswith("ragged"):
        return run_ragged(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
