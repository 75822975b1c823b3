"""Autotuner for the operators' launch schedules.

A schedule is (slices carried per thread, warps per CTA, straight-line steps)
for one operator on one plan (`ctgb_plan_set_schedule`, `ctgb_plan_set_unroll`).
Carrying more slices per thread amortises the per-(view, line) geometry over
more fused multiply-adds but costs registers and therefore resident warps;
fewer warps per CTA changes how views (detector gather) or image rows (image
gather) are grouped; two straight-line steps instead of three skip the third
pixel (cell) that most cells (pixels) do not reach, at the price of a
divergent remainder loop where some do. The best choice depends on the
geometry, the batch and the GPU, so it is measured: every
candidate is timed with CUDA events on the caller's device and the fastest is
kept, in memory and in a JSON cache on disk
(``$CTLIB_GB300_TUNE_CACHE``, default ``~/.cache/ctlib_gb300/tune.json``).

``ops`` applies a cached schedule automatically; ``tune()`` measures (set
``CTLIB_GB300_AUTOTUNE=1`` to tune every new (plan, op, batch) on first use).

Ragged batches have a schedule of their own, the form of their CUDA graph:
one launch per stage over the task list of all slices (``branches=0``), or the
slices' own launches spread over k parallel graph branches. ``tune_ragged``
times each form on the batch's own inputs and caches the fastest under the
batch's signature (every slice's options, the dtype, the operator chain).
"""

from __future__ import annotations

import json
import os
import threading

import torch

from . import _native as N

CANDIDATES_F32 = ((16, 8, 3), (16, 8, 2), (16, 4, 3), (16, 4, 2), (8, 8, 3), (8, 8, 2), (8, 4, 2), (4, 8, 2))
CANDIDATES_F64 = ((4, 8, 3), (4, 4, 3), (2, 8, 3))

_lock = threading.Lock()
_cache = None


def _cache_path() -> str:
    return os.environ.get("CTLIB_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "ctlib_gb300", "tune.json"))


def _load():
    global _cache
    if _cache is None:
        try:
            with open(_cache_path()) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save():
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(_cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def _key(plan, op: int, batch: int) -> str:
    name = torch.cuda.get_device_name(plan.device)
    return f"{name}|{plan.dtype}|{op}|{batch}|{','.join(repr(v) for v in plan.values)}"


def _set(plan, op: int, sb: int, warps: int, unroll: int = 0):
    """Set the plan's schedule for `op` unless it is already the current one
    (one plan serves every batch size, each with its own tuned schedule)."""
    cur = plan.__dict__.setdefault("_current", {})
    if cur.get(op) != (sb, warps, unroll):
        N.check(N.lib().ctgb_plan_set_schedule(plan.handle, op, sb, warps), "schedule")
        N.check(N.lib().ctgb_plan_set_unroll(plan.handle, op, unroll), "schedule")
        cur[op] = (sb, warps, unroll)


def apply_cached(plan, op: int, batch: int) -> bool:
    """Use the cached schedule of (plan, op, batch), or the default one."""
    memo = plan.__dict__.setdefault("_tuned", {})
    if (op, batch) not in memo:
        with _lock:
            hit = _load().get(_key(plan, op, batch))
        if hit is None and os.environ.get("CTLIB_GB300_AUTOTUNE") == "1":
            tune(plan, op, batch)
            hit = memo[(op, batch)]
        if hit is not None and len(hit) == 3:  # older cache entry: (sb, warps, ms)
            hit = [hit[0], hit[1], 0, hit[2]]
        memo[(op, batch)] = None if hit is None else (int(hit[0]), int(hit[1]), int(hit[2]))
    sched = memo[(op, batch)]
    _set(plan, op, *(sched if sched is not None else (0, 0, 0)))
    return sched is not None


def _inputs(plan, op: int, batch: int):
    dev = torch.device("cuda", plan.device)
    img = (batch, 1, plan.height, plan.width)
    sino = (batch, 1, plan.views, plan.dets)
    if op in (N.OP_PROJECTION, N.OP_BACKPROJECTION_T):
        return torch.rand(img, dtype=plan.dtype, device=dev), torch.empty(sino, dtype=plan.dtype, device=dev)
    if op == N.OP_BACKPROJECTION_SV:  # one image per view
        views = (batch, plan.views, plan.height, plan.width)
        return torch.randn(sino, dtype=plan.dtype, device=dev), torch.empty(views, dtype=plan.dtype, device=dev)
    return torch.randn(sino, dtype=plan.dtype, device=dev), torch.empty(img, dtype=plan.dtype, device=dev)


def tune(plan, op: int, batch: int, reps: int = 3, candidates=None) -> dict:
    """Time every candidate schedule of `op` for `batch` slices, keep the best."""
    if candidates is None:
        candidates = CANDIDATES_F32 if plan.dtype == torch.float32 else CANDIDATES_F64
    x, out = _inputs(plan, op, batch)
    stream = torch.cuda.current_stream(x.device)
    results = []
    with torch.cuda.device(x.device):
        for sb, warps, unroll in candidates:
            _set(plan, op, sb, warps, unroll)
            plan.run(op, x, out)  # warm-up (and workspace size for this schedule)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                plan.run(op, x, out)
            b.record(stream)
            torch.cuda.synchronize(x.device)
            results.append((a.elapsed_time(b) / reps, sb, warps, unroll))
    results.sort()
    best_ms, sb, warps, unroll = results[0]
    _set(plan, op, sb, warps, unroll)
    with _lock:
        _load()[_key(plan, op, batch)] = [sb, warps, unroll, best_ms]
        _save()
    plan.__dict__.setdefault("_tuned", {})[(op, batch)] = (sb, warps, unroll)
    return {"slices_per_thread": sb, "warps_per_cta": warps, "unroll": unroll, "ms": best_ms,
            "candidates": [{"slices_per_thread": s, "warps_per_cta": w, "unroll": u, "ms": m}
                           for m, s, w, u in results]}


RAGGED_CANDIDATES = (0, 1, 2, 4, 8)


def _ragged_key(rb, ops) -> str:
    import hashlib
    name = torch.cuda.get_device_name(rb.device)
    sig = repr((tuple(tuple(p.values) for p in rb.plans), str(rb.dtype), tuple(ops)))
    return f"ragged|{name}|{hashlib.sha1(sig.encode()).hexdigest()}"


def ragged_cached(rb, ops):
    """The cached graph form (branch count, 0 = one launch per stage) of a
    ragged batch's operator chain, or None."""
    with _lock:
        hit = _load().get(_ragged_key(rb, ops))
    return None if hit is None else int(hit[0])


def tune_ragged(rb, ops, inputs, reps: int = 3, candidates=RAGGED_CANDIDATES) -> dict:
    """Time the graph forms of `ops` (a chain such as ("projection", "fbp")) on
    the ragged batch `rb` with `inputs`, keep the fastest (CUDA events around
    each replay, mean of `reps` after one warm-up replay)."""
    if isinstance(ops, str):
        ops = (ops,)
    stream = torch.cuda.current_stream(rb.device)
    results = []
    for br in candidates:
        replay, _, _ = rb.graphed(ops, inputs, branches=br)
        replay()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            replay()
        b.record(stream)
        torch.cuda.synchronize(rb.device)
        results.append((a.elapsed_time(b) / reps, br))
        del replay
    results.sort()
    best_ms, best = results[0]
    with _lock:
        _load()[_ragged_key(rb, ops)] = [best, best_ms]
        _save()
    return {"branches": best, "ms": best_ms, "candidates": [{"branches": br, "ms": ms} for ms, br in results]}
