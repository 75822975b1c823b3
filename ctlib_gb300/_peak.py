"""Measured FP32 FMA rate of the current GPU (benchmark support).

The distance-driven operators are bounded by the SIMT FP32 / load pipes, not by
HBM or tensor cores; this probe gives the FP32 denominator of their roofline.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

from . import _native as N

SO = os.path.join(N.BUILD_DIR, "libctgb_peak.so")
SRC = os.path.join(N.CSRC, "peak_fp32.cu")


def build(force: bool = False) -> str:
    if force or not os.path.exists(SO) or os.path.getmtime(SRC) > os.path.getmtime(SO):
        os.makedirs(N.BUILD_DIR, exist_ok=True)
        tmp = SO + ".tmp"
        subprocess.run([N.nvcc(), N.ARCH, "-O3", "-Xcompiler", "-fPIC", "-shared", SRC, "-o", tmp], check=True)
        os.replace(tmp, SO)
    return SO


def measure(device, iters: int = 20000, reps: int = 5) -> dict:
    import torch
    l = ctypes.CDLL(build())
    l.ctgb_peak_ffma.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    props = torch.cuda.get_device_properties(device)
    sms = props.multi_processor_count
    blocks = sms * 8
    out = torch.empty(blocks * 256, device=device)
    st = torch.cuda.current_stream(device)
    per_iter = l.ctgb_peak_ffma_per_iter()
    for _ in range(2):
        l.ctgb_peak_ffma(blocks, iters, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.cuda_stream))
    best = None
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        l.ctgb_peak_ffma(blocks, iters, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.cuda_stream))
        b.record(st)
        torch.cuda.synchronize(device)
        ms = a.elapsed_time(b)
        best = ms if best is None else min(best, ms)
    fmas = blocks * 256 * iters * per_iter
    return {"lane_ops_per_s": fmas / (best / 1e3), "sms": sms, "ms": best,
            "note": "FFMA lane-ops/s, best of %d, %d blocks x 256 threads" % (reps, blocks)}
