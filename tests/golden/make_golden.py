"""Generate tests/golden/*.npz from the reference's own kernels.

Runs in a container that has the CTLIB checkout: ``oracle.build.build_ref()``
compiles the reference kernel source for CPU execution (oracle/ref_emu) and this
script records inputs and outputs for a set of small geometries plus reduced
copies of the benchmark workloads. For ``fbp`` the host-side glue of the
reference wrapper (src/fan_ed_kernel.cu:1348-1380, src/fan_ea_kernel.cu:1074-1105,
src/para_kernel.cu:822-847) is replayed with CPU torch tensor ops in the same
order; the ramp taps come from the reference's ``rlfilter`` kernel and the
filtering convolution is evaluated in fp64 (i.e. cuDNN with TF32 disabled).

    python tests/golden/make_golden.py
"""

from __future__ import annotations

import math
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402
from ctlib_gb300.workloads import (FAN_EA, FAN_ED, PARA, ellipse_phantom, fan_options,  # noqa: E402
                                   gaussian, para_options)

OPS4 = ("projection", "projection_t", "backprojection", "backprojection_t")


def ref_fbp(sino: np.ndarray, opts) -> np.ndarray:
    scan = int(opts[-1])
    V, D = int(opts[0]), int(opts[1])
    dt = torch.float32 if sino.dtype == np.float32 else torch.float64
    t = torch.from_numpy(sino)
    o = torch.tensor(opts, dtype=dt)
    dets, dDet, dAng = o[1], o[5], o[7]
    ar = torch.arange(-float(dets.item()) / 2 + 0.5, float(dets.item()) / 2, 1, dtype=dt)
    if scan == FAN_ED:
        s2r, d2r = o[8], o[9]
        virdDet = dDet * s2r / (s2r + d2r)
        rw = ar * virdDet
        rw = torch.pow(rw, 2)
        rw = rw.view(1, 1, 1, D)
        rw = s2r / torch.sqrt(s2r * s2r + rw)
        rect = t * rw * virdDet
        dfilt = float(virdDet.item())
    elif scan == FAN_EA:
        s2r = o[8]
        rw = ar * dDet
        rw = torch.cos(rw)
        rw = rw * s2r * dDet
        rw = rw.view(1, 1, 1, D)
        rect = t * rw
        dfilt = float(dDet.item())
    else:
        rect = t * dDet
        dfilt = float(dDet.item())
    taps = O.ref_ramp(scan, D, dfilt, sino.dtype.type)
    filt = torch.nn.functional.conv2d(rect.double(), torch.from_numpy(taps).double().view(1, 1, 1, -1),
                                      padding=(0, D - 1)).to(dt)
    img = O.ref_run("backprojection", filt.numpy(), opts, sino.dtype.type)
    out = torch.from_numpy(img) * dAng / 2
    return out.numpy(), taps


def small_cases():
    tp = 2 * math.pi
    return [
        # name, options, batch, dtype
        ("ed_small", fan_options(60, 90, 64, 64, 1.0, 2.0, 0.0, tp / 60, 120.0, 100.0, 0.0, FAN_ED), 2,
         np.float32),
        ("ed_rect_odd_shift", fan_options(72, 91, 48, 40, 1.0, 2.0, 0.3, tp / 72, 120.0, 100.0, 1.5, FAN_ED),
         1, np.float32),
        ("ed_wide_det", fan_options(40, 300, 64, 64, 1.0, 0.9, 0.1, tp / 40, 120.0, 100.0, -0.7, FAN_ED), 1,
         np.float32),
        ("ed_f64", fan_options(60, 90, 64, 64, 1.0, 2.0, 0.2, tp / 60, 120.0, 100.0, 0.5, FAN_ED), 1,
         np.float64),
        ("ea_small", fan_options(60, 90, 64, 64, 1.0, 0.008, 0.0, tp / 60, 120.0, 100.0, 0.0, FAN_EA), 2,
         np.float32),
        ("ea_rect_odd_shift", fan_options(72, 91, 48, 40, 1.0, 0.008, 0.3, tp / 72, 120.0, 100.0, 0.01,
                                          FAN_EA), 1, np.float32),
        ("ea_wide_det", fan_options(40, 300, 64, 64, 1.0, 0.0026, 0.1, tp / 40, 120.0, 100.0, -0.004,
                                    FAN_EA), 1, np.float32),
        ("para_small", para_options(60, 90, 64, 64, 1.0, 1.1, 0.0, math.pi / 60, 0.0), 2, np.float32),
        ("para_rect_odd_shift", para_options(72, 91, 48, 40, 1.0, 1.1, 0.3, math.pi / 72, 1.5), 1,
         np.float32),
        ("para_wide_det_360", para_options(40, 300, 64, 64, 1.0, 0.35, 0.1, tp / 40, -0.7), 1, np.float32),
        # README's 9-entry parallel vector: options[8] is both binshift and scan_type (= 2.0)
        ("para_nine_entry", [60.0, 90.0, 64.0, 64.0, 1.0, 1.1, 0.0, math.pi / 60, 2.0], 1, np.float32),
    ]


def scaled_cases():
    tp = 2 * math.pi
    return [
        ("cfg_parallel_256", para_options(360, 367, 256, 256, 1.0, 1.0, 0.0, math.pi / 360, 0.0), 1,
         np.float32),
        ("cfg_fan_ed_half", fan_options(576, 368, 256, 256, 1.3282, 2.5716, 0.0, tp / 576, 595.0, 490.6, 0.0,
                                        FAN_ED), 1, np.float32),
        ("cfg_fan_ea_half", fan_options(492, 444, 256, 256, 1.4, 0.0022, 0.0, tp / 492, 541.0, 408.0, 0.0,
                                        FAN_EA), 1, np.float32),
    ]


def make(name, opts, batch, dtype, ops=OPS4 + ("fbp",)):
    V, D, W, H = (int(opts[i]) for i in range(4))
    dImg = opts[4]
    img = np.stack([ellipse_phantom(H, W, dImg, 900 + i) for i in range(batch)])[:, None].astype(dtype)
    gs = gaussian((batch, 1, V, D), 7).astype(dtype)
    rec = {"options": np.asarray(opts, np.float64)}
    sino_ref = None
    for op in ops:
        if op in ("projection", "backprojection_t"):
            x = img
        elif op == "fbp":
            x = sino_ref if sino_ref is not None else O.ref_run("projection", img, opts, dtype)
        else:
            x = gs
        if op == "backprojection_sv":
            continue
        if op == "fbp":
            y, taps = ref_fbp(x, opts)
            rec["ramp_taps"] = taps
        else:
            y = O.ref_run(op, x, opts, dtype)
        if op == "projection":
            sino_ref = y
        assert O.ref_oob_count() == 0, name
        assert np.isfinite(y).all(), (name, op)
        rec[f"{op}_in"] = x
        rec[f"{op}_out"] = y
    if "backprojection_sv" in ops:
        rec["backprojection_sv_in"] = gs
        rec["backprojection_sv_out"] = O.ref_run(5, gs, opts, dtype)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **rec)
    print(f"{name}: {os.path.getsize(path) / 1e3:.0f} kB")


def single_view_cases():
    """Single-view backprojection (fan ED only): output B x V x H x W."""
    tp = 2 * math.pi
    sv = ("backprojection_sv",)
    return [
        ("ed_single_view", fan_options(12, 40, 32, 32, 1.0, 2.0, 0.0, tp / 12, 120.0, 100.0, 0.0, FAN_ED), 1,
         np.float32, sv),
        # H != W, start angle and bin shift, two slices
        ("ed_single_view_rect", fan_options(24, 61, 40, 28, 1.0, 2.0, 0.3, tp / 24, 120.0, 100.0, 0.7, FAN_ED), 2,
         np.float32, sv),
        # fp64, 300 bins: two 256-bin reference blocks per view
        ("ed_single_view_f64", fan_options(16, 300, 48, 48, 1.0, 0.5, 0.1, tp / 16, 120.0, 100.0, 0.2, FAN_ED), 1,
         np.float64, sv),
    ]


def main(names=None):
    """Write every fixture, or only those named on the command line."""
    want = (lambda n: True) if not names else (lambda n: n in names)
    for c in small_cases():
        if want(c[0]):
            make(*c)
    for c in single_view_cases():
        if want(c[0]):
            make(*c)
    for name, opts, batch, dtype in scaled_cases():
        if want(name):
            ops = OPS4 + ("fbp",) if name == "cfg_parallel_256" else ("projection", "projection_t", "fbp")
            make(name, opts, batch, dtype, ops)


if __name__ == "__main__":
    main(sys.argv[1:])
