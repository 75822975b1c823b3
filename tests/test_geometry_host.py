"""Host-side checks of libctgb.so that need no GPU: exported symbols, options
validation and the per-view geometry tables the kernels consume."""

import ctypes
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT

from ctlib_gb300.workloads import FAN_EA, FAN_ED, fan_options, para_options


@pytest.fixture(scope="module")
def native():
    from ctlib_gb300 import _native
    _native.build()
    return _native


def _query(native, opts, what, dtype=0):
    l = native.lib()
    o = (ctypes.c_double * len(opts))(*opts)
    n = l.ctgb_geometry_query(o, len(opts), dtype, what, None, 0)
    if n < 0:
        raise ValueError(native.last_error())
    out = (ctypes.c_double * n)()
    l.ctgb_geometry_query(o, len(opts), dtype, what, out, n)
    return np.frombuffer(out, dtype=np.float64).copy()


def test_header_symbols_exported(native):
    with open(os.path.join(ROOT, "include", "ctgb.h")) as f:
        hdr = f.read()
    declared = set(re.findall(r"\b(ctgb_[a-z_]+)\s*\(", hdr))
    assert declared, "no declarations found"
    assert declared == set(native.EXPORTED)
    l = native.lib()
    for name in declared:
        assert hasattr(l, name), name
    assert l.ctgb_version() == 1


CASES = [
    fan_options(60, 90, 64, 64, 1.0, 2.0, 0.0, 2 * math.pi / 60, 120.0, 100.0, 0.0, FAN_ED),
    fan_options(72, 91, 48, 40, 1.0, 2.0, 0.3, 2 * math.pi / 72, 120.0, 100.0, 1.5, FAN_ED),
    fan_options(1152, 736, 512, 512, 0.6641, 1.2858, 0.0, 2 * math.pi / 1152, 595.0, 490.6, 0.0, FAN_ED),
    fan_options(984, 888, 512, 512, 0.7, 0.0011, 0.0, 2 * math.pi / 984, 541.0, 408.0, 0.0, FAN_EA),
    fan_options(72, 91, 48, 40, 1.0, 0.008, 0.3, 2 * math.pi / 72, 120.0, 100.0, 0.01, FAN_EA),
    para_options(360, 367, 256, 256, 1.0, 1.0, 0.0, math.pi / 360, 0.0),
    para_options(72, 91, 48, 40, 1.0, 1.1, 0.3, 2 * math.pi / 72, 1.5),
]


@pytest.mark.parametrize("opts", CASES)
def test_flags_match_oracle(native, oracle_mod, opts):
    flags = _query(native, opts, 0).astype(int)
    xb, fl = oracle_mod.view_flags(opts, oracle_mod.MODE_F32)
    assert np.array_equal((flags & 1).astype(bool), xb)
    assert np.array_equal((flags & 2).astype(bool), fl)


@pytest.mark.parametrize("opts", CASES)
def test_boundaries_increasing_and_seed_accurate(native, opts):
    V, D, W, H = (int(opts[i]) for i in range(4))
    db = _query(native, opts, 1).reshape(V, D + 1)
    assert np.all(np.diff(db, axis=1) > 0)
    inv = _query(native, opts, 4).reshape(V, 5).astype(np.float32)
    scan = int(opts[-1])
    # seed at each cell midpoint lands within one cell of the true cell
    mid = (0.5 * (db[:, :-1] + db[:, 1:])).astype(np.float32)
    u = mid * inv[:, 0:1] / (inv[:, 1:2] + mid * inv[:, 2:3])
    if scan == FAN_EA:
        u = np.arctan(u)
    cb = inv[:, 3:4] + inv[:, 4:5] * u
    err = np.abs(np.floor(cb) - np.arange(D)[None, :])
    assert err.max() <= 1, err.max()


@pytest.mark.parametrize("opts", CASES)
def test_line_maps_reproduce_pixel_edges(native, opts):
    """alpha + sigma*k equals the projection of pixel edge k through the source
    (map_x / map_y, src/fan_ed_kernel.cu:8-15) or along the rays (parallel)."""
    V, D, W, H = (int(opts[i]) for i in range(4))
    L = max(W, H)
    lp = _query(native, opts, 3, dtype=1).reshape(V, L, 2)
    flags = _query(native, opts, 0).astype(int)
    dImg = opts[4]
    scan = int(opts[-1])
    for v in (0, V // 7, V // 3, V - 1):
        ang = v * opts[7] + opts[6]
        xb = bool(flags[v] & 1)
        line = (H // 3) if xb else (W // 3)
        k = np.arange((W if xb else H) + 1)
        got = lp[v, line, 0] + lp[v, line, 1] * k
        if scan == 2:
            if xb:
                y = (H / 2 - line - 0.5) * dImg
                want = math.tan(ang) * y + (-W / 2 + k) * dImg
            else:
                x = (line - W / 2 + 0.5) * dImg
                want = (-H / 2 + k) * dImg + x / math.tan(ang)
        else:
            R = opts[8]
            sx, sy = -math.sin(ang) * R, math.cos(ang) * R
            if xb:
                y = (H / 2 - line - 0.5) * dImg
                x = (-W / 2 + k) * dImg
                want = (sx * y - sy * x) / (y - sy)
            else:
                x = (line - W / 2 + 0.5) * dImg
                y = (-H / 2 + k) * dImg
                want = (sy * x - sx * y) / (x - sx)
        assert np.allclose(got, want, rtol=0, atol=1e-9 * max(1.0, np.abs(want).max())), (v, xb)
        assert lp[v, line, 1] > 0


@pytest.mark.parametrize("bad,msg", [
    ([60.0, 90.0, 64.0, 64.0, 1.0, 2.0, 0.0, 0.1, 120.0, 100.0, 0.0, 3.0], "scan_type"),
    ([60.0, 90.0, 64.0, 64.0, 1.0, 2.0, 0.0, 0.1, 120.0, 100.0, 0.0], "12 entries"),
    ([60.0, 90.5, 64.0, 64.0, 1.0, 2.0, 0.0, 0.1, 120.0, 100.0, 0.0, 0.0], "positive integers"),
    ([60.0, 90.0, 64.0, 64.0, 1.0, 2.0, 0.0, 0.1, 20.0, 100.0, 0.0, 0.0], "inside"),
    ([60.0, 90.0, 64.0, 64.0, -1.0, 2.0, 0.0, 0.1, 0.0, 2.0], "positive"),
])
def test_invalid_options_rejected(native, bad, msg):
    with pytest.raises(ValueError, match=msg):
        _query(native, bad, 0)


def test_fbp_tables_match_reference_taps(native, oracle_mod):
    import glob
    for f in glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")):
        z = np.load(f)
        if "ramp_taps" not in z:
            continue
        dt = 0 if z["ramp_taps"].dtype == np.float32 else 1
        taps = _query(native, list(z["options"]), 6, dtype=dt)
        assert np.array_equal(taps.astype(z["ramp_taps"].dtype), z["ramp_taps"]), f
