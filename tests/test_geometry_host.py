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


@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("opts", CASES)
def test_split_line_maps_exact_high_part(native, opts, dtype):
    """The image gather forms a pixel edge as (fma(sigma_hi, k, alpha_hi),
    fma(sigma_lo, k, alpha_lo)): the high parts lie on one power-of-two grid per
    line, so alpha_hi + sigma_hi * k is exact in the plan's type for every edge k
    of the line, and the pair sums to alpha + sigma * k to the type's precision
    (checked on up to 16 views of each case, every line)."""
    V, D, W, H = (int(opts[i]) for i in range(4))
    L = max(W, H)
    lp = _query(native, opts, 3, dtype=dtype).reshape(V, L, 2)  # the plan's own geometry
    sp = _query(native, opts, 7, dtype=dtype).reshape(V, L, 4)
    flags = _query(native, opts, 0).astype(int)
    bits = 24 if dtype == 0 else 53
    for v in range(0, V, max(1, V // 16)):
        K = W if flags[v] & 1 else H
        used = lp[v, :, 1] > 0
        alpha, sigma = lp[v, used, 0], lp[v, used, 1]
        ah, al, sh, sl = (sp[v, used, j] for j in range(4))
        if dtype == 0:
            for x in (ah, al, sh, sl):
                assert np.array_equal(x.astype(np.float32).astype(np.float64), x)
        # the grid: 2^(exponent of the line's largest edge magnitude + 2 - bits)
        M = np.maximum.reduce([np.abs(alpha), np.abs(alpha + sigma * K), sigma * K])
        q = np.ldexp(1.0, np.frexp(M)[1] + 1 - bits)
        A, S = ah / q, sh / q
        assert np.array_equal(A, np.round(A)) and np.array_equal(S, np.round(S))
        A, S = A.astype(np.int64), S.astype(np.int64)
        edge_hi_max = np.maximum(np.abs(A), np.abs(A + S * K))  # alpha_hi + sigma_hi k is monotone in k
        assert (edge_hi_max < 2 ** bits).all()  # every edge's high part is exact
        k = np.arange(K + 1)[None, :]
        got = (ah[:, None] + sh[:, None] * k) + (al[:, None] + sl[:, None] * k)
        want = alpha[:, None] + sigma[:, None] * k
        scale = np.abs(want).max(axis=1) + sigma
        # fp32: the low parts carry the edge to ~2^-38; fp64: the check itself
        # rounds in double (a few units in the last place)
        tol = 2.0 ** -36 if dtype == 0 else 2.0 ** -50
        assert (np.abs(got - want).max(axis=1) <= tol * scale).all(), v
