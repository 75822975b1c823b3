"""ctypes bindings to the CPU oracle and to the CPU-executed reference kernels.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the CPU-baseline leg of ``bench.py``. The product package never imports it.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

OP_PRJ, OP_PRJ_T, OP_BPRJ, OP_BPRJ_T, OP_FBP, OP_RAMP, OP_BPRJ_SV = 0, 1, 2, 3, 4, 5, 6
OP_NAMES = {"projection": OP_PRJ, "projection_t": OP_PRJ_T, "backprojection": OP_BPRJ,
            "backprojection_t": OP_BPRJ_T, "fbp": OP_FBP, "backprojection_sv": OP_BPRJ_SV}

# modes of oracle_run
MODE_F32 = 0      # fp32 data and arithmetic, reference promotions
MODE_F64 = 1      # fp64 data and arithmetic
MODE_F64_ON_F32 = 2  # fp64 arithmetic, fp32 view angles (FP64 oracle for fp32 inputs)

_lib = None
_ref = None


def _load_oracle():
    global _lib
    if _lib is None:
        path = _build.ORACLE_SO
        if not os.path.exists(path):
            path = _build.build_oracle()
        lib = ctypes.CDLL(path)
        lib.oracle_run.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int]
        lib.oracle_run.restype = ctypes.c_int
        lib.oracle_set_filter.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.oracle_set_filter.restype = ctypes.c_int
        lib.oracle_view_flags.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def ref_available() -> bool:
    return os.path.exists(_build.REF_SO) or _build.ref_root() is not None


def _load_ref():
    global _ref
    if _ref is None:
        path = _build.REF_SO if os.path.exists(_build.REF_SO) else _build.build_ref()
        if path is None:
            raise RuntimeError("reference checkout not available")
        lib = ctypes.CDLL(path)
        lib.ref_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.ref_run.restype = ctypes.c_int
        lib.ref_ramp.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
        lib.ref_ramp.restype = ctypes.c_int
        lib.ref_oob_count.restype = ctypes.c_long
        _ref = lib
    return _ref


def _opts_array(opts):
    o = np.ascontiguousarray(np.asarray(opts, dtype=np.float64).ravel())
    return o, o.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def out_shape(op: int, opts, batch: int):
    o = np.asarray(opts, dtype=np.float64).ravel()
    V, D, W, H = int(o[0]), int(o[1]), int(o[2]), int(o[3])
    if op in (OP_PRJ, OP_BPRJ_T):
        return (batch, 1, V, D)
    if op == OP_BPRJ_SV:  # one image per view (fan equal-distance only)
        return (batch, V, H, W)
    return (batch, 1, H, W)


def run(op, x: np.ndarray, opts, mode: int = MODE_F64_ON_F32, threads: int = 0) -> np.ndarray:
    """Run one operator of the oracle. ``x`` is B x 1 x H x W or B x 1 x V x D."""
    if isinstance(op, str):
        op = OP_NAMES[op]
    lib = _load_oracle()
    dt = np.float32 if mode == MODE_F32 else np.float64
    xin = np.ascontiguousarray(x, dtype=dt)
    batch = xin.shape[0]
    out = np.empty(out_shape(op, opts, batch), dtype=dt)
    o, op_ptr = _opts_array(opts)
    rc = lib.oracle_run(op, op_ptr, o.size, mode, batch, xin.ctypes.data, out.ctypes.data, threads)
    if rc != 0:
        raise ValueError(f"oracle_run failed with code {rc}")
    return out


FILTERS = {"ram-lak": 0, "shepp-logan": 1, "hann": 2}


def fbp(x: np.ndarray, opts, mode: int = MODE_F64_ON_F32, filter: str = "ram-lak", ea_exact: bool = False,
        threads: int = 0) -> np.ndarray:
    """fbp with a chosen filter window (and the exact equal-angle kernel);
    the defaults are the reference's Ram-Lak filter."""
    lib = _load_oracle()
    if lib.oracle_set_filter(FILTERS[filter], int(bool(ea_exact))) != 0:
        raise ValueError(filter)
    try:
        return run(OP_FBP, x, opts, mode, threads)
    finally:
        lib.oracle_set_filter(0, 0)


def view_flags(opts, mode: int = MODE_F32):
    lib = _load_oracle()
    o, op_ptr = _opts_array(opts)
    V = int(o[0])
    xb = np.zeros(V, np.int32)
    fl = np.zeros(V, np.int32)
    if lib.oracle_view_flags(op_ptr, o.size, mode, xb.ctypes.data, fl.ctypes.data) != 0:
        raise ValueError("bad options")
    return xb.astype(bool), fl.astype(bool)


def max_threads() -> int:
    return int(_load_oracle().oracle_max_threads())


# operator numbers of the reference driver (oracle/ref_emu/ref_driver.inc)
REF_OPS = {"projection": 0, "projection_t": 1, "backprojection": 2, "backprojection_t": 3, "backprojection_sv": 5}


def ref_run(op, x: np.ndarray, opts, dtype=np.float32) -> np.ndarray:
    """Run the reference's own kernel (CPU execution); ops 0-3 and 5 (single
    view), by driver number or by name."""
    if isinstance(op, str):
        op = REF_OPS[op]
    lib = _load_ref()
    xin = np.ascontiguousarray(x, dtype=dtype)
    batch = xin.shape[0]
    o, op_ptr = _opts_array(opts)
    if op == 5:
        V, W, H = int(o[0]), int(o[2]), int(o[3])
        shape = (batch, V, H, W)
    else:
        shape = out_shape(op, opts, batch)
    out = np.empty(shape, dtype=dtype)
    rc = lib.ref_run(op, 0 if dtype == np.float32 else 1, op_ptr, o.size, batch, xin.ctypes.data,
                     out.ctypes.data)
    if rc != 0:
        raise ValueError(f"ref_run failed with code {rc}")
    return out


def ref_ramp(scan: int, dets: int, d: float, dtype=np.float32) -> np.ndarray:
    lib = _load_ref()
    out = np.empty(2 * dets - 1, dtype=dtype)
    rc = lib.ref_ramp(scan, 0 if dtype == np.float32 else 1, dets, float(d), out.ctypes.data)
    if rc != 0:
        raise ValueError("ref_ramp failed")
    return out


def ref_oob_count() -> int:
    return int(_load_ref().ref_oob_count())


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
