"""Build and load ``libctgb.so`` (the sm_103a kernels behind include/ctgb.h).

The library is compiled in-tree with nvcc (``build()``); ``lib()`` loads it with
ctypes. There is no fallback: if the library is missing or fails to load, every
operator raises.
"""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD_DIR = os.path.join(PKG, "_build")
SO_PATH = os.path.join(BUILD_DIR, "libctgb.so")
INCLUDE = os.path.join(ROOT, "include")
SOURCES = [os.path.join(CSRC, "ctgb_kernels.cu"), os.path.join(CSRC, "ctgb_laplacian.cu"),
           os.path.join(CSRC, "geometry.cpp")]
HEADERS = [os.path.join(INCLUDE, "ctgb.h"), os.path.join(CSRC, "geometry.h"), os.path.join(CSRC, "ctgb_internal.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

OK, ERR_INVALID, ERR_CUDA, ERR_WORKSPACE = 0, 1, 2, 3
FLOAT32, FLOAT64 = 0, 1
OP_PROJECTION, OP_PROJECTION_T, OP_BACKPROJECTION, OP_BACKPROJECTION_T, OP_FBP = 0, 1, 2, 3, 4
OP_BACKPROJECTION_SV = 5
OP_DATA_GRADIENT = 6  # workspace queries of ctgb_data_gradient

_lock = threading.Lock()
_lib = None


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; set NVCC or put the CUDA toolkit on PATH")


def _stale() -> bool:
    if not os.path.exists(SO_PATH):
        return True
    t = os.path.getmtime(SO_PATH)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libctgb.so for sm_103a (no-op when up to date)."""
    if not force and not _stale():
        return SO_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = SO_PATH + ".tmp"
    # host code (the plan builder) is compiled without FMA contraction so that
    # it rounds the same way on x86-64 and aarch64; fused operations it needs
    # are written as std::fma
    cmd = [nvcc(), ARCH, "-lineinfo", "-O3", "-std=c++17", "-I", INCLUDE, "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-shared", *SOURCES, "-o", tmp]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(tmp, SO_PATH)
    return SO_PATH


def _declare(l):
    c_int, c_size, vp = ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p
    dptr = ctypes.POINTER(ctypes.c_double)
    l.ctgb_plan_create.argtypes = [ctypes.POINTER(vp), dptr, c_int, c_int, c_int]
    l.ctgb_plan_create.restype = c_int
    l.ctgb_plan_destroy.argtypes = [vp]
    l.ctgb_plan_destroy.restype = c_int
    ip = ctypes.POINTER(c_int)
    l.ctgb_plan_info.argtypes = [vp, ip, ip, ip, ip, ip, ip]
    l.ctgb_plan_info.restype = c_int
    l.ctgb_plan_set_schedule.argtypes = [vp, c_int, c_int, c_int]
    l.ctgb_plan_set_schedule.restype = c_int
    l.ctgb_plan_set_unroll.argtypes = [vp, c_int, c_int]
    l.ctgb_plan_set_unroll.restype = c_int
    l.ctgb_plan_set_wait_limit.argtypes = [vp, ctypes.c_ulonglong]
    l.ctgb_plan_set_wait_limit.restype = c_int
    l.ctgb_plan_set_summation.argtypes = [vp, c_int]
    l.ctgb_plan_set_summation.restype = c_int
    l.ctgb_plan_set_filter.argtypes = [vp, c_int, c_int]
    l.ctgb_plan_set_filter.restype = c_int
    l.ctgb_plan_set_kernel_events.argtypes = [vp, vp, vp]
    l.ctgb_plan_set_kernel_events.restype = c_int
    l.ctgb_workspace_size.argtypes = [vp, c_int, c_int]
    l.ctgb_workspace_size.restype = c_size
    for name in ("ctgb_projection", "ctgb_projection_t", "ctgb_backprojection", "ctgb_backprojection_t",
                 "ctgb_fbp", "ctgb_backprojection_sv"):
        f = getattr(l, name)
        f.argtypes = [vp, vp, vp, c_int, vp, c_size, vp]
        f.restype = c_int
    l.ctgb_data_gradient.argtypes = [vp, vp, vp, vp, vp, c_int, vp, c_size, vp]
    l.ctgb_data_gradient.restype = c_int
    l.ctgb_laplacian_workspace_size.argtypes = [c_int, c_int, c_int, c_int]
    l.ctgb_laplacian_workspace_size.restype = c_size
    l.ctgb_laplacian.argtypes = [vp, c_int, c_int, c_int, c_int, vp, vp, vp, c_size, vp]
    l.ctgb_laplacian.restype = c_int
    l.ctgb_projection_noalloc.argtypes = [vp, vp, vp, c_int, vp]
    l.ctgb_projection_noalloc.restype = c_int
    l.ctgb_projection_noalloc_max_bytes.argtypes = []
    l.ctgb_projection_noalloc_max_bytes.restype = c_size
    pp = ctypes.POINTER(vp)
    l.ctgb_ragged_create.argtypes = [ctypes.POINTER(vp), pp, c_int, c_int]
    l.ctgb_ragged_create.restype = c_int
    l.ctgb_ragged_destroy.argtypes = [vp]
    l.ctgb_ragged_destroy.restype = c_int
    l.ctgb_ragged_workspace_size.argtypes = [vp, c_int]
    l.ctgb_ragged_workspace_size.restype = c_size
    l.ctgb_ragged_run.argtypes = [vp, c_int, pp, pp, vp, c_size, vp]
    l.ctgb_ragged_run.restype = c_int
    l.ctgb_last_error.argtypes = []
    l.ctgb_last_error.restype = ctypes.c_char_p
    l.ctgb_version.restype = c_int
    l.ctgb_geometry_query.argtypes = [dptr, c_int, c_int, c_int, dptr, c_size]
    l.ctgb_geometry_query.restype = ctypes.c_long
    l.ctgb_wait_timeouts.argtypes = [c_int, ctypes.POINTER(ctypes.c_ulonglong), c_int]
    l.ctgb_wait_timeouts.restype = c_int
    return l


def lib():
    """The loaded library; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(SO_PATH):
                    raise RuntimeError(
                        f"ctlib_gb300 native library not built ({SO_PATH} missing); "
                        "run `python -c 'import __graft_entry__ as g; g.build()'`")
                _lib = _declare(ctypes.CDLL(SO_PATH))
    return _lib


def last_error() -> str:
    msg = lib().ctgb_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str):
    if rc == OK:
        return
    msg = f"{what}: {last_error()}"
    if rc == ERR_INVALID:
        raise ValueError(msg)
    raise RuntimeError(msg)


EXPORTED = ("ctgb_plan_create", "ctgb_plan_destroy", "ctgb_plan_info", "ctgb_plan_set_schedule", "ctgb_plan_set_unroll", "ctgb_plan_set_filter",
            "ctgb_plan_set_summation", "ctgb_plan_set_wait_limit",
            "ctgb_plan_set_kernel_events",
            "ctgb_workspace_size",
            "ctgb_projection", "ctgb_projection_t", "ctgb_backprojection", "ctgb_backprojection_t",
            "ctgb_fbp", "ctgb_backprojection_sv", "ctgb_data_gradient", "ctgb_projection_noalloc", "ctgb_projection_noalloc_max_bytes", "ctgb_ragged_create",
            "ctgb_ragged_destroy", "ctgb_ragged_workspace_size", "ctgb_ragged_run", "ctgb_last_error",
            "ctgb_version", "ctgb_geometry_query", "ctgb_wait_timeouts", "ctgb_laplacian_workspace_size",
            "ctgb_laplacian")


def wait_timeouts(device: int = 0, reset: bool = False) -> int:
    """Bounded waits of the staged image gather that ran out on `device`
    (ctgb_wait_timeouts); 0 unless a copy pipeline stalled."""
    n = ctypes.c_ulonglong(0)
    check(lib().ctgb_wait_timeouts(int(device), ctypes.byref(n), int(bool(reset))), "wait counter")
    return int(n.value)
