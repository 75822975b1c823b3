"""The reference's own CUDA kernels, run on the GPU (TEST INFRASTRUCTURE ONLY).

The kernels of src/fan_ed_kernel.cu, src/fan_ea_kernel.cu and src/para_kernel.cu
are compiled unchanged for sm_103a by ``oracle/build.py:build_ref_gpu`` and
loaded here through the CUDA driver API (ctypes on libcuda), into the context
that PyTorch uses. Each call reproduces what the reference's host wrapper does
around its kernel (src/fan_ed_kernel.cu:1163-1331, src/fan_ea_kernel.cu:923-1057,
src/para_kernel.cu:685-807):

* grid (ceil(V/512) * B, min(V, 512), ceil(D/256)), 256 threads, no dynamic
  shared memory;
* argument 0 is the image as a ``PackedTensorAccessor<T, 4, RestrictPtrTraits,
  size_t>`` (B, 1, H, W) (for the single-view backprojection, (B, V, H, W)),
  argument 1 the projection (B, 1, V, D), then one device pointer per option
  into the options tensor, in its own order (``views`` = options[0] ... the
  fan geometries' ``binshift`` = options[10], the parallel one's = options[8]);
* projection outputs are left uninitialised (``torch::empty``; here they are
  NaN-filled when ``poison`` is set, so an element the kernel never writes
  shows), image outputs are zero-filled (``torch::zeros``).

The accessor is passed by value as 72 bytes: the data pointer, then the four
sizes and the four strides as 64-bit integers, the layout of
``at::GenericPackedTensorAccessorBase``. Before the first launch of a kernel,
its parameter list is read back from the module (``cuFuncGetParamInfo``) and
checked against exactly this list of sizes and offsets; a mismatch raises
instead of launching.

Only the tests and ``bench.py --impl reference`` use this module: it is the
reference arm, never part of the product path.
"""

from __future__ import annotations

import ctypes
import gzip
import math
import os
import re

from . import build as _build

GRID_DIM, BLOCK_DIM = 512, 256  # src/fan_ed_kernel.cu:4-5
OPS = {0: "prj", 1: "prj_t", 2: "bprj", 3: "bprj_t", 5: "bprj_sv"}
SCAN_NS = {0: "ref_fan_ed", 1: "ref_fan_ea", 2: "ref_para"}
SCAN_SUFFIX = {0: "fan_ed", 1: "fan_ea", 2: "para"}
ACC_BYTES = 72

_inst = None


def available() -> bool:
    return all(os.path.exists(_build.ref_cubin_path(ns)) for ns in SCAN_NS.values())


def laplacian_available() -> bool:
    return os.path.exists(_build.ref_cubin_path(_build.REF_GPU_LAPLACIAN[0]))


class _Driver:
    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        L = self.lib
        vp, u32, sz = ctypes.c_void_p, ctypes.c_uint, ctypes.c_size_t
        sig = {
            "cuInit": [u32],
            "cuCtxGetCurrent": [ctypes.POINTER(vp)],
            "cuModuleLoadData": [ctypes.POINTER(vp), vp],
            "cuModuleGetFunctionCount": [ctypes.POINTER(u32), vp],
            "cuModuleEnumerateFunctions": [ctypes.POINTER(vp), u32, vp],
            "cuFuncGetName": [ctypes.POINTER(ctypes.c_char_p), vp],
            "cuFuncGetParamInfo": [vp, sz, ctypes.POINTER(sz), ctypes.POINTER(sz)],
            "cuLaunchKernel": [vp, u32, u32, u32, u32, u32, u32, u32, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)],
            "cuGetErrorName": [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        self.check(L.cuInit(0), "cuInit")

    def check(self, rc: int, what: str):
        if rc != 0:
            s = ctypes.c_char_p()
            self.lib.cuGetErrorName(rc, ctypes.byref(s))
            raise RuntimeError(f"{what} failed: {rc} ({(s.value or b'?').decode()})")


def _demangle_head(name: str):
    """(kernel, 'f'|'d') from an Itanium-mangled template kernel name
    ``_Z<len><name>I<f|d>E...``; None for anything else."""
    m = re.match(r"_Z(\d+)", name)
    if not m:
        return None
    n = int(m.group(1))
    start = m.end()
    base = name[start:start + n]
    rest = name[start + n:]
    if len(base) != n or not rest.startswith("I") or len(rest) < 3 or rest[2] != "E":
        return None
    return base, rest[1]


class RefCuda:
    """Loaded reference modules in the current device's primary context."""

    def __init__(self, device=None):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device")
        if not available():
            raise RuntimeError("reference cubins not built (oracle/build.py:build_ref_gpu)")
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        torch.zeros(1, device=self.device)  # make the runtime's primary context current
        self.drv = _Driver()
        ctx = ctypes.c_void_p()
        self.drv.check(self.drv.lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context after torch initialisation")
        self.funcs = {}
        self.checked = set()
        self._modules = []
        for scan, ns in SCAN_NS.items():
            self._load_module(scan, ns)
        if laplacian_available():
            self._load_module("laplacian", _build.REF_GPU_LAPLACIAN[0])
        self._cublas = None

    def _load_module(self, key, ns):
        with gzip.open(_build.ref_cubin_path(ns), "rb") as f:
            image = f.read()
        buf = ctypes.create_string_buffer(image, len(image))
        mod = ctypes.c_void_p()
        self.drv.check(self.drv.lib.cuModuleLoadData(ctypes.byref(mod), buf), f"cuModuleLoadData({ns})")
        self._modules.append((mod, buf))
        cnt = ctypes.c_uint()
        self.drv.check(self.drv.lib.cuModuleGetFunctionCount(ctypes.byref(cnt), mod), "cuModuleGetFunctionCount")
        arr = (ctypes.c_void_p * cnt.value)()
        self.drv.check(self.drv.lib.cuModuleEnumerateFunctions(arr, cnt.value, mod), "cuModuleEnumerateFunctions")
        for fn in arr:
            nm = ctypes.c_char_p()
            self.drv.check(self.drv.lib.cuFuncGetName(ctypes.byref(nm), fn), "cuFuncGetName")
            head = _demangle_head(nm.value.decode())
            if head is not None:
                self.funcs[(key,) + head] = ctypes.c_void_p(fn)

    # -- parameter checks ------------------------------------------------------
    def _check_params(self, fn, key, sizes):
        if key in self.checked:
            return
        off_expect = 0
        for i, s in enumerate(sizes):
            off, size = ctypes.c_size_t(), ctypes.c_size_t()
            self.drv.check(self.drv.lib.cuFuncGetParamInfo(fn, i, ctypes.byref(off), ctypes.byref(size)),
                           f"cuFuncGetParamInfo({key}, {i})")
            al = min(s, 8)
            off_expect = (off_expect + al - 1) // al * al
            if size.value != s or off.value != off_expect:
                raise RuntimeError(f"{key}: parameter {i} is {size.value} bytes at {off.value}, "
                                   f"expected {s} at {off_expect}")
            off_expect += s
        off, size = ctypes.c_size_t(), ctypes.c_size_t()
        if self.drv.lib.cuFuncGetParamInfo(fn, len(sizes), ctypes.byref(off), ctypes.byref(size)) == 0:
            raise RuntimeError(f"{key}: more than {len(sizes)} parameters")
        self.checked.add(key)

    def _kernel(self, scan, base, tcode, sizes):
        key = (scan, base, tcode)
        if key not in self.funcs:
            raise RuntimeError(f"reference kernel {base}<{tcode}> not in the module")
        fn = self.funcs[key]
        self._check_params(fn, key, sizes)
        return fn

    @staticmethod
    def _acc(t):
        assert t.dim() == 4 and t.is_contiguous()
        return (ctypes.c_uint64 * 9)(t.data_ptr(), *[int(s) for s in t.shape], *[int(s) for s in t.stride()])

    def _launch(self, fn, grid, block, args, stream):
        bx, by = (block, 1) if isinstance(block, int) else block
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self.drv.check(self.drv.lib.cuLaunchKernel(fn, grid[0], grid[1], grid[2], bx, by, 1, 0,
                                                   ctypes.c_void_p(stream), params, None), "cuLaunchKernel")

    # -- operators -------------------------------------------------------------
    def run(self, op: int, x, options, poison: bool = False, out=None):
        """One reference operator call on ``x`` (on this device) with ``options``
        (a 1-D tensor of the reference's option list, on this device, of x's
        dtype). Returns the output tensor; launches on the current stream."""
        torch = self.torch
        if op not in OPS:
            raise ValueError(f"unknown op {op}")
        if x.device != self.device or options.device != self.device:
            raise ValueError("x and options must be on the module's device")
        if x.dtype not in (torch.float32, torch.float64) or options.dtype != x.dtype:
            raise ValueError("x and options must both be float32 or both float64")
        if options.dim() != 1 or not x.is_contiguous() or not options.is_contiguous():
            raise ValueError("contiguous x and 1-D options expected")
        h = options.detach().to("cpu", torch.float64).tolist()
        # the scan type is the last entry (src/ctlib.cpp:18); the fan kernels
        # read options[0..10], the parallel ones options[0..8]
        scan = int(h[-1]) if h else -1
        if scan not in SCAN_NS or len(h) < (9 if scan == 2 else 11):
            raise ValueError("options must end with the scan type and hold at least 11 values (fan) "
                             "or 9 (parallel)")
        if op == 5 and scan != 0:
            raise ValueError("single-view backprojection exists for the equal-distance fan geometry only")
        V, D, W, H = (int(h[i]) for i in range(4))
        if min(V, D, W, H) <= 0 or x.dim() != 4:
            raise ValueError("bad sizes")
        B = x.shape[0]
        img_in = op in (0, 3)
        want = (B, 1, H, W) if img_in else (B, 1, V, D)
        if tuple(x.shape) != want:
            raise ValueError(f"input shape {tuple(x.shape)} does not match the options' {want}")
        if img_in:
            oshape = (B, 1, V, D)
            out = torch.full(oshape, math.nan, dtype=x.dtype, device=self.device) if poison \
                else torch.empty(oshape, dtype=x.dtype, device=self.device)
            img, prj = x, out
        else:
            oshape = (B, V, H, W) if op == 5 else (B, 1, H, W)
            out = torch.zeros(oshape, dtype=x.dtype, device=self.device)
            img, prj = out, x
        nptr = 9 if scan == 2 else 11
        tcode = "f" if x.dtype == torch.float32 else "d"
        base = f"{OPS[op]}_{SCAN_SUFFIX[scan]}"
        fn = self._kernel(scan, base, tcode, [ACC_BYTES, ACC_BYTES] + [8] * nptr)
        es = x.element_size()
        args = [self._acc(img), self._acc(prj)] + [ctypes.c_uint64(options.data_ptr() + i * es)
                                                   for i in range(nptr)]
        grid = (math.ceil(V / GRID_DIM) * B, min(V, GRID_DIM), math.ceil(D / BLOCK_DIM))
        if grid[0] >= 2 ** 31:
            raise ValueError("batch too large for the reference's grid")
        self._launch(fn, grid, BLOCK_DIM, args, torch.cuda.current_stream(self.device).cuda_stream)
        return out

    def ramp(self, scan: int, dets, d):
        """The reference's rlfilter kernel: 2D-1 Ram-Lak taps for pitch ``d``
        (``dets`` and ``d`` are 0-d device tensors of the output dtype)."""
        torch = self.torch
        D = int(dets.item())
        filt = torch.empty((1, 1, 1, 2 * D - 1), dtype=dets.dtype, device=self.device)
        tcode = "f" if dets.dtype == torch.float32 else "d"
        fn = self._kernel(scan, "rlfilter", tcode, [8, 8, 8])
        args = [ctypes.c_uint64(filt.data_ptr()), ctypes.c_uint64(dets.data_ptr()), ctypes.c_uint64(d.data_ptr())]
        self._launch(fn, (math.ceil((2 * D - 1) / BLOCK_DIM), 1, 1), BLOCK_DIM, args,
                     torch.cuda.current_stream(self.device).cuda_stream)
        return filt

    def fbp(self, projection, options):
        """The reference's fbp: detector weighting, rlfilter taps, a conv2d with
        padding D-1, the backprojection kernel and the dAng/2 scale, step by
        step as in src/fan_ed_kernel.cu:1335-1382, src/fan_ea_kernel.cu:1059-1105
        and src/para_kernel.cu:809-850. The convolution is torch's, under the
        process's cuDNN settings (TF32 allowed for fp32 by default), as for the
        reference."""
        torch = self.torch
        h = options.detach().to("cpu", torch.float64).tolist()
        scan = int(h[-1])
        o = options
        D = int(h[1])
        kw = dict(dtype=projection.dtype, device=self.device)
        if scan == 0:
            s2r, d2r, dDet = o[8], o[9], o[5]
            virdDet = dDet * s2r / (s2r + d2r)
            rw = torch.arange(-D / 2 + 0.5, D / 2, 1, **kw) * virdDet
            rw = torch.pow(rw, 2).view(1, 1, 1, D)
            rw = s2r / torch.sqrt(s2r * s2r + rw)
            weighted = projection * rw * virdDet
            filt = self.ramp(0, o[1], virdDet)
        elif scan == 1:
            s2r, dDet = o[8], o[5]
            rw = torch.arange(-D / 2 + 0.5, D / 2, 1, **kw) * dDet
            rw = (torch.cos(rw) * s2r * dDet).view(1, 1, 1, D)
            weighted = projection * rw
            filt = self.ramp(1, o[1], dDet)
        else:
            weighted = projection * o[5]
            filt = self.ramp(2, o[1], o[5])
        filtered = torch.nn.functional.conv2d(weighted, filt, None, 1, (0, D - 1)).contiguous()
        image = self.run(2, filtered, options)
        return image * o[7] / 2

    def laplacian(self, x, k: int):
        """The reference's laplacian (src/laplacian_cuda_kernel.cu:46-128) step by
        step: its compute_squared_norm and add_norm kernels (grids of 256 threads
        and of 16 x 16 threads), cuBLAS ``gemm(T, N, n, n, dim, -2, x, dim, x, dim,
        1, dist, n)`` on a fresh handle, then torch's topk, median, exp, row sums
        and a float32 sparse COO tensor."""
        torch = self.torch
        if not laplacian_available() or ("laplacian", "add_norm", "f") not in self.funcs:
            raise RuntimeError("reference laplacian cubin not built")
        if x.dim() != 2 or not x.is_contiguous() or x.dtype not in (torch.float32, torch.float64):
            raise ValueError("contiguous 2-D float32 or float64 points expected")
        n, dim = (int(v) for v in x.shape)
        if not 1 <= k <= n:
            raise ValueError("k must be in [1, n]")
        if self._cublas is None:
            self._cublas = _Cublas(torch, self.device)
        cb = self._cublas.lib
        f32 = x.dtype == torch.float32
        tcode = "f" if f32 else "d"
        stream = torch.cuda.current_stream(self.device).cuda_stream
        norm2 = torch.empty(n, dtype=x.dtype, device=self.device)
        dist = torch.empty((n, n), dtype=x.dtype, device=self.device)
        fn = self._kernel("laplacian", "compute_squared_norm", tcode, [40, 4, 4, 8])
        self._launch(fn, (math.ceil(n / 256), 1, 1), 256,
                     [_acc2(x), ctypes.c_int(n), ctypes.c_int(dim), ctypes.c_uint64(norm2.data_ptr())], stream)
        fn = self._kernel("laplacian", "add_norm", tcode, [40, 4, 8])
        nb = math.ceil(n / 16)
        self._launch(fn, (nb, nb, 1), (16, 16), [_acc2(dist), ctypes.c_int(n), ctypes.c_uint64(norm2.data_ptr())],
                     stream)
        h = ctypes.c_void_p()
        if cb.cublasCreate_v2(ctypes.byref(h)) != 0:
            raise RuntimeError("cublasCreate failed")
        try:
            t = ctypes.c_float if f32 else ctypes.c_double
            gemm = cb.cublasSgemm_v2 if f32 else cb.cublasDgemm_v2
            alpha, beta = t(-2.0), t(1.0)
            rc = gemm(h, 1, 0, n, n, dim, ctypes.byref(alpha), ctypes.c_void_p(x.data_ptr()), dim,
                      ctypes.c_void_p(x.data_ptr()), dim, ctypes.byref(beta), ctypes.c_void_p(dist.data_ptr()), n)
            if rc != 0:
                raise RuntimeError(f"cuBLAS gemm failed: {rc}")
        finally:
            cb.cublasDestroy_v2(h)
        coef, indj = torch.topk(dist, k, 1, False)
        median = torch.median(coef)
        coef = coef / median
        coef = torch.exp(-coef)
        coef = coef / coef.sum(1, True)
        coef = coef.view(-1)
        indi = torch.arange(n, dtype=torch.int64, device=self.device).unsqueeze_(1).repeat(1, k)
        ind1 = torch.stack([indi, indj]).view(2, -1)
        return torch.sparse_coo_tensor(ind1, coef, (n, n), dtype=torch.float32, device=self.device)

class _Cublas:
    """The cuBLAS library that PyTorch loaded (found through the process's
    mapped files after one matmul), for the reference's GEMM calls."""

    def __init__(self, torch, device):
        a = torch.ones(2, 2, device=device)
        (a @ a).sum().item()
        path = None
        with open("/proc/self/maps") as f:
            for line in f:
                part = line.split()[-1]
                if "libcublas.so" in os.path.basename(part):
                    path = part
                    break
        if path is None:
            raise RuntimeError("libcublas not loaded by torch")
        L = self.lib = ctypes.CDLL(path)
        vp, ci = ctypes.c_void_p, ctypes.c_int
        L.cublasCreate_v2.argtypes = [ctypes.POINTER(vp)]
        L.cublasDestroy_v2.argtypes = [vp]
        for name, t in (("cublasSgemm_v2", ctypes.c_float), ("cublasDgemm_v2", ctypes.c_double)):
            fn = getattr(L, name)
            fn.argtypes = [vp, ci, ci, ci, ci, ci, ctypes.POINTER(t), vp, ci, vp, ci, ctypes.POINTER(t), vp, ci]
            fn.restype = ci
        L.cublasCreate_v2.restype = ci
        L.cublasDestroy_v2.restype = ci


def _acc2(t):
    assert t.dim() == 2 and t.is_contiguous()
    return (ctypes.c_uint64 * 5)(t.data_ptr(), *[int(s) for s in t.shape], *[int(s) for s in t.stride()])




def get() -> RefCuda:
    global _inst
    if _inst is None:
        _inst = RefCuda()
    return _inst
