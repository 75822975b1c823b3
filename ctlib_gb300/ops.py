"""Drop-in replacements for the functions of CTLIB's ``ctlib`` module.

``projection``, ``projection_t``, ``backprojection``, ``backprojection_t``,
``fbp`` and ``backprojection_sv`` take and return the same tensors as the
reference (src/ctlib.cpp:15-99): images ``B x 1 x H x W``, sinograms
``B x 1 x V x D``, per-view images ``B x V x H x W``, contiguous CUDA tensors
in float32 or float64, and the reference's options vector. Each call returns a
fresh tensor on the input's device and launches on the current CUDA stream.

Differences from the reference, all on error paths or convenience:
* the options vector may live on the CPU or the GPU, in any float dtype (its
  values are rounded to the data dtype, which is what the reference reads);
  a GPU options tensor is read once per (tensor, version), not on every call;
* an unknown scan_type, mismatched shapes or non-CUDA / non-contiguous inputs
  raise ``ValueError`` / ``RuntimeError`` instead of terminating the process
  (src/ctlib.cpp:26) or reading out of bounds;
* inputs with C > 1 channels use channel 0, as the reference does.
"""

from __future__ import annotations

import threading
import weakref
from collections import OrderedDict

import torch

from . import _native as N
from . import tune

_FLOATS = (torch.float32, torch.float64)


class Plan:
    """Geometry of one options vector on one device, uploaded once."""

    def __init__(self, values: tuple, dtype: torch.dtype, device: int):
        import ctypes
        self.values = values
        self.dtype = dtype
        self.device = device
        arr = (ctypes.c_double * len(values))(*values)
        h = ctypes.c_void_p()
        with torch.cuda.device(device):
            rc = N.lib().ctgb_plan_create(ctypes.byref(h), arr, len(values),
                                          0 if dtype == torch.float32 else 1, device)
        N.check(rc, "options")
        self.handle = h
        vals = [ctypes.c_int() for _ in range(6)]
        N.lib().ctgb_plan_info(h, *[ctypes.byref(x) for x in vals])
        self.views, self.dets, self.width, self.height, self.scan_type, _ = (x.value for x in vals)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and N._lib is not None:
            try:
                N._lib.ctgb_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def set_summation(self, compensated: bool):
        """Compensated (default) or one plain fp32 running sum per output
        (ctgb_plan_set_summation). Plans from ``get_plan`` are shared: change
        this only on a plan of your own (``Plan(values, dtype, device)``)."""
        N.check(N.lib().ctgb_plan_set_summation(self.handle, int(bool(compensated))), "summation")

    def workspace_bytes(self, op: int, batch: int) -> int:
        return int(N.lib().ctgb_workspace_size(self.handle, op, batch))

    def run(self, op: int, x: torch.Tensor, out: torch.Tensor, stream=None) -> torch.Tensor:
        """Launch ``op`` on contiguous device tensors (no checks beyond the C side)."""
        batch = x.shape[0]
        nbytes = self.workspace_bytes(op, batch)
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
        if stream is None:
            stream = torch.cuda.current_stream(x.device)
        fn = _FN[op]
        rc = fn(self.handle, x.data_ptr(), out.data_ptr(), batch, ws.data_ptr(), nbytes, stream.cuda_stream)
        N.check(rc, _NAMES[op])
        return out


_NAMES = {N.OP_PROJECTION: "projection", N.OP_PROJECTION_T: "projection_t",
          N.OP_BACKPROJECTION: "backprojection", N.OP_BACKPROJECTION_T: "backprojection_t", N.OP_FBP: "fbp",
          N.OP_BACKPROJECTION_SV: "backprojection_sv"}


class _FnTable(dict):
    def __missing__(self, op):
        l = N.lib()
        fn = {N.OP_PROJECTION: l.ctgb_projection, N.OP_PROJECTION_T: l.ctgb_projection_t,
              N.OP_BACKPROJECTION: l.ctgb_backprojection, N.OP_BACKPROJECTION_T: l.ctgb_backprojection_t,
              N.OP_FBP: l.ctgb_fbp, N.OP_BACKPROJECTION_SV: l.ctgb_backprojection_sv}[op]
        self[op] = fn
        return fn


_FN = _FnTable()

_plan_lock = threading.Lock()
_plans: "OrderedDict[tuple, Plan]" = OrderedDict()
_MAX_PLANS = 256
# values of live CUDA options tensors: id -> (weakref, version, values). An
# entry is used only while its weakref still points at the same object and the
# version counter is unchanged (no in-place update); the finalizer drops it when
# the tensor is collected, so a reused address or id never aliases.
_opt_cache: dict = {}


def _option_values(options) -> tuple:
    if isinstance(options, torch.Tensor):
        if not options.is_cuda:
            return tuple(float(v) for v in options.detach().reshape(-1).tolist())
        key = id(options)
        hit = _opt_cache.get(key)
        if hit is not None and hit[0]() is options and hit[1] == options._version:
            return hit[2]
        vals = tuple(float(v) for v in options.detach().reshape(-1).tolist())
        if hit is None or hit[0]() is not options:
            weakref.finalize(options, _opt_cache.pop, key, None)
        _opt_cache[key] = (weakref.ref(options), options._version, vals)
        return vals
    return tuple(float(v) for v in options)


FILTERS = {"ram-lak": 0, "shepp-logan": 1, "hann": 2}


def get_plan(options, dtype: torch.dtype, device, filt: tuple = (0, 0)) -> Plan:
    """Cached plan for (options values, dtype, device, fbp filter). ``filt`` is
    (window, ea_exact) as for ctgb_plan_set_filter; (0, 0) is the reference's
    Ram-Lak filter."""
    dev = torch.device(device)
    idx = dev.index if dev.index is not None else torch.cuda.current_device()
    vals = _option_values(options)
    key = (vals, dtype, idx, tuple(filt))
    with _plan_lock:
        p = _plans.get(key)
        if p is not None:
            _plans.move_to_end(key)
            return p
    p = Plan(vals, dtype, idx)
    if tuple(filt) != (0, 0):
        N.check(N.lib().ctgb_plan_set_filter(p.handle, int(filt[0]), int(filt[1])), "filter")
    with _plan_lock:
        _plans[key] = p
        while len(_plans) > _MAX_PLANS:
            _plans.popitem(last=False)
    return p


def clear_plans():
    with _plan_lock:
        _plans.clear()
        _opt_cache.clear()


def _check_input(x: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(x, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not x.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not x.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if x.dtype not in _FLOATS:
        raise RuntimeError(f"{name} must be float32 or float64, got {x.dtype}")
    if x.dim() != 4:
        raise ValueError(f"{name} must be 4-D (B x 1 x H x W or B x 1 x V x D), got shape {tuple(x.shape)}")
    if x.shape[1] != 1:
        x = x[:, :1].contiguous()
    return x


def _apply(op: int, x: torch.Tensor, options, name: str, filt: tuple = (0, 0)) -> torch.Tensor:
    x = _check_input(x, name)
    plan = get_plan(options, x.dtype, x.device, filt)
    B = x.shape[0]
    img_shape = (plan.height, plan.width)
    sino_shape = (plan.views, plan.dets)
    if op in (N.OP_PROJECTION, N.OP_BACKPROJECTION_T):
        if tuple(x.shape[2:]) != img_shape:
            raise ValueError(f"{name}: image is {tuple(x.shape[2:])}, options give height x width {img_shape}")
        out = torch.empty((B, 1) + sino_shape, dtype=x.dtype, device=x.device)
    elif op == N.OP_BACKPROJECTION_SV:
        if plan.scan_type != 0:
            raise ValueError("backprojection_sv is defined for equal-distance fan beams (scan_type 0) only")
        if tuple(x.shape[2:]) != sino_shape:
            raise ValueError(f"{name}: sinogram is {tuple(x.shape[2:])}, options give views x dets {sino_shape}")
        out = torch.empty((B, plan.views) + img_shape, dtype=x.dtype, device=x.device)
    else:
        if tuple(x.shape[2:]) != sino_shape:
            raise ValueError(f"{name}: sinogram is {tuple(x.shape[2:])}, options give views x dets {sino_shape}")
        out = torch.empty((B, 1) + img_shape, dtype=x.dtype, device=x.device)
    if B == 0:
        return out
    tune.apply_cached(plan, op, B)
    with torch.cuda.device(x.device):
        return plan.run(op, x, out)


def projection(image: torch.Tensor, options) -> torch.Tensor:
    """A: image B x 1 x H x W -> sinogram B x 1 x V x D (src/ctlib.cpp:56-69)."""
    return _apply(N.OP_PROJECTION, image, options, "image")


def projection_t(projection: torch.Tensor, options) -> torch.Tensor:
    """A^T: sinogram -> image (src/ctlib.cpp:71-84)."""
    return _apply(N.OP_PROJECTION_T, projection, options, "projection")


def backprojection(projection: torch.Tensor, options) -> torch.Tensor:
    """B, the FBP backprojector with distance weighting: sinogram -> image (src/ctlib.cpp:30-43)."""
    return _apply(N.OP_BACKPROJECTION, projection, options, "projection")


def backprojection_t(image: torch.Tensor, options) -> torch.Tensor:
    """B^T: image -> sinogram (src/ctlib.cpp:15-28)."""
    return _apply(N.OP_BACKPROJECTION_T, image, options, "image")


def fbp(projection: torch.Tensor, options, filter: str = "ram-lak", ea_exact: bool = False) -> torch.Tensor:
    """Filtered backprojection: sinogram -> image (src/ctlib.cpp:86-99).

    The defaults reproduce the reference: the Ram-Lak kernel with the
    reference's detector pre-weights. ``filter`` may also be "shepp-logan" or
    "hann" (Ram-Lak under a Hann window); ``ea_exact`` (equal-angle fans only)
    uses the kernel that is exact on equiangular samples, (g/sin g)^2 times
    Ram-Lak, where the reference applies the parallel-beam kernel in angle
    units. Neither option exists in the reference."""
    if filter not in FILTERS:
        raise ValueError(f"filter must be one of {sorted(FILTERS)}, got {filter!r}")
    return _apply(N.OP_FBP, projection, options, "projection", (FILTERS[filter], int(bool(ea_exact))))


def backprojection_sv(projection: torch.Tensor, options) -> torch.Tensor:
    """Single-view backprojection, equal-distance fan beams only: sinogram
    B x 1 x V x D -> B x V x H x W, image v holding view v's term of
    backprojection (src/ctlib.cpp:45-54, src/fan_ed_kernel.cu:946-1161)."""
    return _apply(N.OP_BACKPROJECTION_SV, projection, options, "projection")


def data_gradient(image: torch.Tensor, projection: torch.Tensor, options, return_residual: bool = False):
    """Gradient of the data term 0.5*||A x - y||^2: A^T(A x - y) for an image
    B x 1 x H x W and a measured sinogram B x 1 x V x D (ctgb_data_gradient).
    The same values as ``projection_t(projection(x) - y)``, without the separate
    subtraction and sinogram re-layout. With ``return_residual`` also returns
    A x - y. No single counterpart in the reference, which composes it from
    projection and projection_t (src/ctlib.cpp:56-84)."""
    import ctypes
    x = _check_input(image, "image")
    y = _check_input(projection, "projection")
    if y.dtype != x.dtype or y.device != x.device:
        raise ValueError("image and projection must share dtype and device")
    plan = get_plan(options, x.dtype, x.device)
    B = x.shape[0]
    if tuple(x.shape[2:]) != (plan.height, plan.width):
        raise ValueError(f"image is {tuple(x.shape[2:])}, options give height x width {(plan.height, plan.width)}")
    if tuple(y.shape) != (B, 1, plan.views, plan.dets):
        raise ValueError(f"projection is {tuple(y.shape)}, expected {(B, 1, plan.views, plan.dets)}")
    grad = torch.empty_like(x)
    res = torch.empty_like(y) if return_residual else None
    if B > 0:
        # the two kernels run with the schedules of projection and projection_t
        tune.apply_cached(plan, N.OP_PROJECTION, B)
        tune.apply_cached(plan, N.OP_PROJECTION_T, B)
        nbytes = plan.workspace_bytes(N.OP_DATA_GRADIENT, B)
        with torch.cuda.device(x.device):
            ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
            stream = torch.cuda.current_stream(x.device)
            rc = N.lib().ctgb_data_gradient(plan.handle, x.data_ptr(), y.data_ptr(),
                                            res.data_ptr() if res is not None else None, grad.data_ptr(), B,
                                            ws.data_ptr(), ctypes.c_size_t(nbytes), stream.cuda_stream)
        N.check(rc, "data_gradient")
    return (grad, res) if return_residual else grad


def laplacian(input: torch.Tensor, k: int) -> torch.Tensor:
    """kNN graph adjacency of the n rows of an n x dim tensor (src/ctlib.cpp:101-104,
    src/laplacian_cuda_kernel.cu:46-128): for every point its k nearest points,
    itself included, weighted exp(-d / m) with d the squared distance and m the
    lower median of all n*k selected distances, normalised to sum 1 per row.
    Returns an n x n sparse COO tensor with float32 values, neighbours of each
    row in increasing distance (ctgb_laplacian). Ties in distance go to the
    smaller index; k <= 256."""
    import ctypes
    if not isinstance(input, torch.Tensor):
        raise TypeError("input must be a torch.Tensor")
    if not input.is_cuda:
        raise RuntimeError("input must be a CUDA tensor")
    if not input.is_contiguous():
        raise RuntimeError("input must be contiguous")
    if input.dtype not in _FLOATS:
        raise RuntimeError(f"input must be float32 or float64, got {input.dtype}")
    if input.dim() != 2:
        raise ValueError(f"input must be 2-D (points x dimension), got shape {tuple(input.shape)}")
    n, dim = (int(s) for s in input.shape)
    k = int(k)
    if n < 1 or dim < 1:
        raise ValueError("input must hold at least one point of dimension >= 1")
    if not 1 <= k <= n:
        raise ValueError(f"k must be in [1, {n}], got {k}")
    if k > 256:
        raise ValueError("k > 256 is not supported")
    dt = N.FLOAT32 if input.dtype == torch.float32 else N.FLOAT64
    nbytes = int(N.lib().ctgb_laplacian_workspace_size(n, dim, k, dt))
    ind = torch.empty((2, n * k), dtype=torch.int64, device=input.device)
    val = torch.empty((n * k,), dtype=torch.float32, device=input.device)
    with torch.cuda.device(input.device):
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=input.device)
        stream = torch.cuda.current_stream(input.device)
        rc = N.lib().ctgb_laplacian(input.data_ptr(), n, dim, k, dt, ind.data_ptr(), val.data_ptr(),
                                    ws.data_ptr(), ctypes.c_size_t(nbytes), stream.cuda_stream)
    N.check(rc, "laplacian")
    return torch.sparse_coo_tensor(ind, val, (n, n), dtype=torch.float32, device=input.device)
