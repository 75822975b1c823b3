"""The image gather's view parts, as the library sizes them, against the rule
bench.py uses to count its launches (a sum of the parts runs only when the
views are split): the partial images in ctgb_workspace_size of projection_t
are parts x batch x H x W elements, none for one part."""

import ctypes
import math

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ctlib_gb300 import _native
    _native.build()
    return _native


def _al(x):
    return (x + 255) & ~255


@pytest.mark.parametrize("V,W,H", [(360, 256, 256), (64, 256, 256), (100, 64, 64), (79, 64, 64),
                                   (1152, 512, 512), (300, 512, 512), (200, 512, 512), (984, 400, 363)])
def test_view_split_matches_bench_rule(env, V, W, H):
    import bench
    from ctlib_gb300.workloads import FAN_ED, fan_options
    N = env
    D = 96
    opts = fan_options(V, D, W, H, 1.0, 2.0, 0.0, 2 * math.pi / V, 1200.0, 1000.0, 0.0, FAN_ED)
    lib = N.lib()
    arr = (ctypes.c_double * len(opts))(*opts)
    h = ctypes.c_void_p()
    assert lib.ctgb_plan_create(ctypes.byref(h), arr, len(opts), 0, 0) == 0, N.last_error()
    try:
        ws = lib.ctgb_workspace_size(h, N.OP_PROJECTION_T, 1)
    finally:
        lib.ctgb_plan_destroy(h)
    dp = (D + 2 + 3) & ~3  # cells per sinogram row: D plus two padding cells, to a multiple of 4
    planes = _al(V * dp * 4)  # one slice per thread, one slice
    parts = bench._view_split(V, W * H)
    assert ws - planes == (_al(parts * H * W * 4) if parts > 1 else 0), (ws, planes, parts)
