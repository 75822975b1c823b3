"""ctgb_projection_noalloc: the projection entry point for callers that cannot
allocate device memory at run time (no allocator of their own, or all memory
reserved at start-up). It must give the same sinogram as ctgb_projection, which
uses a caller-provided workspace, bit for bit (the same kernels run on the same
plan), on consecutive calls that reuse its static scratch array, including a
call right after one of a plan with longer image lines, and must refuse
batches whose scratch exceeds that array.

This file is collected last so that a failure here leaves every other test run.
"""

import ctypes
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctlib_gb300 as ct
    from ctlib_gb300 import _native
    _native.build()
    return ct, _native


def test_noalloc_projection_matches_workspace_projection(env):
    ct, N = env
    from ctlib_gb300.workloads import FAN_ED, ellipse_phantom, fan_options
    opts = fan_options(180, 256, 128, 128, 1.5, 2.5, 0.1, 2 * math.pi / 180, 595.0, 490.6, 0.4, FAN_ED)
    img = torch.from_numpy(np.stack([ellipse_phantom(128, 128, 1.5, 70 + i) for i in range(5)])[:, None]).cuda()
    o = torch.tensor(opts, dtype=torch.float32)
    ref = ct.projection(img, o)
    plan = ct.get_plan(o, torch.float32, img.device)
    lib = N.lib()
    need = plan.workspace_bytes(N.OP_PROJECTION, img.shape[0])
    assert 0 < need <= lib.ctgb_projection_noalloc_max_bytes()
    stream = torch.cuda.current_stream()
    for _ in range(2):
        out = torch.full_like(ref, float("nan"))
        rc = lib.ctgb_projection_noalloc(plan.handle, ctypes.c_void_p(img.data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()), img.shape[0],
                                         ctypes.c_void_p(stream.cuda_stream))
        assert rc == N.OK, N.last_error()
        torch.cuda.synchronize()
        # the same kernels on the same plan and schedule: identical bits
        assert torch.equal(out, ref)


def test_noalloc_rejects_batches_beyond_static_scratch(env):
    ct, N = env
    from ctlib_gb300.workloads import FAN_ED, fan_options
    opts = fan_options(64, 96, 512, 512, 0.6641, 1.2858 * 8, 0.0, 2 * math.pi / 64, 595.0, 490.6, 0.0, FAN_ED)
    o = torch.tensor(opts, dtype=torch.float32)
    plan = ct.get_plan(o, torch.float32, torch.device("cuda", 0))
    lib = N.lib()
    batch = 64
    assert plan.workspace_bytes(N.OP_PROJECTION, batch) > lib.ctgb_projection_noalloc_max_bytes()
    x = torch.zeros(1, device="cuda")
    rc = lib.ctgb_projection_noalloc(plan.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                                     batch, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.ERR_WORKSPACE
    assert "static" in N.last_error()


def test_noalloc_after_a_larger_plan(env):
    """A call leaves its layout in the shared array; the next call, of a plan
    whose lines are shorter (other padding), must not be affected by it."""
    ct, N = env
    from ctlib_gb300.workloads import FAN_ED, ellipse_phantom, fan_options
    lib = N.lib()
    stream = torch.cuda.current_stream()
    big = fan_options(96, 200, 203, 197, 1.5, 2.5, 0.0, 2 * math.pi / 96, 595.0, 490.6, 0.0, FAN_ED)
    small = fan_options(80, 120, 61, 77, 1.5, 2.5, 0.2, 2 * math.pi / 80, 595.0, 490.6, 0.3, FAN_ED)
    outs = []
    for opts, seed in ((big, 5), (small, 6)):
        W, H = int(opts[2]), int(opts[3])
        img = torch.from_numpy(np.stack([ellipse_phantom(H, W, 1.5, seed + i) for i in range(3)])[:, None]).cuda()
        o = torch.tensor(opts, dtype=torch.float32)
        plan = ct.get_plan(o, torch.float32, img.device)
        out = torch.full((3, 1, int(opts[0]), int(opts[1])), float("nan"), device="cuda")
        rc = lib.ctgb_projection_noalloc(plan.handle, ctypes.c_void_p(img.data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()), 3, ctypes.c_void_p(stream.cuda_stream))
        assert rc == N.OK, N.last_error()
        torch.cuda.synchronize()
        outs.append((out, ct.projection(img, o)))
    for out, ref in outs:
        assert torch.equal(out, ref)
