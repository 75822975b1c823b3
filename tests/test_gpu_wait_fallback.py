"""The staged image gather's bounded waits, made to run out on purpose.

Every wait of the copy pipeline in the image gather (projection_t,
backprojection, fbp, backprojection_sv) has a limit; when a wait runs out the
CTA stops using the pipeline, drains the copies already issued and finishes its
views on global loads, counting the event (ctgb_wait_timeouts). A plan with a
wait limit of 0 (ctgb_plan_set_wait_limit) gives up on any wait whose copy has
not landed at the first look, which sends nearly every CTA down that path. The
results must not change by a single bit, the events must be counted, and the
same plan at the default limit must run without any.

No fault is injected into the GPU: the copies are real and in bounds; only the
waiting gives up early.
"""

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


_OPS = {"projection_t": 1, "backprojection": 2, "fbp": 4, "backprojection_sv": 5}


@pytest.mark.parametrize("op", sorted(_OPS))
def test_forced_timeouts_fall_back_to_identical_results(env, op):
    ct, N = env
    from ctlib_gb300.ops import Plan
    from ctlib_gb300.workloads import FAN_ED, fan_options
    opts = fan_options(360, 400, 256, 256, 1.3, 1.2858, 0.2, 2 * math.pi / 360, 595.0, 490.6, 0.0, FAN_ED)
    B = 2 if op == "backprojection_sv" else 5
    g = torch.Generator().manual_seed(17)
    x = torch.randn(B, 1, 360, 400, generator=g).cuda()
    want = getattr(ct, op)(x, torch.tensor(opts, dtype=torch.float32))
    plan = Plan(tuple(opts), torch.float32, 0)
    lib = N.lib()
    shape = (B, 360, 256, 256) if op == "backprojection_sv" else (B, 1, 256, 256)
    torch.cuda.synchronize()
    N.wait_timeouts(0, reset=True)
    try:
        N.check(lib.ctgb_plan_set_wait_limit(plan.handle, 0), "wait limit")
        out = torch.full(shape, float("nan"), device="cuda")
        plan.run(_OPS[op], x, out)
        torch.cuda.synchronize()
        forced = N.wait_timeouts(0, reset=True)
        assert forced > 0, "no wait ran out at a limit of 0"
        assert torch.equal(out, want)
        N.check(lib.ctgb_plan_set_wait_limit(plan.handle, 1_000_000_000), "wait limit")
        out2 = torch.full(shape, float("nan"), device="cuda")
        plan.run(_OPS[op], x, out2)
        torch.cuda.synchronize()
        assert N.wait_timeouts(0) == 0
        assert torch.equal(out2, want)
    finally:
        N.wait_timeouts(0, reset=True)


def test_wait_limit_bounds(env):
    ct, N = env
    from ctlib_gb300.ops import Plan
    from ctlib_gb300.workloads import FAN_ED, fan_options
    opts = fan_options(90, 120, 64, 64, 1.0, 2.0, 0.0, 2 * math.pi / 90, 120.0, 100.0, 0.0, FAN_ED)
    plan = Plan(tuple(opts), torch.float32, 0)
    assert N.lib().ctgb_plan_set_wait_limit(plan.handle, 11_000_000_000) == N.ERR_INVALID
    assert N.lib().ctgb_plan_set_wait_limit(None, 0) == N.ERR_INVALID
