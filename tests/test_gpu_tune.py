"""Autotuned schedules (slices per thread, warps per CTA, straight-line steps)
change only the launch shape: outputs must be identical to the default
schedule's, bit for bit, and the choice must be cached."""

import math
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_tune_keeps_results_and_caches(tmp_path, monkeypatch):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    monkeypatch.setenv("CTLIB_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    from ctlib_gb300 import _native as N
    from ctlib_gb300 import ops, tune
    from ctlib_gb300.workloads import FAN_ED, ellipse_phantom, fan_options
    monkeypatch.setattr(tune, "_cache", None)
    opts = fan_options(96, 128, 64, 64, 1.0, 2.0, 0.0, 2 * math.pi / 96, 120.0, 100.0, 0.0, FAN_ED)
    img = torch.from_numpy(np.stack([ellipse_phantom(64, 64, 1.0, i) for i in range(16)])[:, None]).cuda()
    o = torch.tensor(opts, dtype=torch.float32)
    ops.clear_plans()
    plan = ops.get_plan(o, torch.float32, img.device)
    ref_a = ops.projection(img, o)
    ref_at = ops.projection_t(ref_a, o)
    ref_bt = ops.backprojection_t(img, o)
    ref_b = ops.backprojection(ref_a, o)
    for op in (N.OP_PROJECTION, N.OP_PROJECTION_T):
        r = tune.tune(plan, op, img.shape[0], reps=1)
        assert len(r["candidates"]) >= 3
    assert os.path.exists(tmp_path / "tune.json")
    # a schedule tuned for another batch size must not leak into this one
    tune.tune(plan, N.OP_PROJECTION, 1, reps=1)
    ops.projection(img, o)
    assert plan._current[N.OP_PROJECTION] == plan._tuned[(N.OP_PROJECTION, img.shape[0])]
    for sched in tune.CANDIDATES_F32:
        for op in (N.OP_PROJECTION, N.OP_PROJECTION_T, N.OP_BACKPROJECTION, N.OP_BACKPROJECTION_T):
            plan._tuned[(op, img.shape[0])] = sched  # force this schedule for the batch
        a = ops.projection(img, o)
        at = ops.projection_t(a, o)
        assert plan._current[N.OP_PROJECTION] == sched
        assert torch.equal(a, ref_a), sched
        assert torch.equal(at, ref_at), sched
        assert torch.equal(ops.backprojection_t(img, o), ref_bt), sched
        assert torch.equal(ops.backprojection(ref_a, o), ref_b), sched
    ops.clear_plans()
