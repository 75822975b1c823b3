"""Ragged batches (one launch per stage over slices of different geometries,
fp32 or fp64) must reproduce the per-slice calls exactly, directly and from a
CUDA-graph replay."""

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
    from ctlib_gb300 import _native, batched
    _native.build()
    return ct, batched


def _slices():
    from ctlib_gb300.workloads import FAN_EA, FAN_ED, fan_options, para_options
    tp = 2 * math.pi
    return [fan_options(60, 90, 64, 64, 1.0, 2.0, 0.0, tp / 60, 120.0, 100.0, 0.0, FAN_ED),
            fan_options(36, 300, 48, 40, 1.0, 0.9, 0.3, tp / 36, 120.0, 100.0, 0.5, FAN_ED),
            fan_options(72, 91, 48, 40, 1.0, 0.008, 0.3, tp / 72, 120.0, 100.0, 0.01, FAN_EA),
            para_options(90, 67, 32, 48, 1.0, 1.1, 0.1, math.pi / 90, 0.4),
            para_options(12, 128, 96, 96, 1.0, 1.2, 0.0, math.pi / 12, 0.0),
            fan_options(128, 256, 96, 80, 1.5, 2.5, 0.0, tp / 128, 595.0, 490.6, 0.0, FAN_ED),
            # enough views for the image gather to split them into 8 parts,
            # whose partial images a combine stage adds
            fan_options(520, 180, 40, 56, 1.0, 2.0, 0.1, tp / 520, 150.0, 100.0, 0.2, FAN_ED),
            para_options(1100, 80, 32, 32, 1.0, 1.0, 0.0, math.pi / 1100, 0.0)]


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("op", ["projection", "projection_t", "backprojection", "backprojection_t", "fbp"])
def test_ragged_matches_per_slice_calls(env, op, dtype):
    ct, batched = env
    opts = _slices()
    rb = batched.RaggedBatch(opts, dtype=dtype)
    g = torch.Generator().manual_seed(5)
    ins = []
    for o in opts:
        V, D, W, H = (int(o[i]) for i in range(4))
        shape = (1, 1, H, W) if op in ("projection", "backprojection_t") else (1, 1, V, D)
        ins.append(torch.randn(shape, generator=g, dtype=torch.float64).to(dtype).cuda())
    got = rb.run(op, ins)
    for x, o, y in zip(ins, opts, got):
        want = getattr(ct, op)(x, torch.tensor(o, dtype=dtype))
        assert y.dtype == dtype
        assert torch.equal(y, want), (op, o, float((y - want).abs().max()))


def test_ragged_rejects_mixed_dtypes(env):
    ct, batched = env
    from ctlib_gb300 import _native as N
    import ctypes
    opts = _slices()[:2]
    p32 = ct.get_plan(torch.tensor(opts[0]), torch.float32, torch.device("cuda", 0))
    p64 = ct.get_plan(torch.tensor(opts[1]), torch.float64, torch.device("cuda", 0))
    arr = (ctypes.c_void_p * 2)(p32.handle.value, p64.handle.value)
    h = ctypes.c_void_p()
    assert N.lib().ctgb_ragged_create(ctypes.byref(h), arr, 2, 0) == N.ERR_INVALID
    assert "dtype" in N.last_error()


@pytest.mark.parametrize("branches", [0, 1, 3])
def test_ragged_graph_replay(env, branches):
    ct, batched = env
    opts = _slices()
    rb = batched.RaggedBatch(opts)
    from ctlib_gb300.workloads import ellipse_phantom
    imgs = [torch.from_numpy(ellipse_phantom(int(o[3]), int(o[2]), o[4], 40 + i)[None, None]).cuda()
            for i, o in enumerate(opts)]
    replay, static_in, outs = rb.graphed(("projection", "fbp"), imgs, branches=branches)
    # the graph's intermediate buffers and workspaces must stay owned by the
    # replay callable: fresh allocations written between replays must not land
    # on them
    junk = [torch.empty(1 << 20, device="cuda") for _ in range(64)]
    for trial in range(2):
        for t in junk:
            t.fill_(7.0 + trial)
        for s, x in zip(static_in, imgs):
            s.copy_(x * (1.0 + trial))
        replay()
        torch.cuda.synchronize()
        for x, o, y in zip(imgs, opts, outs):
            ot = torch.tensor(o, dtype=torch.float32)
            want = ct.fbp(ct.projection(x * (1.0 + trial), ot), ot)
            assert torch.equal(y, want)


@pytest.mark.parametrize("branches", [0, 2])
def test_ragged_graph_outlives_batch(env, branches):
    """The replay callable keeps alive everything its kernels read: after the
    RaggedBatch object itself is dropped and collected (and fresh allocations
    reuse freed memory), replays still give the per-slice results."""
    import gc
    ct, batched = env
    opts = _slices()
    from ctlib_gb300.workloads import ellipse_phantom
    imgs = [torch.from_numpy(ellipse_phantom(int(o[3]), int(o[2]), o[4], 90 + i)[None, None]).cuda()
            for i, o in enumerate(opts)]
    rb = batched.RaggedBatch(opts)
    replay, static_in, outs = rb.graphed(("projection", "fbp"), imgs, branches=branches)
    del rb
    gc.collect()
    junk = [torch.full((1 << 18,), 3.0, device="cuda") for _ in range(32)]
    replay()
    torch.cuda.synchronize()
    del junk
    for x, o, y in zip(imgs, opts, outs):
        ot = torch.tensor(o, dtype=torch.float32)
        assert torch.equal(y, ct.fbp(ct.projection(x, ot), ot))


def test_ragged_autotuned_form(env, tmp_path, monkeypatch):
    """tune.tune_ragged times every graph form, caches the fastest under the
    batch's signature, and graphed(branches="auto") replays that form with the
    per-slice results."""
    ct, batched = env
    from ctlib_gb300 import tune
    monkeypatch.setenv("CTLIB_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(tune, "_cache", None)
    opts = _slices()
    rb = batched.RaggedBatch(opts)
    from ctlib_gb300.workloads import ellipse_phantom
    imgs = [torch.from_numpy(ellipse_phantom(int(o[3]), int(o[2]), o[4], 60 + i)[None, None]).cuda()
            for i, o in enumerate(opts)]
    chain = ("projection", "fbp")
    assert tune.ragged_cached(rb, chain) is None
    res = tune.tune_ragged(rb, chain, imgs, reps=1)
    assert res["branches"] in tune.RAGGED_CANDIDATES
    assert len(res["candidates"]) == len(tune.RAGGED_CANDIDATES)
    assert tune.ragged_cached(rb, chain) == res["branches"]
    replay, static_in, outs = rb.graphed(chain, imgs)
    replay()
    torch.cuda.synchronize()
    for x, o, y in zip(imgs, opts, outs):
        ot = torch.tensor(o, dtype=torch.float32)
        assert torch.equal(y, ct.fbp(ct.projection(x, ot), ot))
