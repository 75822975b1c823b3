"""fbp filter variants (ctgb_plan_set_filter / fbp(filter=..., ea_exact=...)):
Shepp-Logan, Ram-Lak under a Hann window and the exact equal-angle kernel,
against the FP64 oracle's restatement of the same kernels; the default stays
the reference's Ram-Lak filter."""

import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ct():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctlib_gb300
    from ctlib_gb300 import _native
    _native.build()
    return ctlib_gb300


def _geom(scan):
    from ctlib_gb300.workloads import FAN_EA, FAN_ED, fan_options, para_options
    if scan == 0:
        return fan_options(90, 101, 64, 56, 1.0, 2.0, 0.3, 2 * math.pi / 90, 120.0, 100.0, 0.2, FAN_ED)
    if scan == 1:
        return fan_options(90, 101, 64, 56, 1.0, 0.01, 0.3, 2 * math.pi / 90, 120.0, 100.0, 0.002, FAN_EA)
    return para_options(90, 101, 64, 56, 1.0, 1.1, 0.3, math.pi / 90, 0.2)


def _sinogram(oracle_mod, opts, dtype):
    from ctlib_gb300.workloads import ellipse_phantom
    O = oracle_mod
    img = np.stack([ellipse_phantom(56, 64, 1.0, 700 + i) for i in range(3)])[:, None]
    mode = O.MODE_F64_ON_F32 if dtype == np.float32 else O.MODE_F64
    return O.run("projection", img, opts, mode).astype(dtype), mode


@pytest.mark.parametrize("scan", [0, 1, 2])
@pytest.mark.parametrize("filt", ["ram-lak", "shepp-logan", "hann"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_filter_windows_vs_oracle(ct, oracle_mod, scan, filt, dtype):
    O = oracle_mod
    opts = _geom(scan)
    y, mode = _sinogram(O, opts, dtype)
    ty = torch.from_numpy(y).cuda()
    got = ct.fbp(ty, torch.tensor(opts, dtype=ty.dtype), filter=filt).cpu().numpy()
    want = O.fbp(y, opts, mode, filter=filt)
    tol = 1e-5 if dtype == np.float32 else 1e-12
    assert O.rel_l2(got, want) <= tol, O.rel_l2(got, want)


@pytest.mark.parametrize("filt", ["ram-lak", "shepp-logan", "hann"])
def test_exact_equal_angle_kernel(ct, oracle_mod, filt):
    O = oracle_mod
    opts = _geom(1)
    y, mode = _sinogram(O, opts, np.float32)
    ty = torch.from_numpy(y).cuda()
    o = torch.tensor(opts, dtype=torch.float32)
    got = ct.fbp(ty, o, filter=filt, ea_exact=True).cpu().numpy()
    want = O.fbp(y, opts, mode, filter=filt, ea_exact=True)
    assert O.rel_l2(got, want) <= 1e-5
    # a different kernel from the reference's
    assert O.rel_l2(got, ct.fbp(ty, o, filter=filt).cpu().numpy()) > 1e-4


def test_defaults_and_errors(ct, oracle_mod):
    opts = torch.tensor(_geom(0), dtype=torch.float32)
    y, _ = _sinogram(oracle_mod, _geom(0), np.float32)
    ty = torch.from_numpy(y).cuda()
    ref = ct.fbp(ty, opts)
    # plans with other filters are separate and leave the default untouched
    ct.fbp(ty, opts, filter="hann")
    assert torch.equal(ct.fbp(ty, opts, filter="ram-lak"), ref)
    assert torch.equal(ct.fbp(ty, opts), ref)
    with pytest.raises(ValueError):
        ct.fbp(ty, opts, filter="cosine")
    with pytest.raises(ValueError):
        ct.fbp(ty, opts, ea_exact=True)  # equal-distance geometry
