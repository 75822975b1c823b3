"""The fused data-term gradient A^T(A x - y) (ctgb_data_gradient):

* the same values, bit for bit, as projection, a subtraction and projection_t;
* against the FP64 oracle's composition of the same operators, for every
  geometry, in fp32 and fp64;
* the autograd loss 0.5*||A x - y||^2 built on it;
* an unrolled gradient-descent reconstruction against the oracle's recursion.
"""

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
        return fan_options(72, 91, 48, 40, 1.0, 2.0, 0.2, 2 * math.pi / 72, 120.0, 100.0, 0.4, FAN_ED)
    if scan == 1:
        return fan_options(72, 91, 48, 40, 1.0, 0.01, 0.2, 2 * math.pi / 72, 120.0, 100.0, 0.004, FAN_EA)
    return para_options(72, 91, 48, 40, 1.0, 1.1, 0.2, math.pi / 72, 0.4)


@pytest.mark.parametrize("batch", [1, 5, 16])
def test_gradient_equals_composition_headline(ct, batch):
    """On the 512^2, 1152-view fan-ED geometry: the fused gradient and residual
    equal projection(x) - y and projection_t of it exactly."""
    from ctlib_gb300.ops import data_gradient
    from ctlib_gb300.workloads import fan_ed_512
    o = torch.tensor(fan_ed_512(1).slices[0].options, dtype=torch.float32)
    g = torch.Generator().manual_seed(20 + batch)
    x = torch.rand(batch, 1, 512, 512, generator=g).cuda()
    y = torch.randn(batch, 1, 1152, 736, generator=g).cuda()
    grad, res = data_gradient(x, y, o, return_residual=True)
    r_ref = ct.projection(x, o) - y
    assert torch.equal(res, r_ref)
    assert torch.equal(grad, ct.projection_t(r_ref, o))


@pytest.mark.parametrize("scan", [0, 1, 2])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gradient_vs_oracle(ct, oracle_mod, scan, dtype):
    from ctlib_gb300.ops import data_gradient
    O = oracle_mod
    opts = _geom(scan)
    rng = np.random.default_rng(30 + scan)
    x = rng.random((3, 1, 40, 48)).astype(dtype)
    y = rng.standard_normal((3, 1, 72, 91)).astype(dtype)
    mode = O.MODE_F64_ON_F32 if dtype == np.float32 else O.MODE_F64
    r_want = O.run("projection", x, opts, mode) - y.astype(np.float64)
    g_want = O.run("projection_t", r_want, opts, mode)
    tx, ty = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    grad, res = data_gradient(tx, ty, torch.tensor(opts, dtype=tx.dtype), return_residual=True)
    tol = 1e-5 if dtype == np.float32 else 1e-12
    assert O.rel_l2(res.cpu().numpy(), r_want) <= tol
    assert O.rel_l2(grad.cpu().numpy(), g_want) <= tol
    # without a residual output the gradient is the same
    assert torch.equal(data_gradient(tx, ty, torch.tensor(opts, dtype=tx.dtype)), grad)


def test_data_fidelity_autograd(ct):
    from ctlib_gb300.autograd import data_fidelity
    from ctlib_gb300.ops import data_gradient
    opts = torch.tensor(_geom(0), dtype=torch.float32)
    g = torch.Generator().manual_seed(9)
    x = torch.rand(2, 1, 40, 48, generator=g).cuda().requires_grad_(True)
    y = torch.randn(2, 1, 72, 91, generator=g).cuda().requires_grad_(True)
    loss = data_fidelity(x, y, opts)
    loss.backward()
    grad, res = data_gradient(x.detach(), y.detach(), opts, return_residual=True)
    want = 0.5 * float((res.double() ** 2).sum())
    assert abs(float(loss.detach()) - want) <= 1e-6 * want
    assert torch.equal(x.grad, grad)
    assert torch.equal(y.grad, -res)


def test_unrolled_gradient_descent_vs_oracle(ct, oracle_mod):
    """x <- x - a * A^T(A x - y), 10 iterations on the equal-angle fan geometry
    from the fused gradient, against the same recursion with the FP64 oracle."""
    from ctlib_gb300.ops import data_gradient
    from ctlib_gb300.workloads import ellipse_phantom
    O = oracle_mod
    opts = _geom(1)
    x_true = np.stack([ellipse_phantom(40, 48, 1.0, 500 + i) for i in range(2)])[:, None]
    y = O.run("projection", x_true, opts, O.MODE_F64_ON_F32).astype(np.float32)
    step, iters = 2e-4, 10
    o = torch.tensor(opts, dtype=torch.float32)
    yt = torch.from_numpy(y).cuda()
    x = torch.zeros(2, 1, 40, 48, device="cuda")
    for _ in range(iters):
        x = x - step * data_gradient(x, yt, o)
    xr = np.zeros((2, 1, 40, 48))
    for _ in range(iters):
        xr = xr - step * O.run("projection_t", O.run("projection", xr, opts, O.MODE_F64_ON_F32) - y, opts,
                               O.MODE_F64_ON_F32)
    assert O.rel_l2(x.cpu().numpy(), xr) <= 1e-5
