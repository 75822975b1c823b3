"""Autograd pairs: each operator's backward is its hand-written adjoint.

* gradcheck in fp64 (finite differences vs the adjoint kernel) on a 64x64 crop
  of the fan equal-distance geometry;
* an unrolled 10-iteration gradient-descent reconstruction x <- x - a*A^T(Ax - y)
  on equal-angle fan geometry with per-iteration activation checkpointing; the
  gradient of the final loss with respect to the measured sinogram is checked
  against the same recursion evaluated with the FP64 oracle's A and A^T.
"""

import math

import numpy as np
import pytest
import torch
from torch.utils.checkpoint import checkpoint

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ctlib_gb300 import _native, autograd
    _native.build()
    return autograd


def _crop_geometry(scan=0):
    # the fan-ED benchmark geometry (595 / 490.6 mm, 0.6641 mm pixels) cropped to
    # 64 x 64 pixels with a detector row covering it
    from ctlib_gb300.workloads import fan_options, FAN_ED, FAN_EA
    if scan == FAN_ED:
        return fan_options(48, 72, 64, 64, 0.6641, 1.2858, 0.1, 2 * math.pi / 48, 595.0, 490.6, 0.0, FAN_ED)
    return fan_options(48, 72, 64, 64, 0.7, 0.0011, 0.1, 2 * math.pi / 48, 541.0, 408.0, 0.0, FAN_EA)


@pytest.mark.parametrize("which", ["projection", "projection_t", "backprojection", "backprojection_t"])
def test_gradcheck_fp64(ag, which):
    opts = torch.tensor(_crop_geometry(), dtype=torch.float64)
    g = torch.Generator().manual_seed(3)
    if which in ("projection", "backprojection_t"):
        x = torch.randn(1, 1, 64, 64, generator=g, dtype=torch.float64)
    else:
        x = torch.randn(1, 1, 48, 72, generator=g, dtype=torch.float64)
    x = x.cuda().requires_grad_(True)
    fn = getattr(ag, which)
    assert torch.autograd.gradcheck(lambda t: fn(t, opts), (x,), eps=1e-6, atol=1e-8, rtol=1e-6,
                                    fast_mode=True)


def test_dot_product_fp32_headline_geometry(ag):
    """Adjoint mismatch of A / A^T in fp32 on the full 512^2, 1152-view fan-ED
    geometry: |<Ax,y> - <x,A^T y>| / |<Ax,y>| <= 1e-6 with Gaussian x and
    y = A x' + Gaussian noise (y correlated with Ax keeps <Ax,y> away from 0,
    so the ratio measures the operators rather than a near-zero denominator)."""
    from ctlib_gb300.workloads import fan_ed_512
    o = torch.tensor(fan_ed_512(1).slices[0].options, dtype=torch.float32)
    g = torch.Generator().manual_seed(7)
    x = torch.randn(2, 1, 512, 512, generator=g).cuda()
    x2 = x + 0.5 * torch.randn(2, 1, 512, 512, generator=g).cuda()
    y = ag.projection(x2, o) + torch.randn(2, 1, 1152, 736, generator=g).cuda()
    lhs = float((ag.projection(x, o).double() * y.double()).sum())
    rhs = float((x.double() * ag.projection_t(y, o).double()).sum())
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs), abs(lhs - rhs) / abs(lhs)


def test_unrolled_gd_checkpointed_gradient(ag, oracle_mod):
    O = oracle_mod
    from ctlib_gb300.workloads import ellipse_phantom
    opts = _crop_geometry(1)
    ot = torch.tensor(opts, dtype=torch.float32)
    B, iters, step = 2, 10, 2e-4
    x_true = np.stack([ellipse_phantom(64, 64, 0.7, 300 + i) for i in range(B)])[:, None]
    y_np = O.run("projection", x_true, opts, O.MODE_F64_ON_F32).astype(np.float32)
    y = torch.from_numpy(y_np).cuda().requires_grad_(True)
    xt = torch.from_numpy(x_true).cuda()

    def one_iter(x, yy):
        return x - step * ag.projection_t(ag.projection(x, ot) - yy, ot)

    x = torch.zeros(B, 1, 64, 64, device="cuda")
    for _ in range(iters):
        x = checkpoint(one_iter, x, y, use_reentrant=False)
    loss = 0.5 * ((x - xt) ** 2).sum()
    loss.backward()
    got = y.grad.double().cpu().numpy()

    # the same recursion with the FP64 oracle: forward, then reverse accumulation
    A = lambda v: O.run("projection", v, opts, O.MODE_F64_ON_F32)
    At = lambda v: O.run("projection_t", v, opts, O.MODE_F64_ON_F32)
    xs = [np.zeros((B, 1, 64, 64))]
    for _ in range(iters):
        xs.append(xs[-1] - step * At(A(xs[-1]) - y_np))
    gx = xs[-1] - x_true
    gy = np.zeros_like(y_np, dtype=np.float64)
    for _ in range(iters):
        gy += step * A(gx)
        gx = gx - step * At(A(gx))
    assert O.rel_l2(got, gy) <= 1e-5, O.rel_l2(got, gy)
