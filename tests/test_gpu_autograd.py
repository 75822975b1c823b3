"""Autograd pairs: each operator's backward is its hand-written adjoint.

* gradcheck in fp64 (the full finite-difference Jacobian vs the adjoint
  kernel) on 64x64 crops of the fan equal-distance, equal-angle and parallel
  geometries, for all four operators;
* the fp32 dot-product test <Ax,y> = <x,A^T y> on the full fan-ED, fan-EA and
  parallel benchmark geometries;
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


def _crop_parallel():
    from ctlib_gb300.workloads import para_options
    return para_options(48, 72, 64, 64, 1.0, 1.3, 0.1, math.pi / 48, 0.2)


def _geometry_table(opts, what):
    """Host geometry table `what` of ctgb_geometry_query, in fp64."""
    import ctypes
    from ctlib_gb300 import _native as N
    l = N.lib()
    o = (ctypes.c_double * len(opts))(*opts)
    n = l.ctgb_geometry_query(o, len(opts), 1, what, None, 0)
    assert n > 0, N.last_error()
    out = (ctypes.c_double * n)()
    l.ctgb_geometry_query(o, len(opts), 1, what, out, n)
    return np.frombuffer(out, dtype=np.float64).copy()


def ea_bt_factor(opts):
    """Per sinogram element (view, external bin) the factor dImg / cbar by which
    the reference's equal-angle backprojection_t exceeds the transpose of its
    backprojection (src/fan_ea_kernel.cu:590-607): fq * cell width, fq being
    the projection's dImg / (cbar * width), mapped from increasing-boundary
    order to the sinogram's bin order of each view."""
    V, D = int(opts[0]), int(opts[1])
    flags = _geometry_table(opts, 0).astype(np.int64)
    db = _geometry_table(opts, 1).reshape(V, D + 1)
    fq = _geometry_table(opts, 2).reshape(V, D)
    f = fq * np.diff(db, axis=1)
    flip = (flags & 2) != 0
    f[flip] = f[flip, ::-1]
    return f


GEOMETRIES = {"fan_ed": lambda: _crop_geometry(0), "fan_ea": lambda: _crop_geometry(1), "parallel": _crop_parallel}


@pytest.mark.parametrize("geom", sorted(GEOMETRIES))
@pytest.mark.parametrize("which", ["projection", "projection_t", "backprojection", "backprojection_t"])
def test_gradcheck_fp64(ag, geom, which):
    """Full finite-difference Jacobian (not a random projection of it) against
    the Jacobian the hand-written adjoint kernel gives, in fp64 on a 64 x 64
    crop, 48 views x 72 bins. For equal-angle fans the backprojector pair is
    the reference's, whose backprojection_t carries an extra dImg / cbar per
    (view, bin): there the check runs on the pair with that factor divided out
    of the adjoint, which makes it the exact transpose (the factor itself is
    ea_bt_factor, from the plan's geometry tables)."""
    opts_l = GEOMETRIES[geom]()
    opts = torch.tensor(opts_l, dtype=torch.float64)
    g = torch.Generator().manual_seed(3)
    img_in = which in ("projection", "backprojection_t")
    shape = (1, 1, 64, 64) if img_in else (1, 1, 48, 72)
    x = torch.randn(shape, generator=g, dtype=torch.float64).cuda().requires_grad_(True)
    fn = getattr(ag, which)
    if geom == "fan_ea" and which in ("backprojection", "backprojection_t"):
        q3 = torch.from_numpy(ea_bt_factor(opts_l)).view(1, 1, 48, 72).cuda()
        if which == "backprojection":
            # f = B; its autograd gradient is the reference's backprojection_t,
            # q3 * B^T g, and a hook divides q3 back out before it reaches t
            def f(t):
                t2 = t * 1.0
                t2.register_hook(lambda gr: None if gr is None else gr / q3)
                return ag.backprojection(t2, opts)
        else:
            # f = backprojection_t / q3 = B^T; the gradient reaching the
            # operator's output is g / q3, which a hook turns back into g, so
            # the operator's backward (backprojection) gives B g
            def f(t):
                out = ag.backprojection_t(t, opts)
                out.register_hook(lambda gr: None if gr is None else gr * q3)
                return out / q3
        assert torch.autograd.gradcheck(f, (x,), eps=1e-6, atol=1e-8, rtol=1e-6, fast_mode=False)
        return
    assert torch.autograd.gradcheck(lambda t: fn(t, opts), (x,), eps=1e-6, atol=1e-8, rtol=1e-6,
                                    fast_mode=False)


def test_ea_backprojector_pair_factor(ag):
    """Equal-angle backprojection_t is exactly q3 times the transpose of
    backprojection (fp64 dot products): <B y, x> = <y, backprojection_t(x) / q3>,
    while without the division the identity fails by the factor's spread."""
    opts_l = _crop_geometry(1)
    opts = torch.tensor(opts_l, dtype=torch.float64)
    g = torch.Generator().manual_seed(9)
    x = torch.randn(2, 1, 64, 64, generator=g, dtype=torch.float64).cuda()
    y = torch.randn(2, 1, 48, 72, generator=g, dtype=torch.float64).cuda()
    q3 = torch.from_numpy(ea_bt_factor(opts_l)).view(1, 1, 48, 72).cuda()
    lhs = float((ag.backprojection(y, opts) * x).sum())
    bt = ag.backprojection_t(x, opts)
    assert abs(lhs - float((y * bt / q3).sum())) <= 1e-11 * abs(lhs)
    assert abs(lhs - float((y * bt).sum())) > 1e-3 * abs(lhs)


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


@pytest.mark.parametrize("workload", ["fan_ea_512", "parallel_256"])
def test_dot_product_fp32_full_geometries(ag, workload):
    """The fp32 adjoint mismatch |<Ax,y> - <x,A^T y>| / |<Ax,y>| <= 1e-6 on the
    full equal-angle (512^2, 984 views, 888 bins) and parallel (256^2, 360
    views, 367 bins) geometries, inputs built as in the fan-ED test."""
    from ctlib_gb300.workloads import WORKLOADS
    o_l = WORKLOADS[workload]().slices[0].options
    o = torch.tensor(o_l, dtype=torch.float32)
    V, D, W, H = (int(o_l[i]) for i in range(4))
    g = torch.Generator().manual_seed(7)
    x = torch.randn(2, 1, H, W, generator=g).cuda()
    x2 = x + 0.5 * torch.randn(2, 1, H, W, generator=g).cuda()
    y = ag.projection(x2, o) + torch.randn(2, 1, V, D, generator=g).cuda()
    lhs = float((ag.projection(x, o).double() * y.double()).sum())
    rhs = float((x.double() * ag.projection_t(y, o).double()).sum())
    print(f"{workload}: adjoint mismatch {abs(lhs - rhs) / abs(lhs):.2e}")
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
