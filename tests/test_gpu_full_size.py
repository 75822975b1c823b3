"""Parity at the benchmark sizes: one slice of each benchmark geometry through
every operator against the FP64 oracle, and size-independent properties of the
full 16-slice headline batch.

* fp32 outputs within rel-L2 1e-5 of the FP64 oracle (projection,
  projection_t, backprojection, backprojection_t on seeded Gaussian inputs; fbp
  on the oracle's projection of a phantom), for the parallel-beam 256^2 /
  360-view, fan-beam equal-distance 512^2 / 1152-view, fan-beam equal-angle
  512^2 / 984-view and fan-beam equal-distance 1024^2 / 2304-view geometries;
* linearity of A and A^T over the 16 x 512^2 batch: A(2x + 3y) against
  2 A(x) + 3 A(y) within rel-L2 1e-6;
* the adjoint identity <A x, y> = <x, A^T y> on the 8 x 1024^2 stress batch
  within 1e-5 (relative), accumulated in fp64.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

OPS = ("projection", "projection_t", "backprojection", "backprojection_t", "fbp")


@pytest.fixture(scope="module")
def ct():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctlib_gb300
    from ctlib_gb300 import _native
    _native.build()
    return ctlib_gb300


def _workload(name):
    from ctlib_gb300.workloads import WORKLOADS
    return WORKLOADS[name]()


@pytest.mark.parametrize("name", ["parallel_256", "fan_ed_512", "fan_ea_512", "fan_ed_1024"])
@pytest.mark.parametrize("op", OPS)
def test_benchmark_geometry_vs_fp64(ct, oracle_mod, name, op):
    from ctlib_gb300.workloads import ellipse_phantom, gaussian
    O = oracle_mod
    s = _workload(name).slices[0]
    opts = list(s.options)
    V, D, W, H = (int(opts[i]) for i in range(4))
    if op in ("projection", "backprojection_t"):
        x = gaussian((1, 1, H, W), 71).astype(np.float32)
    elif op == "fbp":
        img = ellipse_phantom(H, W, opts[4], s.seed)[None, None]
        x = O.run("projection", img, opts, O.MODE_F64_ON_F32).astype(np.float32)
    else:
        x = gaussian((1, 1, V, D), 72).astype(np.float32)
    want = O.run(op, x, opts, O.MODE_F64_ON_F32)
    t = torch.from_numpy(x).cuda()
    got = getattr(ct, op)(t, torch.tensor(opts, dtype=torch.float32)).cpu().numpy()
    assert np.isfinite(got).all()
    e = O.rel_l2(got, want)
    print(f"{name} {op}: rel-L2 vs FP64 {e:.2e}")
    assert e <= 1e-5, e


def test_linearity_headline_batch(ct, oracle_mod):
    O = oracle_mod
    w = _workload("fan_ed_512")
    o = torch.tensor(w.slices[0].options, dtype=torch.float32)
    g = torch.Generator().manual_seed(5)
    x = torch.randn(16, 1, 512, 512, generator=g).cuda()
    y = torch.randn(16, 1, 512, 512, generator=g).cuda()
    lhs = ct.projection(2 * x + 3 * y, o)
    rhs = 2 * ct.projection(x, o) + 3 * ct.projection(y, o)
    assert O.rel_l2(lhs.cpu().numpy(), rhs.cpu().numpy()) <= 1e-6
    s = torch.randn(16, 1, 1152, 736, generator=g).cuda()
    u = torch.randn(16, 1, 1152, 736, generator=g).cuda()
    lhs = ct.projection_t(2 * s + 3 * u, o)
    rhs = 2 * ct.projection_t(s, o) + 3 * ct.projection_t(u, o)
    assert O.rel_l2(lhs.cpu().numpy(), rhs.cpu().numpy()) <= 1e-6


def test_adjoint_identity_stress_batch(ct):
    w = _workload("fan_ed_1024")
    o = torch.tensor(w.slices[0].options, dtype=torch.float32)
    g = torch.Generator().manual_seed(6)
    x = torch.rand(8, 1, 1024, 1024, generator=g).cuda()
    ax = ct.projection(x, o)
    y = ax + 0.1 * torch.randn(ax.shape, generator=g).cuda()  # correlated with A x
    aty = ct.projection_t(y, o)
    lhs = float((ax.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs), (lhs, rhs)
