"""The reference's own CUDA kernels on this GPU (oracle/ref_cuda.py, compiled
unchanged for sm_103a) against

* the golden fixtures, which the same kernels produced when executed on the CPU
  (oracle/ref_emu): this pins the CPU execution to the GPU one. Tolerance
  (rel-L2) 1e-12 for fp64; 1e-6 for fp32, where the order of the kernels'
  atomicAdd calls differs between the two executions (two GPU runs differ by up
  to 4e-7), except projection_t on the 256^2 / 576-view fan fixtures: there the
  reference's fp32 pixel walk is 1.5e-4 away from exact and the CPU build,
  which contracts a few multiply-adds differently, moves it by up to 6e-6, so
  1e-5;
* this package's CUDA operators, with the tolerances that the parity tests use
  against the golden fixtures;
* on the 512^2, 1152-view, 736-bin fan-beam equal-distance geometry: this
  package within 1e-5 of the FP64 oracle, and within the reference's own
  distance from it (plus 1e-5) of the reference.

Skipped where the cubins were not built (they are compiled from a CTLIB
checkout by oracle/build.py:build_ref_gpu).
"""

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden_files

pytestmark = pytest.mark.gpu

REF_OP = {"projection": 0, "projection_t": 1, "backprojection": 2, "backprojection_t": 3, "backprojection_sv": 5}


@pytest.fixture(scope="module")
def ref():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("reference cubins not built")
    return ref_cuda.get()


@pytest.fixture(scope="module")
def ct():
    import ctlib_gb300
    from ctlib_gb300 import _native
    _native.build()
    return ctlib_gb300


@pytest.fixture(autouse=True)
def _no_tf32():
    old = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    yield
    torch.backends.cudnn.allow_tf32 = old


def _cases():
    out = []
    for f in golden_files():
        z = np.load(f"{GOLDEN}/{f}")
        for op in list(REF_OP) + ["fbp"]:
            if f"{op}_in" in z:
                out.append((f, op))
    return out


def _ref_call(ref, op, x, opts, poison=True):
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    o = torch.tensor(list(opts), dtype=t.dtype, device="cuda")
    out = ref.fbp(t, o) if op == "fbp" else ref.run(REF_OP[op], t, o, poison=poison)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("fname,op", _cases())
def test_ref_gpu_matches_cpu_execution(ref, oracle_mod, fname, op):
    z = np.load(f"{GOLDEN}/{fname}")
    x, want, opts = z[f"{op}_in"], z[f"{op}_out"], z["options"]
    got = _ref_call(ref, op, x, opts)
    assert got.shape == want.shape and got.dtype == want.dtype
    assert np.isfinite(got).all(), "the reference kernel left elements unwritten"
    if x.dtype == np.float64:
        tol = 1e-12
    else:
        tol = 1e-5 if fname.startswith("cfg_fan") and op == "projection_t" else 1e-6
    assert oracle_mod.rel_l2(got, want) <= tol


@pytest.mark.parametrize("fname,op", _cases())
def test_ours_vs_ref_gpu(ref, ct, oracle_mod, fname, op):
    from test_gpu_parity import _ref_tol
    z = np.load(f"{GOLDEN}/{fname}")
    x, opts = z[f"{op}_in"], z["options"]
    want = _ref_call(ref, op, x, opts)
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    got = getattr(ct, op)(t, torch.tensor(list(opts), dtype=t.dtype)).cpu().numpy()
    tol = 1e-12 if x.dtype == np.float64 else _ref_tol(fname, op)
    assert oracle_mod.rel_l2(got, want) <= tol


@pytest.mark.parametrize("op", ["projection", "projection_t", "backprojection", "backprojection_t"])
def test_headline_geometry_vs_ref_gpu(ref, ct, oracle_mod, op):
    """fan-beam equal-distance, 2 x 512^2 phantoms, 1152 views, 736 bins; the
    sinogram inputs are the FP64 oracle's projection of the phantoms."""
    from ctlib_gb300.workloads import ellipse_phantom, fan_ed_512
    O = oracle_mod
    opts = fan_ed_512(1).slices[0].options
    img = np.stack([ellipse_phantom(512, 512, 1.0, 900 + i) for i in range(2)])[:, None].astype(np.float32)
    if op in ("projection", "backprojection_t"):
        x = img
    else:
        x = O.run("projection", img, opts, O.MODE_F64_ON_F32).astype(np.float32)
    exact = O.run(op, x, opts, O.MODE_F64_ON_F32)
    r = _ref_call(ref, op, x, opts)
    t = torch.from_numpy(x).cuda()
    ours = getattr(ct, op)(t, torch.tensor(opts, dtype=torch.float32)).cpu().numpy()
    assert np.isfinite(r).all()
    e_ours, e_ref = O.rel_l2(ours, exact), O.rel_l2(r, exact)
    print(f"{op}: rel-L2 vs FP64 ours {e_ours:.2e} reference {e_ref:.2e}; ours vs reference "
          f"{O.rel_l2(ours, r):.2e}")
    assert e_ours <= 1e-5, e_ours
    assert O.rel_l2(ours, r) <= e_ref + 1e-5, (O.rel_l2(ours, r), e_ref)
