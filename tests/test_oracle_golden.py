"""Pin the CPU oracle against the reference's own kernels.

tests/golden/*.npz hold inputs and outputs of the reference's kernel source
(src/fan_ed_kernel.cu, src/fan_ea_kernel.cu, src/para_kernel.cu) executed on the
CPU by oracle/ref_emu (generator: tests/golden/make_golden.py).

Two checks per operator:
* the fp32 oracle, which follows the reference's fp32 promotions, against the
  reference's fp32 output;
* the FP64 oracle (fp32 view angles, fp64 arithmetic) against the same output.

The reference's fp32 walk accumulates pixel positions (``i0x += dImage``,
src/fan_ed_kernel.cu:368-391) and rounds detector boundaries to fp32, which puts
its own fp32 output ~3e-6 (rel-L2) from fp64 on phantom-like inputs but up to
~2e-4 on white-noise sinograms at 256^2 / 576 views. Tolerances below are set
per input kind accordingly; each is written next to the case it covers.
"""

import numpy as np
import pytest

from conftest import GOLDEN, golden_files

OPS = ("projection", "projection_t", "backprojection", "backprojection_t", "fbp", "backprojection_sv")


def _cases():
    out = []
    for f in golden_files():
        z = np.load(f"{GOLDEN}/{f}")
        for op in OPS:
            if f"{op}_in" in z:
                out.append((f, op))
    return out


def _fp64_tol(fname: str, op: str) -> float:
    if fname.startswith("cfg_fan") and op == "projection_t":
        return 3e-4   # white-noise sinogram input: reference fp32 drift dominates
    if fname.startswith("cfg_fan") and op == "fbp":
        return 3e-5   # ramp-filtered (high-pass) sinogram feeds the fp32 walk
    return 1e-5


@pytest.mark.parametrize("fname,op", _cases())
def test_fp64_oracle_matches_reference(oracle_mod, fname, op):
    O = oracle_mod
    z = np.load(f"{GOLDEN}/{fname}")
    x, y = z[f"{op}_in"], z[f"{op}_out"]
    mode = O.MODE_F64_ON_F32 if x.dtype == np.float32 else O.MODE_F64
    got = O.run(op, x, z["options"], mode)
    err = O.rel_l2(got, y)
    assert err <= _fp64_tol(fname, op), f"{fname}:{op} rel-L2 {err:.3e}"


@pytest.mark.parametrize("fname,op", [c for c in _cases() if not c[0].startswith("cfg_")])
def test_fp32_oracle_tracks_reference_rounding(oracle_mod, fname, op):
    """The fp32 oracle against the reference's fp32 output. The reference is
    compiled with FMA contraction (as nvcc compiles it by default) and the
    oracle without (so it rounds the same on every host), so single roundings
    differ; white-noise inputs expose them at up to ~5e-6 (rel-L2)."""
    O = oracle_mod
    z = np.load(f"{GOLDEN}/{fname}")
    x, y = z[f"{op}_in"], z[f"{op}_out"]
    mode = O.MODE_F32 if x.dtype == np.float32 else O.MODE_F64
    got = O.run(op, x, z["options"], mode)
    err = O.rel_l2(got, y)
    tol = 5e-6 if x.dtype == np.float32 else 1e-13
    assert err <= tol, f"{fname}:{op} rel-L2 {err:.3e}"


@pytest.mark.parametrize("fname", [f for f in golden_files() if "ramp_taps" in np.load(f"{GOLDEN}/{f}")])
def test_ramp_taps_bit_exact(oracle_mod, fname):
    O = oracle_mod
    z = np.load(f"{GOLDEN}/{fname}")
    taps = z["ramp_taps"]
    D = int(z["options"][1])
    got = _ramp(O, z["options"], taps.dtype)
    assert got.shape == (2 * D - 1,)
    assert np.array_equal(got.view(np.uint32 if taps.dtype == np.float32 else np.uint64),
                          taps.view(np.uint32 if taps.dtype == np.float32 else np.uint64))


def _ramp(O, opts, dtype):
    import ctypes
    lib = O._load_oracle()
    o, ptr = O._opts_array(opts)
    out = np.empty(2 * int(o[1]) - 1, dtype)
    mode = O.MODE_F32 if dtype == np.float32 else O.MODE_F64
    rc = lib.oracle_run(O.OP_RAMP, ptr, o.size, mode, 1, None, out.ctypes.data, 0)
    assert rc == 0
    return out


def test_adjoint_pairs_fp64(oracle_mod):
    """<Ax, y> = <x, A^T y> and <Bx, y> = <x, B^T y> in fp64 (ED, parallel);
    for EA, B^T carries the reference's extra dImg/cbar factor
    (src/fan_ea_kernel.cu:590-607), so only A/A^T is an exact pair there."""
    O = oracle_mod
    import math
    from ctlib_gb300.workloads import fan_options, para_options, FAN_ED, FAN_EA
    rng = np.random.default_rng(7)
    cases = [fan_options(50, 70, 40, 36, 1.0, 2.0, 0.2, 2 * math.pi / 50, 120.0, 100.0, 0.7, FAN_ED),
             fan_options(50, 70, 40, 36, 1.0, 0.01, 0.2, 2 * math.pi / 50, 120.0, 100.0, 0.002, FAN_EA),
             para_options(50, 70, 40, 36, 1.0, 1.1, 0.2, math.pi / 50, 0.6)]
    for o in cases:
        x = rng.standard_normal((1, 1, 36, 40))
        y = rng.standard_normal((1, 1, 50, 70))
        Ax = O.run("projection", x, o, O.MODE_F64)
        Aty = O.run("projection_t", y, o, O.MODE_F64)
        lhs, rhs = float((Ax * y).sum()), float((x * Aty).sum())
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0), (o[-1], lhs, rhs)
        if int(o[-1]) != FAN_EA:
            Bty = O.run("backprojection_t", x, o, O.MODE_F64)
            By = O.run("backprojection", y, o, O.MODE_F64)
            lhs, rhs = float((Bty * y).sum()), float((x * By).sum())
            assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0), (o[-1], lhs, rhs)


@pytest.mark.parametrize("fname", [f for f in golden_files() if "backprojection_sv_in" in np.load(f"{GOLDEN}/{f}")])
def test_single_view_backprojection_sums_to_backprojection(oracle_mod, fname):
    """backprojection_sv is backprojection before its sum over views: summing
    its B x V x H x W output over views gives backprojection."""
    O = oracle_mod
    z = np.load(f"{GOLDEN}/{fname}")
    x = z["backprojection_sv_in"].astype(np.float64)
    sv = O.run("backprojection_sv", x, z["options"], O.MODE_F64)
    bp = O.run("backprojection", x, z["options"], O.MODE_F64)
    assert sv.shape == (x.shape[0], x.shape[2], bp.shape[2], bp.shape[3])
    assert O.rel_l2(sv.sum(axis=1, keepdims=True), bp) <= 1e-13


def test_single_view_backprojection_fan_ed_only(oracle_mod):
    from ctlib_gb300.workloads import FAN_EA, fan_options
    opts = fan_options(8, 20, 16, 16, 1.0, 0.01, 0.0, 0.5, 120.0, 100.0, 0.0, FAN_EA)
    with pytest.raises(ValueError):
        oracle_mod.run("backprojection_sv", np.zeros((1, 1, 8, 20)), opts, oracle_mod.MODE_F64)
