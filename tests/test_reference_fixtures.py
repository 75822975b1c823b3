"""The golden fixtures are the reference's own outputs: where a CTLIB checkout
is present, its kernels (src/fan_ed_kernel.cu, src/fan_ea_kernel.cu,
src/para_kernel.cu, executed on the CPU by oracle/ref_emu) are run again on
every fixture's inputs and must reproduce the recorded outputs bit for bit;
fbp replays the wrapper's torch glue the same way (tests/golden/make_golden.py).
Skipped where no checkout is available (the GPU machines)."""

import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden_files

OPS = ("projection", "projection_t", "backprojection", "backprojection_t", "backprojection_sv")


def _cases():
    out = []
    for f in golden_files():
        z = np.load(f"{GOLDEN}/{f}")
        for op in OPS + ("fbp",):
            if f"{op}_in" in z:
                out.append((f, op))
    return out


@pytest.fixture(scope="module")
def ref():
    import oracle
    if not oracle.ref_available():
        pytest.skip("no CTLIB checkout to run the reference kernels from")
    oracle._load_ref()
    return oracle


@pytest.mark.parametrize("fname,op", _cases())
def test_fixture_is_reference_output(ref, fname, op):
    z = np.load(f"{GOLDEN}/{fname}")
    x, want, opts = z[f"{op}_in"], z[f"{op}_out"], z["options"]
    before = ref.ref_oob_count()
    if op == "fbp":
        sys.path.insert(0, GOLDEN)
        from make_golden import ref_fbp
        got, _ = ref_fbp(x, list(opts))
    else:
        got = ref.ref_run(op, x, opts, x.dtype.type)
    assert ref.ref_oob_count() == before
    assert got.shape == want.shape and got.dtype == want.dtype
    assert np.array_equal(got, want)
