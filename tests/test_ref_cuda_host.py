"""Host-side pieces of the reference's GPU build (oracle/build.py:build_ref_gpu,
oracle/ref_cuda.py) that need no GPU: the wrapper text, the kernel-name
parsing and the argument checks made before any launch."""

import pytest

from oracle import build as obuild
from oracle import ref_cuda


def test_wrapper_instantiates_every_kernel():
    for ns, fname in obuild._KERNEL_FILES:
        text = obuild._ref_gpu_wrapper(ns, fname)
        kernels, nptr = obuild.REF_GPU_KERNELS[ns]
        assert f'#include "{fname}"' in text
        for t in ("float", "double"):
            for k in kernels:
                line = [ln for ln in text.splitlines() if f" {k}<{t}>(" in ln]
                assert len(line) == 1
                assert line[0].count(f"const {t}* __restrict__") == nptr
            assert f"rlfilter<{t}>" in text


def test_demangled_heads():
    assert ref_cuda._demangle_head("_Z10prj_fan_edIfEvN2at27GenericPackedTensorAccessorIT_Lm4ENS0_17"
                                   "RestrictPtrTraitsEmEES4_PKS1_S7_S7_S7_S7_S7_S7_S7_S7_S7_S7_") == \
        ("prj_fan_ed", "f")
    assert ref_cuda._demangle_head("_Z12prj_t_fan_eaIdEvN2at27Gen") == ("prj_t_fan_ea", "d")
    assert ref_cuda._demangle_head("_Z8rlfilterIfEvPT_PKS0_S3_") == ("rlfilter", "f")
    assert ref_cuda._demangle_head("_Z8rlfilterfv") is None
    assert ref_cuda._demangle_head("main") is None
    assert ref_cuda._demangle_head("_Z40short") is None


def test_kernel_names_cover_ops():
    for scan, suffix in ref_cuda.SCAN_SUFFIX.items():
        kernels, _ = obuild.REF_GPU_KERNELS[ref_cuda.SCAN_NS[scan]]
        for op, base in ref_cuda.OPS.items():
            if op == 5 and scan != 0:
                continue
            assert f"{base}_{suffix}" in kernels


def test_no_gpu_no_module():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    with pytest.raises(RuntimeError):
        ref_cuda.RefCuda()

