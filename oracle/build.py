"""Build recipes for the test-side checkers (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles ``dd_oracle.cpp`` (the CPU restatement) into
  ``oracle/_build/liboracle.so``.
* ``build_ref()`` compiles the reference's own kernel source, read in place from
  a CTLIB checkout (``src/fan_ed_kernel.cu``, ``src/fan_ea_kernel.cu``,
  ``src/para_kernel.cu``), for CPU execution through ``ref_emu/cuda_emu.h``, into
  ``oracle/_ref/libctref.so``. Only the kernel part of each file is used (from
  after its ``#include`` lines up to its first host wrapper); it is streamed to
  the compiler through a pipe, so no copy of the reference source is written
  anywhere. Two ``__shared__`` scalars that every thread writes with the same
  value (``ang_error`` and ``dPoint0``, e.g. src/fan_ed_kernel.cu:53,50) are made
  thread-private: the reference reads each of them and then overwrites it within
  one barrier interval (src/fan_ed_kernel.cu:75-76 and :146), which on the GPU is
  harmless because all warps read before any writes, but which a one-thread-at-
  a-time execution would otherwise turn into a real read-after-write.

* ``build_ref_gpu()`` compiles the same three reference files, and the
  graph-Laplacian kernels of ``src/laplacian_cuda_kernel.cu``, for the GPU, as
  the reference's ``CUDAExtension`` does but for sm_103a, into
  ``oracle/_ref/ref_<file>.cubin.gz``, which ``ref_cuda.py`` loads through the
  CUDA driver API. A generated wrapper (``oracle/_build/ref_gpu/*.cu``)
  includes the reference file by name from the checkout (no copy), turns the
  host wrappers' ``AT_DISPATCH_FLOATING_TYPES`` launches into nothing (they
  need libtorch at run time) and instantiates every kernel for float and
  double. It needs nvcc and the torch headers, so it runs only where a
  checkout is present; the compressed cubins travel with the repository's
  working tree to machines without one.

``build_oracle`` and ``build_ref`` use plain g++ (no cmake, no torch headers). The oracle is built with
``-ffp-contract=off`` so it rounds identically on x86-64 and aarch64 (the fused
operations it means are written as std::fma). The reference kernels are built
with FMA contraction on, as nvcc compiles them by default (--fmad=true), so
expressions such as ``idxview * *dAng + *Ang0`` become one fused multiply-add
as on the GPU.
"""

from __future__ import annotations

import os
import platform
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "libctref.so")
# The CTLIB checkout whose kernels these recipes compile: $CTLIB_REF_ROOT when
# set, else the read-only mount of the build container. Where neither exists
# (a machine that only runs the prebuilt files), build_ref and build_ref_gpu
# return None and the tests that need them skip.
REF_ROOT_ENV = "CTLIB_REF_ROOT"
DEFAULT_REF_ROOT = "/root/reference"


def ref_root() -> str | None:
    """The checkout to build from, or None when there is none."""
    for cand in (os.environ.get(REF_ROOT_ENV), DEFAULT_REF_ROOT):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None

CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off"]


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "dd_oracle.cpp")
    if force or _stale(ORACLE_SO, [src]):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = ORACLE_SO + ".tmp"
        subprocess.run(["g++", *CXXFLAGS, "-fopenmp", src, "-o", tmp], check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


_KERNEL_FILES = (("ref_fan_ed", "fan_ed_kernel.cu"), ("ref_fan_ea", "fan_ea_kernel.cu"),
                 ("ref_para", "para_kernel.cu"))
_PRIVATE = (("__shared__ double ang_error;", "double ang_error;"),
            ("__shared__ scalar_t dPoint0;", "scalar_t dPoint0;"))


def _kernel_text(path: str) -> str:
    with open(path, "r") as f:
        lines = f.read().split("\n")
    out, started = [], False
    for ln in lines:
        if not started:
            if ln.startswith("#include"):
                continue
            started = True
        if re.match(r"^torch::Tensor\b", ln):
            break
        out.append(ln)
    text = "\n".join(out)
    for a, b in _PRIVATE:
        text = text.replace(a, b)
    return text


def build_ref(root: str | None = None, force: bool = False) -> str | None:
    """Compile the reference kernels for CPU execution; None if no checkout."""
    root = root or ref_root()
    if root is None:
        return None
    srcdir = os.path.join(root, "src")
    if not os.path.isdir(srcdir):
        return None
    deps = [os.path.join(srcdir, f) for _, f in _KERNEL_FILES]
    deps += [os.path.join(HERE, "ref_emu", "cuda_emu.h"), os.path.join(HERE, "ref_emu", "ref_driver.inc"),
             os.path.abspath(__file__)]
    if not (force or _stale(REF_SO, deps)):
        return REF_SO
    parts = ['#include "cuda_emu.h"']
    for ns, fname in _KERNEL_FILES:
        parts.append(f"namespace {ns} {{")
        parts.append(f'#line 1 "{fname}"')
        parts.append(_kernel_text(os.path.join(srcdir, fname)))
        parts.append(f"}}  // namespace {ns}")
    with open(os.path.join(HERE, "ref_emu", "ref_driver.inc")) as f:
        parts.append(f.read())
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_SO + ".tmp"
    flags = [f for f in CXXFLAGS if f != "-ffp-contract=off"] + ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    subprocess.run(["g++", *flags, "-w", "-I", os.path.join(HERE, "ref_emu"), "-x", "c++", "-",
                    "-o", tmp], input="\n".join(parts).encode(), check=True)
    os.replace(tmp, REF_SO)
    return REF_SO


# kernels of each reference file with the number of option pointers they take
# (src/fan_ed_kernel.cu:24-946, src/fan_ea_kernel.cu:23-904,
#  src/para_kernel.cu:8-666); rlfilter takes (filter, dets, dDet)
REF_GPU_KERNELS = {
    "ref_fan_ed": (("prj_fan_ed", "prj_t_fan_ed", "bprj_fan_ed", "bprj_t_fan_ed", "bprj_sv_fan_ed"), 11),
    "ref_fan_ea": (("prj_fan_ea", "prj_t_fan_ea", "bprj_fan_ea", "bprj_t_fan_ea"), 11),
    "ref_para": (("prj_para", "prj_t_para", "bprj_para", "bprj_t_para"), 9),
}


# the graph-Laplacian file (src/laplacian_cuda_kernel.cu:10-43): two kernels on a
# 2-D accessor; its GEMM is a cuBLAS call replayed by ref_cuda.py
REF_GPU_LAPLACIAN = ("ref_laplacian", "laplacian_cuda_kernel.cu")


def ref_cubin_path(ns: str) -> str:
    return os.path.join(REF_DIR, f"{ns}.cubin.gz")


def _ref_gpu_wrapper(ns: str, fname: str) -> str:
    lines = [
        "// Written by oracle/build.py: the reference's kernels of " + fname + ",",
        "// included by name from the checkout, instantiated for float and double.",
        "// Test infrastructure only.",
        "#include <torch/extension.h>",
        "#undef AT_DISPATCH_FLOATING_TYPES",
        "#define AT_DISPATCH_FLOATING_TYPES(TYPE, NAME, ...)",
        f'#include "{fname}"',
    ]
    if ns == REF_GPU_LAPLACIAN[0]:
        for t in ("float", "double"):
            a2 = f"torch::PackedTensorAccessor<{t}, 2, torch::RestrictPtrTraits, size_t>"
            lines.append(f"template __global__ void compute_squared_norm<{t}>({a2}, int, int, {t}* __restrict__);")
            lines.append(f"template __global__ void add_norm<{t}>({a2}, int, {t}* __restrict__);")
        return "\n".join(lines) + "\n"
    kernels, nptr = REF_GPU_KERNELS[ns]
    acc = "torch::PackedTensorAccessor<T, 4, torch::RestrictPtrTraits, size_t>"
    for t in ("float", "double"):
        a = acc.replace("<T,", f"<{t},")
        ptrs = ", ".join([f"const {t}* __restrict__"] * nptr)
        for k in kernels:
            lines.append(f"template __global__ void {k}<{t}>({a}, {a}, {ptrs});")
        lines.append(f"template __global__ void rlfilter<{t}>({t}* __restrict__, const {t}* __restrict__, "
                     f"const {t}* __restrict__);")
    return "\n".join(lines) + "\n"


# nvcc flags of torch's CUDAExtension build of the reference (setup.py), with the
# architecture set to this GPU
_REF_NVCC = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-w",
             "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
             "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__",
             "--expt-relaxed-constexpr", "-DTORCH_EXTENSION_NAME=ctlib", "-DTORCH_API_INCLUDE_EXTENSION_H"]


def build_ref_gpu(root: str | None = None, force: bool = False) -> list[str] | None:
    """Compile the reference kernels to compressed sm_103a cubins; None if no checkout."""
    import gzip
    import shutil
    import sysconfig
    root = root or ref_root()
    if root is None:
        return None
    srcdir = os.path.join(root, "src")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.isdir(srcdir) or not os.path.exists(nvcc):
        return None
    try:
        from torch.utils.cpp_extension import include_paths
        incs = include_paths()
    except Exception:
        return None
    incs = incs + [srcdir, sysconfig.get_paths()["include"]]
    wdir = os.path.join(BUILD_DIR, "ref_gpu")
    os.makedirs(wdir, exist_ok=True)
    os.makedirs(REF_DIR, exist_ok=True)
    jobs = []
    for ns, fname in _KERNEL_FILES + (REF_GPU_LAPLACIAN,):
        out = ref_cubin_path(ns)
        if not (force or _stale(out, [os.path.join(srcdir, fname), os.path.abspath(__file__)])):
            continue
        wrapper = os.path.join(wdir, ns + ".cu")
        with open(wrapper, "w") as f:
            f.write(_ref_gpu_wrapper(ns, fname))
        cubin = os.path.join(wdir, ns + ".cubin")
        cmd = [nvcc, *_REF_NVCC, *[a for i in incs for a in ("-I", i)], "-D_GLIBCXX_USE_CXX11_ABI=1",
               wrapper, "-o", cubin]
        jobs.append((subprocess.Popen(cmd), cubin, out))
    for proc, cubin, out in jobs:
        if proc.wait() != 0:
            raise RuntimeError(f"nvcc failed for {cubin}")
        with open(cubin, "rb") as f, gzip.open(out + ".tmp", "wb") as g:
            g.write(f.read())
        os.replace(out + ".tmp", out)
    return [ref_cubin_path(ns) for ns, _ in _KERNEL_FILES + (REF_GPU_LAPLACIAN,)]


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_gpu(force="--force" in sys.argv))
