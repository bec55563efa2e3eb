"""Compile the CUDA library ``hiten_gb300/libhitengpu.so`` for sm_103a.

One translation unit (csrc/hg_api.cu including the kernel header), built
in-tree with nvcc: ``-gencode arch=compute_103a,code=sm_103a``, C++20,
``--fmad=false`` (no multiply-add contraction: every product and sum is
rounded separately, as in the reference's numba kernels; fused operations
appear only as explicit fma() calls).  The CUDA runtime is linked
statically so the library carries no dependency on a particular
libcudart next to the PyTorch wheel.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libhitengpu.so")
SOURCES = [os.path.join(CSRC, "hg_api.cu")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("hg_kernels.cuh", "hg_crmath.cuh", "hg_crmath_tables.h",
                                                  "hg_tableaux.h")] + [os.path.join(REPO, "include", "hitengpu.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the hiten_gb300 CUDA library cannot be built")


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in DEPS + [__file__])


def build(force=False, verbose=False):
    """Build the library if any source is newer than it; return its path."""
    if not force and not stale():
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), "-std=c++20", ARCH, "-O3", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
           "-cudart", "static", "-I" + os.path.join(REPO, "include"), "-I" + CSRC, "-o", tmp] + SOURCES
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
