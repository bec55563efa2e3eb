"""Compile the CUDA library ``hiten_gb300/libhitengpu.so`` for sm_103a.

Translation units csrc/hg_*.cu (each including the kernel header) are
compiled in parallel and linked in-tree with nvcc: ``-gencode arch=compute_103a,code=sm_103a``, C++20,
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
BUILD_DIR = os.path.join(HERE, "_build")
SOURCES = [os.path.join(CSRC, "hg_api.cu"), os.path.join(CSRC, "hg_noalloc.cu"), os.path.join(CSRC, "hg_section.cu"),
           os.path.join(CSRC, "hg_connect.cu"), os.path.join(CSRC, "hg_correct.cu"),
           os.path.join(CSRC, "hg_correct_graph.cu"), os.path.join(CSRC, "hg_serve.cu")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("hg_kernels.cuh", "hg_pair.cuh", "hg_crmath.cuh", "hg_crmath_tables.h",
                                                  "hg_tableaux.h", "hg_internal.h")] + [os.path.join(REPO, "include", "hitengpu.h")]
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
    # host code: no contraction and no builtin pow (the reference's numpy
    # arithmetic); device code: --fmad=false
    flags = ["-std=c++20", ARCH, "-O3", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-builtin-pow",
             "-I" + os.path.join(REPO, "include"), "-I" + CSRC]
    if verbose:
        flags.append("-Xptxas=-v")
    objs = [os.path.join(BUILD_DIR, os.path.basename(s) + ".o") for s in SOURCES]
    os.makedirs(BUILD_DIR, exist_ok=True)
    # one translation unit per process, compiled in parallel
    procs = [subprocess.Popen([nvcc(), "-c"] + flags + ["-o", o, s]) for s, o in zip(SOURCES, objs)]
    rcs = [p.wait() for p in procs]
    if any(rcs):
        raise RuntimeError(f"nvcc failed ({rcs})")
    subprocess.check_call([nvcc(), ARCH, "-shared", "-cudart", "static", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
