"""Build the CPU oracle (``oracle/_build/libhgo.so``) with gcc.

-ffp-contract=off keeps every multiply and add separately rounded, as the
reference's numba kernels (fastmath=False) do; the only fused operations
are the explicit fma() calls that mirror numpy's dot.  -fno-builtin stops gcc
from rewriting pow(x, 2.0) as x*x: the reference run without numba calls
libm pow there, which is not always correctly rounded.  Quad-precision pow
comes from libquadmath on x86-64 and from binary128 long double on aarch64.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhgo.so")
SOURCES = [os.path.join(HERE, "hgo.c")]
HEADERS = [os.path.join(HERE, "hgo.h"), os.path.join(HERE, "hgo_tableaux.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SOURCES + HEADERS + [__file__])


def build(force=False):
    """Compile the oracle if needed and return the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fno-builtin", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + SOURCES + ["-lm", "-lpthread"]
    if platform.machine() not in ("aarch64", "arm64"):
        cmd.append("-lquadmath")
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
