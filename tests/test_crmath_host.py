"""The correctly rounded power functions of the kernels (csrc/hg_crmath.cuh),
compiled as host C++, agree with quad-precision pow rounded once."""
import os
import platform
import subprocess

from conftest import REPO


def test_crmath_matches_quad_pow(tmp_path):
    exe = str(tmp_path / "crmath_check")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-builtin",
           "-I" + os.path.join(REPO, "hiten_gb300", "csrc"), os.path.join(REPO, "tests", "native", "crmath_check.cpp"),
           "-o", exe]
    if platform.machine() not in ("aarch64", "arm64"):
        cmd.append("-lquadmath")
    subprocess.check_call(cmd)
    out = subprocess.check_output([exe, "200000"]).decode().split()
    n, bad15, bad25, badp = map(int, out)
    assert n == 200000 and bad15 == 0 and bad25 == 0 and badp == 0


def test_integer_pipe_compares_match_ieee(tmp_path):
    """The kernels' step control compares bit patterns on the integer pipes
    (hg_gt0, hg_lt_pos, hg_gt, ...); each equals the IEEE comparison, NaNs of
    either sign and signed zeros included."""
    exe = str(tmp_path / "cmp_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                           "-I" + os.path.join(REPO, "hiten_gb300", "csrc"),
                           os.path.join(REPO, "tests", "native", "cmp_check.cpp"), "-o", exe])
    checks, bad = map(int, subprocess.check_output([exe, "100000"]).decode().split())
    assert checks > 1_000_000 and bad == 0


def test_log_reduction_on_integer_pipes_is_bit_identical(tmp_path):
    """hg_log_dd forms its reduction (exponent, sqrt(2) fold, table index
    with round-half-even, F = 1 + j/1024) from the bit pattern; the outputs
    equal those of the same function with the reduction in floating point,
    bit for bit, on random, boundary and tie inputs.  hg_exp_dd's overflow
    guards compare on the integer pipes too."""
    exe = str(tmp_path / "logexp_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-builtin",
                           "-I" + os.path.join(REPO, "hiten_gb300", "csrc"),
                           os.path.join(REPO, "tests", "native", "logexp_check.cpp"), "-o", exe])
    n_in, bad, n_exp, bad_exp = map(int, subprocess.check_output([exe, "400000"]).decode().split())
    assert n_in > 1_000_000 and bad == 0 and n_exp == 15 and bad_exp == 0
