"""The kernels divide through hg_div_rn (one reciprocal per denominator, then
a corrected product); it must return the same bits as IEEE division."""
import os
import platform
import subprocess

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu


def test_div_rn_matches_ieee_division(gpu, tmp_path):
    exe = str(tmp_path / "markstein_check")
    subprocess.check_call(["nvcc", "-std=c++17", "-gencode=arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
                           "-I" + os.path.join(REPO, "hiten_gb300", "csrc"),
                           os.path.join(REPO, "tests", "native", "markstein_check.cu"), "-o", exe])
    out = subprocess.check_output([exe, str(1 << 30)], timeout=300).decode().split()
    assert out[2] == "no" or out[2] == "no error" or out[2].startswith("no"), out
    assert int(out[0]) == 1 << 30
    assert int(out[1]) == 0, f"{out[1]} quotients differ from IEEE division"


def test_pow15_25_device_matches_host_method_and_quad(gpu, tmp_path):
    """The device x^1.5 / x^2.5 (Goldschmidt square root from the hardware
    estimate) gives the bits of the host method and of quad-precision pow."""
    exe = str(tmp_path / "pow15_check")
    cmd = ["nvcc", "-std=c++17", "-gencode=arch=compute_103a,code=sm_103a", "-O3", "--fmad=false",
           "-I" + os.path.join(REPO, "hiten_gb300", "csrc"), os.path.join(REPO, "tests", "native", "pow15_check.cu"),
           "-o", exe]
    if platform.machine() not in ("aarch64", "arm64"):
        cmd.append("-lquadmath")
    subprocess.check_call(cmd)
    out = subprocess.check_output([exe, str(1 << 30), str(1 << 18)], timeout=600).decode().split()
    n, bad, seed_log2, nq, qbad, err = int(out[0]), int(out[1]), float(out[2]), int(out[3]), int(out[4]), out[5]
    assert err == "ok"
    assert n == 1 << 30 and bad == 0, f"{bad} of {n} powers differ from the host method"
    assert seed_log2 < -14, "hardware estimate less accurate than two iterations absorb"
    assert nq == 1 << 18 and qbad == 0, f"{qbad} powers differ from quad precision"
