"""The kernels divide through hg_div_rn (one reciprocal per denominator, then
a corrected product); it must return the same bits as IEEE division."""
import os
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
