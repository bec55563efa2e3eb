"""The native halo-correction driver of the C ABI (hg_correct_halo) against
the Python corrector (same kernels, same host arithmetic except the 2x2
solve: the driver reproduces x86-64 LAPACK's rounding, the Python path uses
this host's numpy, which on aarch64 rounds differently in the last bit and
can move the step at which |r| < 1e-12 is first met): statuses equal,
iteration counts within 2, converged states and periods within the
corrected-orbit tolerance 1e-10; and against the reference's own corrected
orbits (<= 1e-10)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_native_matches_python_corrector(gpu):
    from hiten_gb300 import corrector, halo
    mu = W.MU_EM
    pt, az, zen = W.halo_guess_params(256, seed=4)
    g = np.concatenate([halo.third_order_guess(mu, 1, az[pt == 1], zen[pt == 1]),
                        halo.third_order_guess(mu, 2, az[pt == 2], zen[pt == 2])])
    g[:3, 0] += np.array([0.3, -0.2, 0.05])   # hopeless guesses: no crossing or a failed line search
    py = corrector.correct_halo(g, mu)
    nat = corrector.correct_halo_native(g, mu)
    assert np.array_equal(py.status, nat.status)
    assert np.max(np.abs(py.iterations - nat.iterations)) <= 2
    ok = py.status == 0
    assert ok.sum() > 200
    assert np.max(np.abs(py.x0[ok] - nat.x0[ok])) <= 1e-10
    assert np.max(np.abs(py.period[ok] - nat.period[ok])) <= 1e-10


def test_native_matches_reference_golden(gpu):
    from hiten_gb300 import corrector
    h = np.load(os.path.join(GOLDEN, "halo.npz"))
    res = corrector.correct_halo_native(h["guess"], float(h["mu"]))
    assert np.all(res.status == 0)
    assert np.max(np.abs(res.x0 - h["x0"])) <= 1e-10
    assert np.max(np.abs(res.period - h["period"])) <= 1e-10
    assert np.all(np.abs(res.iterations - h["iterations"]) <= 1)
