"""The batched Newton corrector's host logic (hiten_gb300/corrector.py) driven
by the CPU oracle in PYTHON mode reproduces the reference's orbit.correct()
results bit for bit (corrected state, period, iteration count), starting
from the reference's own initial guesses (tests/golden/halo.npz)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle_backends import OracleShootingBackend


@pytest.fixture(scope="module")
def halo():
    return np.load(os.path.join(GOLDEN, "halo.npz"))


@pytest.mark.parametrize("trials", [None, 4])
def test_corrector_logic_reproduces_reference(oracle, halo, trials):
    from hiten_gb300 import corrector
    mu = float(halo["mu"])
    be = OracleShootingBackend(oracle, mu, oracle.MODE_PYTHON)
    res = corrector.correct_halo(halo["guess"], mu, options=corrector.HaloCorrectionOptions(trials_per_round=trials),
                                 backend=be)
    oracle.set_mode(oracle.MODE_PYTHON)
    assert np.all(res.status == 0)
    assert np.array_equal(res.iterations, halo["iterations"])
    assert np.array_equal(res.x0, halo["x0"])
    assert np.array_equal(res.period, halo["period"])


def test_third_order_guess_matches_reference(halo):
    from hiten_gb300 import halo as H
    mu = float(halo["mu"])
    for i in range(len(halo["point"])):
        g = H.third_order_guess(mu, int(halo["point"][i]), halo["az"][i], str(halo["zenith"][i]))[0]
        assert np.max(np.abs(g - halo["guess"][i])) <= 1e-12
