"""Batched halo-family continuation (hiten_gb300/continuation.py) driven by
the CPU oracle in PYTHON mode reproduces the reference's own orbit.generate()
families bit for bit: members, periods, continued parameters, accepted and
rejected counts and iterations (tests/golden/family.npz: a secant family, a
natural-parameter family and a secant family whose first steps are too long
and get halved).  All three families advance together, one batched
correction per round."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle_backends import OracleShootingBackend


@pytest.fixture(scope="module")
def fam():
    return np.load(os.path.join(GOLDEN, "family.npz"))


def _options(fam, i):
    from hiten_gb300.continuation import ContinuationOptions
    z0 = fam[f"{i}/seed"][2]
    return ContinuationOptions(step=(float(fam[f"{i}/step"]),), target=([z0 - 1.0], [z0 + 1.0]),
                               max_members=int(fam[f"{i}/members"]), stepper=str(fam[f"{i}/stepper"]))


def test_families_reproduce_reference(oracle, fam):
    from hiten_gb300 import continuation as Cn
    mu = float(fam["mu"])
    n = 3
    seeds = np.array([fam[f"{i}/seed"] for i in range(n)])
    periods = np.array([float(fam[f"{i}/seed_period"]) for i in range(n)])
    be = OracleShootingBackend(oracle, mu, oracle.MODE_PYTHON)
    res = Cn.continue_halo_families(seeds, periods, mu, options=[_options(fam, i) for i in range(n)], backend=be)
    oracle.set_mode(oracle.MODE_PYTHON)
    for i, r in enumerate(res):
        assert r.accepted_count == int(fam[f"{i}/accepted"]), i
        assert r.rejected_count == int(fam[f"{i}/rejected"]), i
        assert r.iterations == int(fam[f"{i}/iterations"]), i
        assert np.array_equal(np.array(r.family), fam[f"{i}/family"]), i
        assert np.array_equal(np.array(r.periods), fam[f"{i}/periods"]), i
        assert np.array_equal(np.array(r.parameter_values), fam[f"{i}/params"]), i
    assert res[2].rejected_count > 0


def test_step_clamp_and_shrink_policy():
    from hiten_gb300.continuation import ContinuationOptions, _Family
    o = ContinuationOptions(step=(0.5,), step_max=0.3, step_min=0.01, stepper="natural",
                            shrink_policy=lambda s: s * 0.1)
    f = _Family(np.array([0.8, 0, 0.01, 0, 0.1, 0]), 3.0, o)
    assert np.allclose(f.predict(), [0.8, 0, 0.51, 0, 0.1, 0])  # the first prediction uses the raw step
    f.reject()
    assert np.allclose(f.step, [0.05])                          # shrink policy, then clamped into range
    f.reject()
    assert np.allclose(f.step, [0.01])                          # clamped at step_min
    with pytest.raises(ValueError):
        _Family(np.zeros(6), 1.0, ContinuationOptions(stepper="pseudo-arclength"))
