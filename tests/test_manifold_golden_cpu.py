"""Manifold seeding, its eigenvector choice and orbit stability on the host,
pinned to the reference's own outputs (tests/golden/manifold.npz, made by
tests/golden/make_golden_manifold.py from the unmodified reference).

Given the reference's STM grid, the library's eigen-decomposition picks the
same eigenvector and its seeding gives the same seeds as
_compute_manifold_section, bit for bit; its stability indices of the
reference's monodromy matrices equal orbit.compute_stability()'s, and the CPU
oracle (reference arithmetic) reproduces those monodromy matrices.  numpy's
eig and matmul are the host's LAPACK/BLAS: bit equality is asserted on the
fixture host's architecture (x86-64), agreement to 1e-13 elsewhere."""
import os
import platform

import numpy as np
import pytest

from hiten_gb300 import manifold as M
from hiten_gb300 import stability as S

HERE = os.path.dirname(os.path.abspath(__file__))
SAME_HOST = platform.machine() in ("x86_64", "AMD64")


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "manifold.npz"))


def _eq(a, b, rtol=1e-13):
    if SAME_HOST:
        assert np.array_equal(a, b)
    else:
        assert np.allclose(a, b, rtol=rtol, atol=rtol)


@pytest.mark.parametrize("tag", ["stable", "unstable"])
def test_eigen_decomposition_and_eigenvector(g, tag):
    sn, un, cn, Ws, Wu, Wc = S.eigenvalue_decomposition(g[f"{tag}/phi_T"], 1e-6)
    _eq(sn, g[f"{tag}/sn"])
    _eq(un, g[f"{tag}/un"])
    _eq(Ws, g[f"{tag}/Ws"])
    _eq(Wu, g[f"{tag}/Wu"])
    v = M.stable_eigvec(g[f"{tag}/phi_T"], stable=(tag == "stable"))
    _eq(v, g[f"{tag}/eigvec"])
    assert v.dtype == np.complex128


@pytest.mark.parametrize("tag", ["stable", "unstable"])
def test_seeds_match_compute_manifold_section(g, tag):
    tt, PHI, T = g[f"{tag}/tt"], g[f"{tag}/PHI"], float(g[f"{tag}/period"])
    d = int(g[f"{tag}/direction"])
    got = np.array([M.seeds(tt, PHI, T, [f], [disp], g[f"{tag}/eigvec"], direction=d)[0]
                    for f, disp in zip(g[f"{tag}/fractions"], g[f"{tag}/displacements"])])
    _eq(got, g[f"{tag}/seeds"])


def test_missing_eigenvector_raises(g):
    with pytest.raises(ValueError, match="not available"):
        M.stable_eigvec(g["stable/phi_T"], stable=True, NN=3)


def test_stability_indices_match_compute_stability(g):
    for k in range(len(g["stab_period"])):
        nu, w, V = S.stability_indices(g["stab_monodromy"][k])
        _eq(nu, g["stab_nu"][k])
        _eq(w, g["stab_eigvals"][k])
        _eq(V, g["stab_eigvecs"][k])


def test_oracle_reproduces_the_reference_monodromy(g, oracle):
    """The oracle in the reference's arithmetic gives the monodromy matrices
    the reference decomposed, bit for bit (dynamics/rtbp.py:258-340 with its
    defaults: DOP853 1e-12, 2000 dense samples, the last one)."""
    oracle.set_mode(oracle.MODE_PYTHON)
    for k in range(len(g["stab_period"])):
        y0 = np.zeros(42)
        y0[:36] = np.eye(6).ravel()
        y0[36:] = g["stab_x0"][k]
        y, _, _, _ = oracle.dop853_dense(y0, np.linspace(0.0, float(g["stab_period"][k]), 2000), float(g["mu"]),
                                         max_step=1e4, flip=(36, 42))
        assert np.array_equal(y[-1, :36].reshape(6, 6), g["stab_monodromy"][k])


def test_filters_reference_values_from_states(g):
    """The acceptance quantities recomputed from the reference's sampled
    trajectories in numba's arithmetic (x**2 -> x*x, x**0.5 -> sqrt) stay
    within a few ulps of the reference's pure-Python values (libm pow)."""
    mu = float(g["mu"])
    for k, st in enumerate(g["stable/traj_states"]):
        x, y, z = st[:, 0], st[:, 1], st[:, 2]
        r1 = np.sqrt(((x + mu) * (x + mu) + y * y) + z * z)
        assert r1.min() == g["stable/traj_min_r1"][k]
