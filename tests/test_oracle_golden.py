"""The CPU oracle in PYTHON mode reproduces the reference's own outputs
(golden fixtures generated by tests/golden/make_golden.py) bit for bit."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import stm_state

pytestmark = pytest.mark.filterwarnings("ignore")


def _load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def _cases(f):
    return sorted(set(k.rsplit("/", 1)[0] for k in f.files if "/" in k))


@pytest.fixture(scope="module")
def py_oracle(oracle):
    oracle.set_mode(oracle.MODE_PYTHON)
    yield oracle
    oracle.set_mode(oracle.MODE_PYTHON)


def test_rhs6_rhs42_bit_exact(py_oracle):
    r = _load("rhs.npz")
    mu = float(r["mu"])
    d6 = np.array([py_oracle.rhs(s, mu) for s in r["s6"]])
    d42 = np.array([py_oracle.rhs(s, mu) for s in r["y42"]])
    assert np.array_equal(d6, r["d6"])
    assert np.array_equal(d42, r["d42"])


@pytest.mark.parametrize("case", _cases(np.load(os.path.join(GOLDEN, "fixed.npz"))))
def test_fixed_bit_exact(py_oracle, case):
    f = _load("fixed.npz")
    mu = float(f["mu"])
    kind = case.split("/")[0]
    y0 = f[case + "/y0"]
    S = f[case + "/states"]
    if kind == "rk8_42":
        out, st = py_oracle.fixed_rk(8, y0, np.linspace(0.0, 3.0, 3001), mu)
        out = out[::100]
    elif kind == "rk4_42":
        out, st = py_oracle.fixed_rk(4, y0, np.linspace(0.0, 1.5, 601), mu)
        out = out[::50]
    elif kind == "rk8_42_bwd":
        out, st = py_oracle.fixed_rk(8, stm_state(y0), np.linspace(0.0, 2.0, 401), mu, fwd=-1, flip=(36, 42))
        out = out[::50]
    else:
        order = int(kind[2])
        fwd = -1 if kind.endswith("bwd") else 1
        out, st = py_oracle.fixed_rk(order, y0, np.linspace(0.0, 2.0, 801), mu, fwd=fwd)
        out = out[::20]
    assert st == 0
    assert np.array_equal(out, S)


@pytest.mark.parametrize("case", _cases(np.load(os.path.join(GOLDEN, "adaptive.npz"))))
def test_adaptive_bit_exact(py_oracle, case):
    a = _load("adaptive.npz")
    mu = float(a["mu"])
    kind, i = case.split("/")
    y0 = a[case + "/y0"]
    t = a[case + "/t"]
    S = a[case + "/states"]
    if kind == "stm_halo":
        fwd = 1 if i == "0" else -1
        out, na, nr, st = py_oracle.dop853_dense(stm_state(y0), np.linspace(0.0, 2.749936405299241, 40), mu,
                                                 fwd=fwd, flip=(36, 42))
        assert np.array_equal(out, S)
    elif kind == "dense6":
        out, na, nr, st = py_oracle.dop853_dense(y0, np.linspace(0.0, 4.0, 101), mu, rtol=1e-11, atol=1e-11)
        assert np.array_equal(out, S)
    elif kind.startswith("manifold"):
        fwd = 1 if kind.endswith("fwd") else -1
        r = py_oracle.dop853_event(y0, 0.0, 8.0, mu, 0, 1 - mu, 0, 1, max_step=1e4, fwd=fwd, flip=(0, 6))
        if r["n_hits"]:
            assert r["hit_t"][0] * fwd == t[-1] and np.array_equal(r["hit_y"][0], S[-1])
        else:
            assert t[-1] == 8.0 * fwd and np.array_equal(r["y_end"], S[-1])
    elif kind == "fixed_event":
        hit, th, yh, _ = py_oracle.fixed_rk_event(8, y0, np.linspace(0.0, 6.0, 601), mu, 1, 0.0, -1)
        assert hit == 1
        assert th == t[-1] and np.array_equal(yh, S[-1])
    else:  # section: y = 0, decreasing
        r = py_oracle.dop853_event(y0, 0.0, 20.0, mu, 1, 0.0, -1, 1, rtol=1e-11, atol=1e-11, max_step=1e4)
        assert r["n_hits"] == 1
        assert r["hit_t"][0] == t[-1] and np.array_equal(r["hit_y"][0], S[-1])


def test_singlehit_crossing_bit_exact(py_oracle):
    """poincare/singlehit/backend.py: alignment to 1e-12 is a zero-span no-op,
    then DOP853 (rtol=atol=1e-12, max_step=inf) over [0, pi - 1e-12]."""
    c = _load("crossing.npz")
    mu = float(c["mu"])
    for i in range(len(c["t"])):
        r = py_oracle.dop853_event(c["y0"][i], 0.0, np.pi - 1e-12, mu, 1, 0.0, 0, 1)
        assert r["n_hits"] == 1
        assert 1e-12 + r["hit_t"][0] == c["t"][i]
        assert np.array_equal(r["hit_y"][0], c["state"][i])
