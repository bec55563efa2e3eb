"""Argument validation of the reference-shaped API (no GPU needed: every
check runs before any device work), mirroring integrators/base.py:148-191 and
dynamics/base.py:461-493."""
import numpy as np
import pytest

from hiten_gb300 import dynamics as D
from hiten_gb300 import integrators as I

MU = 0.012150585609624


def test_runge_kutta_factory():
    assert isinstance(I.RungeKutta(8), I.GpuFixedRK) and I.RungeKutta(8).order == 8
    assert isinstance(I.RungeKutta(853), I.GpuDOP853)
    with pytest.raises(ValueError):
        I.RungeKutta(5)
    with pytest.raises(ValueError):
        I.FixedRK(3)
    with pytest.raises(ValueError):
        I.AdaptiveRK(5)


@pytest.mark.parametrize("integ", [I.RungeKutta(8), I.RungeKutta(853)])
def test_validate_inputs(integ):
    sys6 = D.CR3BPSystem(MU, 6)
    with pytest.raises(ValueError, match="dimension"):
        integ.integrate(sys6, np.zeros(5), np.linspace(0, 1, 3))
    with pytest.raises(ValueError, match="at least 2"):
        integ.integrate(sys6, np.zeros(6), np.array([0.0]))
    with pytest.raises(ValueError, match="monotonic"):
        integ.integrate(sys6, np.zeros(6), np.array([0.0, 1.0, 0.5]))
    # zero span short-circuit: constant solution, no device work
    sol = integ.integrate(sys6, np.arange(6.0), np.zeros(4))
    assert sol.states.shape == (4, 6) and np.all(sol.states == np.arange(6.0))


def test_propagate_dynsys_zero_span_and_validation():
    s = D.CR3BPSystem(MU, 42)
    with pytest.raises(ValueError):
        D.propagate_dynsys(s, np.zeros(6), 0.0, 1.0)
    sol = D.propagate_dynsys(D.CR3BPSystem(MU, 6), np.ones(6), 0.0, 1e-12, forward=-1, steps=2)
    assert np.array_equal(sol.states, np.ones((2, 6))) and np.array_equal(sol.times, -np.array([0.0, 1e-12]))
    with pytest.raises(ValueError):
        D.propagate_dynsys(D.CR3BPSystem(MU, 6), np.ones(6), 0.0, 1.0, method="symplectic")
    with pytest.raises(ValueError):
        D.EventConfig(direction=2)
    with pytest.raises(ValueError):
        D.CR3BPSystem(MU, 7)


def test_flip_ranges():
    assert D._flip_range(None, 6) == (0, 6)
    assert D._flip_range(slice(36, 42), 42) == (36, 42)
    assert D._flip_range([3, 4, 5], 6) == (3, 6)
    with pytest.raises(ValueError):
        D._flip_range([0, 2], 6)
