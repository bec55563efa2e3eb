"""The reference's event-semantics cases (integrators/_tests/test_events.py)
on the oracle, in the kernels' arithmetic (DEVICE mode) and the reference's
(PYTHON mode): the outcomes the reference asserts, on CR3BP motion (see
tests/event_semantics.py), for DOP853 and for fixed-step RK4 with an event,
including a step that ends exactly on the plane."""
import numpy as np
import pytest

from event_semantics import BASE, CASES, MU, check_case


@pytest.mark.parametrize("mode", ["DEVICE", "PYTHON"])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_dop853_event_case(oracle, mode, case):
    name, y0, tmax, c, direction, expect = case
    oracle.set_mode(getattr(oracle, f"MODE_{mode}"))
    try:
        r = oracle.dop853_event(y0, 0.0, tmax, MU, 0, c, direction, 1, max_step=1e4)
    finally:
        oracle.set_mode(oracle.MODE_PYTHON)
    check_case(name, y0, tmax, c, direction, expect, r["n_hits"], r["hit_t"][0] if r["n_hits"] else np.nan,
               r["hit_y"][0] if r["n_hits"] else None, r["t_end"], r["y_end"])


@pytest.mark.parametrize("mode", ["DEVICE", "PYTHON"])
def test_dop853_endpoint_zero_is_detected(oracle, mode):
    """The plane placed exactly at the state the integrator reaches at tmax
    (the last step lands on tmax): g is exactly 0 at that step's end, which
    counts as a crossing; the hit is at tmax on the plane."""
    oracle.set_mode(getattr(oracle, f"MODE_{mode}"))
    try:
        tmax = 0.1
        free = oracle.dop853_event(BASE, 0.0, tmax, MU, 0, -10.0, 0, 1, max_step=1e4)
        c = float(free["y_end"][0])
        r = oracle.dop853_event(BASE, 0.0, tmax, MU, 0, c, +1, 1, max_step=1e4)
    finally:
        oracle.set_mode(oracle.MODE_PYTHON)
    assert free["n_hits"] == 0 and r["n_hits"] == 1
    assert abs(r["hit_t"][0] - tmax) < 1e-12
    assert abs(r["hit_y"][0][0] - c) < 1e-12


def test_fixed_rk4_endpoint_zero_is_detected(oracle):
    """Fixed-step RK4 stepping exactly onto the plane at t = 0.1."""
    t = np.linspace(0.0, 0.1, 11)
    oracle.set_mode(oracle.MODE_DEVICE)
    try:
        states, _ = oracle.fixed_rk(4, BASE, t, MU)
        c = float(states[-1][0])
        hit, th, yh, _ = oracle.fixed_rk_event(4, BASE, t, MU, 0, c, +1)
    finally:
        oracle.set_mode(oracle.MODE_PYTHON)
    # the refinement stops once |g| <= gtol = 1e-12, i.e. within 1e-12 / |dx/dt| of the
    # endpoint in time (the reference's unit-slope case makes the two bounds equal)
    assert hit and abs(th - 0.1) < 2e-12 and abs(yh[0] - c) <= 1e-12
