"""The reference's event-semantics cases (integrators/_tests/test_events.py,
restated on CR3BP motion in tests/event_semantics.py) on the GPU: the
outcomes the reference asserts, and bit for bit the oracle's DEVICE mode --
DOP853 with an event, fixed-step RK4 with an event, and steps that end
exactly on the plane."""
import numpy as np
import pytest

from event_semantics import BASE, CASES, MU, check_case

pytestmark = pytest.mark.gpu


def _device(oracle, fn):
    oracle.set_mode(oracle.MODE_DEVICE)
    try:
        return fn()
    finally:
        oracle.set_mode(oracle.MODE_PYTHON)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_dop853_event_case(gpu, oracle, case):
    name, y0, tmax, c, direction, expect = case
    ev = gpu.EventSpec(index=0, offset=c, direction=direction, max_hits=1)
    r = gpu.propagate_dop853(y0[None], 0.0, tmax, MU, max_step=1e4, event=ev)
    n = int(r.n_hits[0])
    ht = float(r.hit_t[0, 0]) if n else np.nan
    hy = r.hit_y[0, 0].cpu().numpy() if n else None
    check_case(name, y0, tmax, c, direction, expect, n, ht, hy, float(r.t_end[0]), r.y_end[0].cpu().numpy())
    o = _device(oracle, lambda: oracle.dop853_event(y0, 0.0, tmax, MU, 0, c, direction, 1, max_step=1e4))
    assert n == o["n_hits"] and float(r.t_end[0]) == o["t_end"]
    assert np.array_equal(r.y_end[0].cpu().numpy(), o["y_end"])
    if n:
        assert ht == o["hit_t"][0] and np.array_equal(hy, o["hit_y"][0])


def test_dop853_endpoint_zero_is_detected(gpu, oracle):
    tmax = 0.1
    free = gpu.propagate_dop853(BASE[None], 0.0, tmax, MU, max_step=1e4)
    c = float(free.y_end[0, 0])
    ev = gpu.EventSpec(index=0, offset=c, direction=+1, max_hits=1)
    r = gpu.propagate_dop853(BASE[None], 0.0, tmax, MU, max_step=1e4, event=ev)
    assert int(r.n_hits[0]) == 1
    assert abs(float(r.hit_t[0, 0]) - tmax) < 1e-12 and abs(float(r.hit_y[0, 0, 0]) - c) < 1e-12
    o = _device(oracle, lambda: oracle.dop853_event(BASE, 0.0, tmax, MU, 0, c, +1, 1, max_step=1e4))
    assert float(r.hit_t[0, 0]) == o["hit_t"][0] and np.array_equal(r.hit_y[0, 0].cpu().numpy(), o["hit_y"][0])


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fixed_rk4_event_case(gpu, oracle, case):
    """The same cases with fixed-step RK4 (integrators/rk.py:655-718, cubic
    Hermite refinement): GPU == oracle, and the expected outcome."""
    name, y0, tmax, c, direction, expect = case
    t = np.linspace(0.0, tmax, 21)
    ev = gpu.EventSpec(index=0, offset=c, direction=direction)
    _, ht, hy, nh = gpu.propagate_fixed_event(y0[None], t, MU, ev, order=4)
    hit, th, yh, _ = _device(oracle, lambda: oracle.fixed_rk_event(4, y0, t, MU, 0, c, direction))
    assert int(nh[0]) == int(hit) == int(expect), name
    if hit:
        assert float(ht[0]) == th and np.array_equal(hy[0].cpu().numpy(), yh)
        assert abs(yh[0] - c) <= 1e-12


def test_fixed_rk4_endpoint_zero_is_detected(gpu, oracle):
    t = np.linspace(0.0, 0.1, 11)
    states = gpu.propagate_fixed(BASE[None], t, MU, order=4)
    c = float(states[-1, 0, 0])
    ev = gpu.EventSpec(index=0, offset=c, direction=+1)
    _, ht, hy, nh = gpu.propagate_fixed_event(BASE[None], t, MU, ev, order=4)
    hit, th, yh, _ = _device(oracle, lambda: oracle.fixed_rk_event(4, BASE, t, MU, 0, c, +1))
    assert int(nh[0]) == 1 and hit
    assert float(ht[0]) == th and np.array_equal(hy[0].cpu().numpy(), yh)
    assert abs(th - 0.1) < 2e-12 and abs(yh[0] - c) <= 1e-12
