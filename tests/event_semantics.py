"""The reference's event-semantics cases (integrators/_tests/test_events.py)
restated on CR3BP motion, shared by the CPU and GPU tests.

The reference checks its event logic on one-dimensional flows (dy/dt = +-1,
constant, relaxation).  The kernels integrate the CR3BP only, so each case
is set on a plane event g = x - c crossed by a state far from both primaries
moving along x (|vx| = 1), over spans short enough that x is monotone: the
same situations -- a crossing in the requested direction, one filtered out
by the direction, a start exactly on the plane moving away, a start 1e-9
below it, a plane never reached, and a step that ends exactly on the plane
(the endpoint zero the reference counts, utils.py:13-39) -- with the
reference's expected outcomes.  Where the reference compares with an
analytic hit time, the hit is compared here with SciPy's DOP853 event root at
rtol = atol = 1e-14 and the hit state with the plane."""
import numpy as np

from hiten_gb300 import workloads as W

MU = W.MU_EM
BASE = np.array([0.5, 0.3, 0.0, 1.0, 0.0, 0.0])  # moving along +x, far from both primaries


def _state(x, vx):
    s = BASE.copy()
    s[0], s[3] = x, vx
    return s


# name, initial state, tmax, plane offset c (g = x - c), direction, expected hit
CASES = [
    ("positive_crossing", _state(0.5, 1.0), 0.2, 0.55, +1, True),
    ("negative_crossing", _state(0.5, -1.0), 0.2, 0.45, -1, True),
    ("strict_direction_no_hit", _state(0.5, 1.0), 0.1, 0.55, -1, False),
    ("start_on_plane_moving_away", _state(0.55, 1.0), 0.05, 0.55, +1, False),
    ("any_direction_crossing", _state(0.5, 1.0), 0.2, 0.55, 0, True),
    ("filtered_by_direction_no_hit", _state(0.5, -1.0), 0.2, 0.45, +1, False),
    ("never_reached_no_hit", _state(0.5, 1.0), 0.1, 0.0, 0, False),
    ("very_early_from_near_plane", _state(0.55 - 1e-9, 1.0), 0.1, 0.55, +1, True),
]


def f6(t, s):
    x, y, z, vx, vy, vz = s
    r1 = np.sqrt((x + MU) ** 2 + y * y + z * z)
    r2 = np.sqrt((x - 1 + MU) ** 2 + y * y + z * z)
    ax = 2 * vy + x - (1 - MU) * (x + MU) / r1 ** 3 - MU * (x - 1 + MU) / r2 ** 3
    ay = -2 * vx + y - (1 - MU) * y / r1 ** 3 - MU * y / r2 ** 3
    az = -(1 - MU) * z / r1 ** 3 - MU * z / r2 ** 3
    return np.array([vx, vy, vz, ax, ay, az])


def scipy_hit_time(y0, tmax, c, direction):
    """SciPy DOP853 at 1e-14 with its own event root finder: the first hit time or None."""
    from scipy.integrate import solve_ivp

    def g(t, s):
        return s[0] - c
    g.terminal = True
    g.direction = direction
    sol = solve_ivp(f6, (0.0, tmax), y0, method="DOP853", rtol=1e-14, atol=1e-14, events=g)
    return float(sol.t_events[0][0]) if len(sol.t_events[0]) else None


def check_case(name, y0, tmax, c, direction, expect_hit, n_hits, hit_t, hit_y, t_end, y_end):
    """The reference's assertions for the case (its tolerances: the hit time
    within 1e-10 of the exact one, the hit state on the plane; without a hit,
    the run ends at tmax)."""
    if not expect_hit:
        assert n_hits == 0, name
        assert abs(t_end - tmax) < 1e-15, name
        return
    assert n_hits == 1, name
    assert abs(hit_y[0] - c) < 1e-10, name
    ref = scipy_hit_time(y0, tmax, c, direction)
    assert ref is not None and abs(hit_t - ref) < 1e-10, (name, hit_t, ref)
    if name == "very_early_from_near_plane":
        assert abs(hit_t - 1e-9) < 1e-9, name
