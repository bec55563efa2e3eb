"""The kernels' arithmetic against an exact solution, beside the reference's.

tests/golden/truth_mpmath.npz holds the CR3BP solved by mpmath's Taylor
method at 30 digits (tests/golden/make_truth_mpmath.py) for 24 states of each
adaptive workload sample in libm_spread.npz: the synodic section (DOP853
1e-11 to t = 20, decreasing y = 0 crossings, terminal at the 8th) and the
stable manifold (t = -8, terminal x = 1 - mu).  The same file holds the
reference's arithmetic on those states under both glibc pow builds.  The
oracle's DEVICE mode is the kernels' arithmetic (the GPU equals it bit for
bit); here it must find the same crossings as the exact solution and be as
close to it as the reference is.  Run with -s for the table: the three are
equally far from the exact solution on every trajectory to about three
digits -- the integrator's own error at these tolerances (median 2e-7 on the
section arcs, 3e-8 on the manifold, O(1) on the arcs that pass close to a
primary) dwarfs what the last bit of a controller power moves."""
import os

import numpy as np
import pytest

from helpers import truth_distances
from hiten_gb300 import workloads as W

MU = W.MU_EM
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load():
    return np.load(os.path.join(GOLDEN, "truth_mpmath.npz")), np.load(os.path.join(GOLDEN, "libm_spread.npz"))


def test_truth_is_converged():
    t, s = _load()
    assert float(t["check"]) < 1e-15  # tolerance 1e-25 against 1e-21: the truth moved by less than this
    n = len(t["section_y0"])
    assert np.array_equal(t["section_y0"], s["section_y0"][:n])
    assert np.array_equal(t["manifold_y0"], s["manifold_y0"][:n])


def device_run(hgo, tag, y0):
    hgo.set_mode(hgo.MODE_DEVICE)
    try:
        if tag == "section":
            r = hgo.dop853_event_batch(y0, 0.0, 20.0, MU, 1, 0.0, -1, 8, rtol=1e-11, atol=1e-11, max_step=1e4)
        else:
            r = hgo.dop853_event_batch(y0, 0.0, 8.0, MU, 0, 1 - MU, 0, 1, max_step=1e4, fwd=-1, flip=(0, 6))
    finally:
        hgo.set_mode(hgo.MODE_PYTHON)
    return r["hit_t"], r["hit_y"], r["n_hits"], r["y_end"]


def compare(tag, mine, name):
    """Distances of `mine` and of the reference's two builds to the truth;
    asserts equal crossing counts and accuracy of the same size."""
    t, s = _load()
    n = len(t[f"{tag}_y0"])
    d_mine = truth_distances(tag, *mine, t)
    ref = {b: truth_distances(tag, s[f"{b}/{tag}_hit_t"][:n], s[f"{b}/{tag}_hit_y"][:n], s[f"{b}/{tag}_n_hits"][:n],
                              s[f"{b}/{tag}_y_end"][:n], t) for b in ("fma", "nofma")}
    print(f"\n{tag}: distance to the exact solution | {name} | reference (glibc FMA pow) | reference (non-FMA)")
    for i in range(n):
        print(f"  {i:3d} | {d_mine[i]:.2e} | {ref['fma'][i]:.2e} | {ref['nofma'][i]:.2e}")
    worst_ref = np.maximum(ref["fma"], ref["nofma"])
    print(f"  median | {np.median(d_mine):.2e} | {np.median(ref['fma']):.2e} | {np.median(ref['nofma']):.2e}")
    assert np.all(np.isfinite(d_mine)), "a crossing count differs from the exact solution's"
    assert np.all(np.isfinite(worst_ref))
    # the same accuracy: medians within 3x, the worst within 10x of the reference's worst
    assert np.median(d_mine) <= 3.0 * np.median(ref["fma"]) and np.median(ref["fma"]) <= 3.0 * np.median(d_mine)
    assert d_mine.max() <= 10.0 * worst_ref.max()
    return d_mine


@pytest.mark.parametrize("tag", ["section", "manifold"])
def test_kernel_arithmetic_as_close_to_truth_as_the_reference(oracle, tag):
    t, _ = _load()
    compare(tag, device_run(oracle, tag, t[f"{tag}_y0"]), "kernels' arithmetic")
