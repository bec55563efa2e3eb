"""The GPU against an exact solution (mpmath Taylor method at 30 digits,
tests/golden/truth_mpmath.npz), beside the reference's arithmetic under both
glibc pow builds: the same crossings, the same accuracy (assertions of
tests/test_truth_mpmath_cpu.py), and bit for bit the oracle's DEVICE mode on
these states.  Run with -s for the table."""
import numpy as np
import pytest

from test_truth_mpmath_cpu import MU, _load, compare, device_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tag", ["section", "manifold"])
def test_gpu_as_close_to_truth_as_the_reference(gpu, oracle, tag):
    t, _ = _load()
    y0 = t[f"{tag}_y0"]
    if tag == "section":
        ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
        r = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, event=ev)
    else:
        from hiten_gb300 import manifold as M
        r = M.propagate_to_plane(y0, MU, tf=8.0, forward=-1)
    g = tuple(x.cpu().numpy() for x in (r.hit_t, r.hit_y, r.n_hits, r.y_end))
    compare(tag, g, "GPU")
    dev = device_run(oracle, tag, y0)
    assert np.array_equal(g[2], dev[2])
    for i in range(len(y0)):
        k = int(dev[2][i])
        assert np.array_equal(g[0][i, :k], dev[0][i, :k]) and np.array_equal(g[1][i, :k], dev[1][i, :k])
    assert np.array_equal(g[3], dev[3])
