"""The device-resident halo correction (hg_correct_halo_graph: every orbit's
Newton iterations and line searches inside one CUDA graph) against the
native host driver over the same kernels, whose arithmetic it repeats except
for the quadratic term's powers (correctly rounded on the device, the C
library's pow on the host): the same statuses, iteration counts within one,
converged states and periods within the corrected-orbit tolerance 1e-10 --
and against the reference's own corrected orbits (<= 1e-10).  The graph is
cached on the handle: a second call with the same problem replays it and
gives the same bits; a call with another size rebuilds it."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def _guesses(n, seed):
    from hiten_gb300 import halo
    pt, az, zen = W.halo_guess_params(n, seed=seed)
    return np.concatenate([halo.third_order_guess(MU, 1, az[pt == 1], zen[pt == 1]),
                           halo.third_order_guess(MU, 2, az[pt == 2], zen[pt == 2])])


def test_graph_matches_native_driver(gpu):
    import torch
    from hiten_gb300 import _lib, corrector
    g = _guesses(256, 4)
    g[:3, 0] += np.array([0.3, -0.2, 0.05])   # hopeless guesses: no crossing or a failed line search
    nat = corrector.correct_halo_native(g, MU)
    ws = torch.empty(int(_lib.load().hg_correct_halo_graph_workspace_bytes(len(g))) + 256, dtype=torch.uint8,
                     device="cuda")
    gr = corrector.correct_halo_graph(g, MU, workspace=ws)
    assert np.array_equal(gr.status, nat.status)
    assert np.max(np.abs(gr.iterations - nat.iterations)) <= 1
    ok = nat.status == 0
    assert ok.sum() > 200
    assert np.max(np.abs(gr.x0[ok] - nat.x0[ok])) <= 1e-10
    assert np.max(np.abs(gr.period[ok] - nat.period[ok])) <= 1e-10
    assert np.all(gr.residual_norm[ok] < 1e-12)
    # the cached graph replays with the same bits
    again = corrector.correct_halo_graph(g, MU, workspace=ws)
    for f in ("x0", "period", "iterations", "status", "residual_norm"):
        assert np.array_equal(getattr(again, f), getattr(gr, f), equal_nan=True), f


def test_graph_matches_reference_golden(gpu):
    from hiten_gb300 import corrector
    h = np.load(os.path.join(GOLDEN, "halo.npz"))
    res = corrector.correct_halo_graph(h["guess"], float(h["mu"]))
    assert np.all(res.status == 0)
    assert np.max(np.abs(res.x0 - h["x0"])) <= 1e-10
    assert np.max(np.abs(res.period - h["period"])) <= 1e-10
    assert np.all(np.abs(res.iterations - h["iterations"]) <= 1)


def test_graph_sizes_and_options(gpu):
    """A different batch size rebuilds the graph; a tighter iteration budget
    ends orbits with the final residual check (HG_NEWTON_DIVERGED when not
    converged), as the host driver does."""
    from hiten_gb300 import corrector
    g = _guesses(40, 9)
    a = corrector.correct_halo_graph(g[:17], MU)
    b = corrector.correct_halo_native(g[:17], MU)
    assert np.array_equal(a.status, b.status)
    o = corrector.HaloCorrectionOptions(max_attempts=4)
    c = corrector.correct_halo_graph(g, MU, options=o)
    d = corrector.correct_halo_native(g, MU, options=o)
    # an orbit whose residual lands at the tolerance after the last allowed
    # step may end on either side of it (the last-bit difference)
    assert np.sum(c.status != d.status) <= 1
    assert np.all(c.iterations[c.status == 4] == 4)
    assert np.any(c.status == 4) and np.any(c.status == 0)
    ok = (d.status == 0) & (c.status == 0)
    assert np.max(np.abs(c.x0[ok] - d.x0[ok])) <= 1e-10


def test_graph_stm_layouts_give_the_same_bits(gpu):
    """The correction graph's STM leg on the three-warp, paired, 14- and
    7-lane layouts (the first two read the live count from device memory):
    the same corrected orbits bit for bit."""
    from hiten_gb300 import corrector
    from hiten_gb300 import propagate as P
    g = _guesses(64, 12)
    res = {}
    for lanes in (18, 12, 14, 7):
        with P.tuning(lanes_d42=lanes):
            res[lanes] = corrector.correct_halo_graph(g, MU)
    for lanes in (12, 14, 7):
        for f in ("x0", "period", "iterations", "status", "residual_norm"):
            assert np.array_equal(getattr(res[lanes], f), getattr(res[18], f), equal_nan=True), (lanes, f)
