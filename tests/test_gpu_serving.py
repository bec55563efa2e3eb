"""Continuous batching: every request's result is the same, bit for bit,
whether it is solved alone or merged with concurrent requests of other
sizes and kinds, and under a small HBM budget that forces admission to wait."""
import numpy as np
import pytest

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("budget", [8 << 30, 256 << 10])
def test_served_results_equal_alone(gpu, budget):
    from hiten_gb300 import serving
    mu = W.MU_EM
    reqs = serving.poisson_requests(200.0, 0.25, mu, seed=5, size_scale=0.02)
    assert len({r.kind for r in reqs}) == 3
    eng = serving.ServingEngine(mu, hbm_budget_bytes=budget, max_concurrent=4)
    stats = eng.serve(reqs)
    eng.close()
    assert stats.n == len(reqs)
    for r in reqs:
        alone = serving._solve(r.kind, r.payload, mu, None)
        _same(r.result, alone)
        assert r.done >= r.admitted


def test_slot_level_served_results_equal_alone(gpu):
    """Lane-level continuous batching (manifold and synodic requests in the
    native server's slot pools, entering as slots free up): every result is
    bit-identical to the request solved alone."""
    from hiten_gb300 import serving
    mu = W.MU_EM
    reqs = serving.poisson_requests(200.0, 0.25, mu, seed=7, size_scale=0.05)
    assert len({r.kind for r in reqs}) == 3
    eng = serving.ServingEngine(mu, max_concurrent=4, slots=True, pool_slots=4096)
    stats = eng.serve(reqs)
    eng.close()
    assert stats.n == len(reqs)
    for r in reqs:
        alone = serving._solve(r.kind, r.payload, mu, None)
        _same(r.result, alone)
        assert r.done >= r.admitted


def test_sequential_plain_form(gpu):
    from hiten_gb300 import serving
    mu = W.MU_EM
    reqs = serving.poisson_requests(100.0, 0.1, mu, seed=6, size_scale=0.02)
    st = serving.run_sequential(reqs, mu)
    assert st.n == len(reqs) and st.wall_s > 0
    s = st.summary()
    assert s["p99_ms"] >= s["p50_ms"] >= 0
