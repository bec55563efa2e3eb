"""Host logic of the continuous-batching engine, without a device: the
admission pass (arrival order, per-kind merging, the HBM footprint budget, one
stream per open batch, an oversized request never starved), the split of a
merged batch's results back to its requests, the latency summary and the
seeded request stream."""
import numpy as np

from hiten_gb300 import serving as S
from hiten_gb300 import workloads as W


def _req(rid, kind, n, arrival=0.0):
    return S.Request(rid=rid, kind=kind, payload=np.zeros((n, 6)), arrival=arrival)


def test_admit_merges_per_kind_in_arrival_order():
    w = [_req(0, "manifold", 10), _req(1, "synodic", 5), _req(2, "manifold", 7), _req(3, "correct", 2)]
    adm, keep, used = S.admit(w, 0, 1 << 40, free_streams=2)
    # two streams free: manifold and synodic open batches, correct waits
    assert list(adm) == ["manifold", "synodic"]
    assert [r.rid for r in adm["manifold"]] == [0, 2]
    assert [r.rid for r in adm["synodic"]] == [1]
    assert [r.rid for r in keep] == [3]
    assert used == sum(r.footprint for r in w[:3])
    assert all(r.admitted is not None for r in w[:3]) and w[3].admitted is None


def test_admit_respects_the_footprint_budget():
    a, b, c = _req(0, "manifold", 100), _req(1, "manifold", 100), _req(2, "manifold", 1)
    budget = a.footprint + c.footprint
    adm, keep, used = S.admit([a, b, c], 0, budget, free_streams=4)
    # b does not fit after a; c (later, smaller) still does: arrival order, no head-of-line block
    assert [r.rid for r in adm["manifold"]] == [0, 2]
    assert [r.rid for r in keep] == [1]
    assert used == budget
    # memory in use from running batches: nothing new fits
    adm, keep, used2 = S.admit([b], budget, budget, free_streams=4)
    assert adm == {} and keep == [b] and used2 == budget


def test_admit_never_starves_an_oversized_request():
    big = _req(0, "synodic", 10_000)
    adm, keep, used = S.admit([big], 0, budget=1, free_streams=1)
    assert [r.rid for r in adm["synodic"]] == [0] and keep == [] and used == big.footprint
    # but not while anything else is running
    adm, keep, _ = S.admit([big], 5, budget=1, free_streams=1)
    assert adm == {} and keep == [big]


def test_split_and_summary():
    res = {"y_end": np.arange(12.0).reshape(6, 2), "status": np.arange(6)}
    parts = S._split("manifold", res, [1, 3, 2])
    assert [p["status"].tolist() for p in parts] == [[0], [1, 2, 3], [4, 5]]
    assert np.array_equal(parts[1]["y_end"], res["y_end"][1:4])
    st = S.ServingStats(n=4, wall_s=2.0, latencies=[0.1, 0.2, 0.3, 0.4], traj_steps=1000, batches=2)
    s = st.summary()
    assert s["requests"] == 4 and s["batches"] == 2
    assert abs(s["p50_ms"] - 250.0) < 1e-9 and abs(s["p99_ms"] - np.percentile([0.1, 0.2, 0.3, 0.4], 99) * 1e3) < 1e-9
    assert s["traj_steps_per_s"] == 500.0 and s["requests_per_s"] == 2.0


def test_poisson_stream_is_seeded_and_ordered():
    a = S.poisson_requests(200.0, 0.05, W.MU_EM, seed=3, size_scale=0.01)
    b = S.poisson_requests(200.0, 0.05, W.MU_EM, seed=3, size_scale=0.01)
    assert len(a) == len(b) > 0
    assert [r.arrival for r in a] == sorted(r.arrival for r in a)
    assert all(0.0 < r.arrival < 0.05 for r in a)
    for x, y in zip(a, b):
        assert (x.rid, x.kind, x.arrival) == (y.rid, y.kind, y.arrival)
        assert np.array_equal(x.payload, y.payload) and x.payload.shape[1] == 6
