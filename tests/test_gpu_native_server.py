"""The native request server (hg_serve_*): requests sharing a problem run in
one pool of device-resident trajectory slots and each gets the bits of a
direct call on it alone (small and wide 6-dim requests, multi-hit events, a
42-dim request); a request entering while another runs, requests larger
than the pool, an arena too small for any pool; a queued request can be
cancelled; latency statistics are reported."""
import numpy as np
import pytest

from helpers import stm_state
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def _direct(gpu, y0, t0, tmax, kw):
    r = gpu.propagate_dop853(y0, t0, tmax, MU, **kw)
    out = {"y_end": r.y_end.cpu().numpy(), "t_end": r.t_end.cpu().numpy(), "n_accept": r.n_accept.cpu().numpy(),
           "status": r.status.cpu().numpy()}
    if r.n_hits is not None:
        out.update(n_hits=r.n_hits.cpu().numpy(), hit_t=r.hit_t.cpu().numpy(), hit_y=r.hit_y.cpu().numpy())
    return out


def test_native_server_matches_direct_calls(gpu):
    from hiten_gb300.serving import NativeServer
    man = dict(fwd=-1, flip=(0, 6), event=gpu.EventSpec(index=0, offset=1 - MU, direction=0, max_hits=1))
    sec = dict(rtol=1e-11, atol=1e-11, event=gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8))
    rng = np.random.default_rng(0)
    reqs = []
    for n in (37, 200, 5000):   # the 5000-state merge runs as host-scheduled segments
        reqs.append((W.HALO_L1_AZ02_X0 + rng.uniform(-1e-5, 1e-5, (n, 6)), 0.0, 8.0, man))
    for n, seed in ((100, 1), (64, 2)):
        reqs.append((W.section_states(n, seed=seed), 0.0, 20.0, sec))
    y42 = np.array([stm_state(W.HALO_L1_AZ02_X0 + d) for d in np.linspace(-1e-4, 1e-4, 5)[:, None] * np.eye(6)[0]])
    reqs.append((y42, 0.0, W.HALO_L1_AZ02_T, dict(fwd=-1, flip=(36, 42))))
    srv = NativeServer(max_concurrent=3)
    try:
        ids = [srv.submit(y, MU, t0, t1, **kw) for y, t0, t1, kw in reqs]
        for rid in ids:
            srv.wait(rid)
            assert srv.poll(rid) == 2
        got = [srv.fetch(rid) for rid in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert st["requests"] == len(reqs) and st["batches"] >= 1 and st["p99_ms"] >= st["p50_ms"] > 0
    for (y, t0, t1, kw), g in zip(reqs, got):
        d = _direct(gpu, y, t0, t1, dict(kw, scheduled=False))
        for k in ("y_end", "t_end", "n_accept", "status"):
            assert np.array_equal(g[k], d[k]), k
        if "n_hits" in d:
            assert np.array_equal(g["n_hits"], d["n_hits"])
            for i, h in enumerate(d["n_hits"]):
                assert np.array_equal(g["hit_t"][i, :h], d["hit_t"][i, :h])
                assert np.array_equal(g["hit_y"][i, :h], d["hit_y"][i, :h])


def test_native_server_cancels_queued_request(gpu):
    from hiten_gb300.serving import NativeServer
    srv = NativeServer(max_concurrent=1)
    try:
        ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
        big = srv.submit(W.section_states(20000, seed=5), MU, 0.0, 20.0, rtol=1e-11, atol=1e-11, event=ev)
        queued = srv.submit(W.section_states(10, seed=6), MU, 0.0, 3.0)   # another problem: waits for the slot
        assert srv.poll(queued) == 0
        assert srv.cancel(queued)
        srv.wait(big)
        assert srv.fetch(big)["y_end"].shape == (20000, 6)
        assert not srv.cancel(big)
    finally:
        srv.close()


def test_native_server_arena_limits(gpu):
    """A small device arena gives a small slot pool: a request many times its
    size streams through it (its trajectories enter as slots free up) with
    the bits of a direct call; an arena too small for even a 32-slot pool
    fails the request (state 3) and the server stays usable."""
    import time

    from hiten_gb300.serving import NativeServer
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
    kw = dict(rtol=1e-11, atol=1e-11, event=ev)
    y_big = W.section_states(12000, seed=11)
    srv = NativeServer(hbm_budget_bytes=24 << 20, max_concurrent=2, staging_bytes=8 << 20)
    try:
        big = srv.submit(y_big, MU, 0.0, 5.0, **kw)
        srv.wait(big)
        got = srv.fetch(big)
        st = srv.stats()
    finally:
        srv.close()
    assert st["batches"] > 10  # many segments: the pool holds a fraction of the request
    d = _direct(gpu, y_big, 0.0, 5.0, dict(kw, scheduled=False))
    for f in ("y_end", "t_end", "n_accept", "status", "n_hits"):
        assert np.array_equal(got[f], d[f]), f
    for i in np.nonzero(d["n_hits"])[0][:500]:
        h = d["n_hits"][i]
        assert np.array_equal(got["hit_t"][i, :h], d["hit_t"][i, :h])
        assert np.array_equal(got["hit_y"][i, :h], d["hit_y"][i, :h])
    tiny = NativeServer(hbm_budget_bytes=64 << 10, max_concurrent=1, staging_bytes=64 << 10)
    try:
        rid = tiny.submit(W.section_states(10, seed=3), MU, 0.0, 1.0, **kw)
        t0 = time.time()
        while tiny.poll(rid) < 2 and time.time() - t0 < 30:
            time.sleep(0.01)
        assert tiny.poll(rid) == 3
    finally:
        tiny.close()


def test_native_server_admits_while_running(gpu):
    """Continuous batching at the slot level: a request submitted while
    another of the same problem runs enters the running pool at the next
    segment boundary -- both are running at the same time -- and both get
    the bits of direct calls."""
    import time

    from hiten_gb300.serving import NativeServer
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
    kw = dict(rtol=1e-11, atol=1e-11, event=ev)
    ya, yb = W.section_states(8000, seed=21), W.section_states(1500, seed=22)
    srv = NativeServer(max_concurrent=2)
    overlap = False
    try:
        a = srv.submit(ya, MU, 0.0, 20.0, **kw)
        t0 = time.time()
        while srv.poll(a) == 0 and time.time() - t0 < 30:
            time.sleep(0.0005)
        b = srv.submit(yb, MU, 0.0, 20.0, **kw)
        while time.time() - t0 < 60:
            sa, sb = srv.poll(a), srv.poll(b)
            if sa == 1 and sb >= 1:
                overlap = True
                break
            if sa >= 2:
                break
            time.sleep(0.0005)
        srv.wait(a)
        srv.wait(b)
        ga, gb = srv.fetch(a), srv.fetch(b)
    finally:
        srv.close()
    assert overlap, "the second request did not enter while the first was running"
    for y, g in ((ya, ga), (yb, gb)):
        d = _direct(gpu, y, 0.0, 20.0, dict(kw, scheduled=False))
        for f in ("y_end", "t_end", "n_accept", "status", "n_hits"):
            assert np.array_equal(g[f], d[f]), f
