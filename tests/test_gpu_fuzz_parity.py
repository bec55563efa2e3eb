"""Seeded fuzz of the GPU propagation against the CPU oracle (DEVICE mode),
bit for bit: random tolerances, spans (scalar and per trajectory),
directions and flips, event component / direction / offset / hit count,
6-dim lane layout (1, 2, 6 lanes; 4-warp spread blocks) and execution plan
(single pass, segmented with resumes, scheduled)."""
import numpy as np
import pytest

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


@pytest.fixture(scope="module")
def dev_oracle(oracle):
    oracle.set_mode(oracle.MODE_DEVICE)
    yield oracle
    oracle.set_mode(oracle.MODE_PYTHON)


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("case", range(24))
def test_fuzz_dop853_events_bitexact(gpu, dev_oracle, case):
    rng = np.random.default_rng(1000 + case)
    n = int(rng.integers(1, 90))
    if rng.random() < 0.5:
        y0 = W.section_states(n, seed=case)
    else:
        y0 = W.HALO_L1_AZ02_X0 + rng.normal(0, 10 ** rng.uniform(-6, -2), (n, 6))
    tol = 10 ** rng.uniform(-13, -8)
    fwd = int(rng.choice([1, -1]))
    flip = (0, 6) if rng.random() < 0.7 else (3, 6)
    tmax = float(rng.uniform(0.5, 12.0))
    if rng.random() < 0.3:
        tmax = rng.uniform(0.5, 12.0, n)
    ev_index = int(rng.integers(0, 3))
    offset = float(np.median(y0[:, ev_index])) if rng.random() < 0.6 else 0.0
    ev_dir = int(rng.choice([-1, 0, 1]))
    max_hits = int(rng.integers(1, 6))
    lanes = int(rng.choice([1, 2, 6]))
    spread = int(rng.random() < 0.2)
    plan = rng.choice(["single", "segmented", "scheduled"])
    kw = {"scheduled": plan == "scheduled", "segmented": plan == "segmented"}
    if plan == "segmented":
        kw.update(seg_steps=int(rng.integers(1, 40)), max_segments=int(rng.integers(1, 4)))
    ev = gpu.EventSpec(index=ev_index, offset=offset, direction=ev_dir, max_hits=max_hits)
    with gpu.tuning(lanes_d6=lanes, spread=spread, seg_steps=int(rng.integers(2, 33))):
        res = gpu.propagate_dop853(y0, 0.0, tmax, MU, rtol=tol, atol=tol, fwd=fwd, flip=flip, event=ev, **kw)
    def oracle_run(y, t1):
        return dev_oracle.dop853_event_batch(y, 0.0, t1, MU, ev_index, offset, ev_dir, max_hits, rtol=tol, atol=tol,
                                             max_step=1e4, fwd=fwd, flip=flip)

    if np.ndim(tmax) == 0:
        ref = oracle_run(y0, tmax)
    else:  # per-trajectory end times: one oracle call per trajectory
        parts = [oracle_run(y0[i:i + 1], float(tmax[i])) for i in range(n)]
        ref = {k: np.concatenate([q[k] for q in parts]) for k in parts[0]}
    assert np.array_equal(_np(res.y_end), ref["y_end"])
    assert np.array_equal(_np(res.t_end), ref["t_end"])
    assert np.array_equal(_np(res.n_accept), ref["n_accept"])
    assert np.array_equal(_np(res.n_hits), ref["n_hits"])
    ht, hy = _np(res.hit_t), _np(res.hit_y)
    for i, k in enumerate(ref["n_hits"]):
        assert np.array_equal(ht[i, :k], ref["hit_t"][i, :k])
        assert np.array_equal(hy[i, :k], ref["hit_y"][i, :k])


@pytest.mark.parametrize("case", range(12))
def test_fuzz_fixed_rk_bitexact(gpu, dev_oracle, case):
    rng = np.random.default_rng(2000 + case)
    order = int(rng.choice([4, 6, 8]))
    dim = int(rng.choice([6, 42]))
    n = int(rng.integers(1, 40))
    y0 = W.stm_fixed_batch(64, seed=case)[:n] if dim == 42 else W.section_states(n, seed=case)
    steps = int(rng.integers(2, 400))
    t = np.linspace(0.0, float(rng.uniform(0.1, 3.0)), steps + 1)
    out_every = int(rng.integers(1, 50))
    fwd = int(rng.choice([1, -1]))
    flip = (36, 42) if dim == 42 else (0, 6)
    with gpu.tuning(lanes_d42=int(rng.choice([7, 14, 12])), block=int(rng.choice([32, 64, 128]))):
        out = _np(gpu.propagate_fixed(y0, t, MU, order=order, out_every=out_every, fwd=fwd, flip=flip))
    ref, st = dev_oracle.fixed_rk_batch(order, y0, t, MU, out_every=out_every, fwd=fwd, flip=flip)
    assert st == 0
    assert np.array_equal(out, ref.transpose(1, 0, 2))


@pytest.mark.parametrize("case", range(10))
def test_fuzz_dop853_dense_42_bitexact(gpu, dev_oracle, case):
    rng = np.random.default_rng(3000 + case)
    n = int(rng.integers(1, 6))
    y0 = W.stm_fixed_batch(64, seed=100 + case)[:n]
    tol = 10 ** rng.uniform(-12, -9)
    T = float(rng.uniform(0.3, 3.0))
    m = int(rng.integers(2, 60))
    fwd = int(rng.choice([1, -1]))
    with gpu.tuning(lanes_d42=int(rng.choice([7, 14, 12, 18]))):
        res = gpu.propagate_dop853(y0, 0.0, T, MU, rtol=tol, atol=tol, fwd=fwd, flip=(36, 42), n_samples=m)
    out = _np(res.samples)
    for i in range(n):
        ref, na, nr, st = dev_oracle.dop853_dense(y0[i], np.linspace(0.0, T, m), MU, rtol=tol, atol=tol, fwd=fwd,
                                                  flip=(36, 42))
        assert np.array_equal(out[:, i], ref)
        assert int(_np(res.n_accept)[i]) == na and int(_np(res.n_reject)[i]) == nr
