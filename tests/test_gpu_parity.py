"""GPU kernels vs the CPU oracle (DEVICE mode: numba's integer powers,
correctly rounded fractional powers) -- bit-exact -- and vs the reference's
golden outputs within the stated tolerances (fixed step <= 1e-12 relative,
adaptive <= 1e-9 on non-chaotic spans)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import rowwise_rel, stm_state
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


@pytest.fixture(params=[(1, 32, 0, 7), (2, 32, 0, 14), (1, 128, 0, 14), (2, 64, 0, 7), (6, 32, 0, 14),
                        (6, 128, 0, 7), (1, 32, 1, 14), (6, 32, 1, 7), (2, 32, 0, 12)],
                ids=["lanes1-b32-d42x7", "lanes2-b32-d42x14", "lanes1-b128-d42x14", "lanes2-b64-d42x7",
                     "lanes6-b32-d42x14", "lanes6-b128-d42x7", "lanes1-spread-d42x14", "lanes6-spread-d42x7",
                     "lanes2-b32-d42pair"])
def shape(request, gpu):
    """Every launch shape must give the same bits (6-dim lanes, block, spread,
    42-dim lanes)."""
    lanes, block, spread, lanes42 = request.param
    with gpu.tuning(lanes_d6=lanes, block=block, spread=spread, lanes_d42=lanes42):
        yield request.param


@pytest.fixture(scope="module")
def dev_oracle(oracle):
    oracle.set_mode(oracle.MODE_DEVICE)
    yield oracle
    oracle.set_mode(oracle.MODE_PYTHON)


def _np(t):
    return t.detach().cpu().numpy()


# ------------------------------------------------------------------ fixed step
@pytest.mark.parametrize("order", [4, 6, 8])
@pytest.mark.parametrize("dim", [6, 42])
def test_fixed_matches_oracle_bitexact(gpu, shape, dev_oracle, order, dim):
    n_traj = 37  # crosses warp/group boundaries
    if dim == 42:
        y0 = W.stm_fixed_batch(1024, seed=0)[:n_traj]
    else:
        y0 = W.section_states(n_traj, seed=1)
    t = np.linspace(0.0, 1.0, 201)
    out = _np(gpu.propagate_fixed(y0, t, MU, order=order, out_every=10))
    ref, st = dev_oracle.fixed_rk_batch(order, y0, t, MU, out_every=10)
    assert st == 0
    assert np.array_equal(out, ref.transpose(1, 0, 2))


@pytest.mark.parametrize("lanes42", [7, 14, 12])
def test_fixed_rk8_stm_config_rows_bitexact(gpu, dev_oracle, lanes42):
    """The 42-dim RK8 workload (t in [0,3], 3000 steps, every 100th state) on 16 states."""
    y0 = W.stm_fixed_batch(1024, seed=0)[:16]
    t = np.linspace(0.0, 3.0, 3001)
    with gpu.tuning(lanes_d42=lanes42):
        out = _np(gpu.propagate_fixed(y0, t, MU, order=8, out_every=100))
    ref, st = dev_oracle.fixed_rk_batch(8, y0, t, MU, out_every=100)
    assert np.array_equal(out, ref.transpose(1, 0, 2))


def test_fixed_backward_flip_bitexact(gpu, dev_oracle):
    x = W.stm_fixed_batch(1024, seed=0)[200:205, 36:]
    y0 = np.array([stm_state(v) for v in x])
    t = np.linspace(0.0, 2.0, 401)
    out = _np(gpu.propagate_fixed(y0, t, MU, order=8, out_every=50, fwd=-1, flip=(36, 42)))
    ref, _ = dev_oracle.fixed_rk_batch(8, y0, t, MU, out_every=50, fwd=-1, flip=(36, 42))
    assert np.array_equal(out, ref.transpose(1, 0, 2))


def test_fixed_vs_reference_golden(gpu):
    """Against the reference's own RK8/RK4 outputs: <= 1e-12 relative (row-wise inf-norm)."""
    f = np.load(os.path.join(GOLDEN, "fixed.npz"))
    for i in range(6):
        y0 = f[f"rk8_42/{i}/y0"]
        out = _np(gpu.propagate_fixed(y0[None], np.linspace(0.0, 3.0, 3001), MU, order=8, out_every=100))[:, 0]
        assert rowwise_rel(out, f[f"rk8_42/{i}/states"]) <= 1e-12
    for i in range(3):
        y0 = f[f"rk8_6/{i}/y0"]
        out = _np(gpu.propagate_fixed(y0[None], np.linspace(0.0, 2.0, 801), MU, order=8, out_every=20))[:, 0]
        assert rowwise_rel(out, f[f"rk8_6/{i}/states"]) <= 1e-12


# ------------------------------------------------------------------ DOP853
def _cmp_event(res, ref, dim):
    n_hits = _np(res.n_hits)
    assert np.array_equal(n_hits, ref["n_hits"])
    assert np.array_equal(_np(res.n_accept), ref["n_accept"])
    assert np.array_equal(_np(res.n_reject), ref["n_reject"])
    assert np.array_equal(_np(res.t_end), ref["t_end"])
    assert np.array_equal(_np(res.y_end), ref["y_end"])
    ht, hy = _np(res.hit_t), _np(res.hit_y)
    for i, k in enumerate(n_hits):
        assert np.array_equal(ht[i, :k], ref["hit_t"][i, :k])
        assert np.array_equal(hy[i, :k], ref["hit_y"][i, :k])


@pytest.mark.parametrize("fwd", [1, -1])
def test_dop853_manifold_event_bitexact(gpu, shape, dev_oracle, fwd):
    rng = np.random.default_rng(7)
    y0 = W.HALO_L1_AZ02_X0 + rng.uniform(-1e-5, 1e-5, (45, 6))
    ev = gpu.EventSpec(index=0, offset=1 - MU, direction=0, max_hits=1)
    res = gpu.propagate_dop853(y0, 0.0, 8.0, MU, fwd=fwd, flip=(0, 6), event=ev)
    ref = dev_oracle.dop853_event_batch(y0, 0.0, 8.0, MU, 0, 1 - MU, 0, 1, max_step=1e4, fwd=fwd, flip=(0, 6))
    _cmp_event(res, ref, 6)


def test_dop853_section_multihit_bitexact(gpu, shape, dev_oracle):
    y0 = W.section_states(70, seed=9)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
    res = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, event=ev)
    ref = dev_oracle.dop853_event_batch(y0, 0.0, 20.0, MU, 1, 0.0, -1, 8, rtol=1e-11, atol=1e-11, max_step=1e4)
    _cmp_event(res, ref, 6)
    assert np.all(_np(res.status) == 0)


@pytest.mark.parametrize("fwd", [1, -1])
def test_planar_states_match_oracle(gpu, shape, dev_oracle, fwd):
    """Planar states (z = vz = 0, both signs of zero), DOP853 with an event
    and fixed RK8, both time directions: the oracle's values.  The quotients'
    Markstein correction returns +0 for a -0 numerator where IEEE division
    keeps -0, so the sign of an exactly zero component is not compared."""
    y0 = W.section_states(40, seed=12)
    y0[:, 2] = np.where(np.arange(40) % 2 == 0, 0.0, -0.0)
    y0[:, 5] = np.where(np.arange(40) % 3 == 0, -0.0, 0.0)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=3)
    res = gpu.propagate_dop853(y0, 0.0, 4.0, MU, rtol=1e-11, atol=1e-11, fwd=fwd, flip=(0, 6), event=ev)
    ref = dev_oracle.dop853_event_batch(y0, 0.0, 4.0, MU, 1, 0.0, -1, 3, rtol=1e-11, atol=1e-11, max_step=1e4,
                                        fwd=fwd, flip=(0, 6))
    _cmp_event(res, ref, 6)
    assert np.all(_np(res.y_end)[:, [2, 5]] == 0.0)
    t = np.linspace(0.0, 1.0, 101)
    out = _np(gpu.propagate_fixed(y0, t, MU, order=8, out_every=20, fwd=fwd, flip=(0, 6)))
    ref2, st = dev_oracle.fixed_rk_batch(8, y0, t, MU, out_every=20, fwd=fwd, flip=(0, 6))
    assert st == 0
    assert np.array_equal(out, ref2.transpose(1, 0, 2))


def test_dop853_singlehit_window_bitexact(gpu, shape, dev_oracle):
    rng = np.random.default_rng(3)
    y0 = W.HALO_L1_AZ02_X0 + np.c_[rng.uniform(-1e-3, 1e-3, 33), np.zeros(33), rng.uniform(-1e-3, 1e-3, 33),
                                   np.zeros(33), rng.uniform(-1e-3, 1e-3, 33), np.zeros(33)]
    ev = gpu.EventSpec(index=1, offset=0.0, direction=0, max_hits=1)
    res = gpu.propagate_dop853(y0, 0.0, np.pi - 1e-12, MU, max_step=np.inf, event=ev)
    ref = dev_oracle.dop853_event_batch(y0, 0.0, np.pi - 1e-12, MU, 1, 0.0, 0, 1)
    _cmp_event(res, ref, 6)


def test_dop853_stm_dense_bitexact(gpu, shape, dev_oracle):
    x0 = W.HALO_L1_AZ02_X0
    y0 = np.array([stm_state(x0 + d) for d in np.linspace(-1e-4, 1e-4, 9)[:, None] * np.eye(6)[0]])
    T = W.HALO_L1_AZ02_T
    for fwd in (1, -1):
        res = gpu.propagate_dop853(y0, 0.0, T, MU, fwd=fwd, flip=(36, 42), n_samples=40)
        out = _np(res.samples)
        for i in range(len(y0)):
            ref, na, nr, st = dev_oracle.dop853_dense(y0[i], np.linspace(0.0, T, 40), MU, fwd=fwd, flip=(36, 42))
            assert np.array_equal(out[:, i], ref)
            assert int(_np(res.n_accept)[i]) == na and int(_np(res.n_reject)[i]) == nr


def test_dop853_dense_last_matches_full(gpu):
    x0 = W.HALO_L1_AZ02_X0
    y0 = np.array([stm_state(x0)] * 5)
    tf = np.array([1.0, 1.5, 2.0, 2.5, 2.7])
    full = [gpu.propagate_dop853(y0[i:i + 1], 0.0, tf[i], MU, n_samples=500).samples[-1, 0] for i in range(5)]
    last = gpu.propagate_dop853(y0, 0.0, tf, MU, n_samples=500, sample_last_only=True).samples[0]
    for i in range(5):
        assert np.array_equal(_np(last[i]), _np(full[i]))


def test_dop853_vs_reference_golden(gpu):
    a = np.load(os.path.join(GOLDEN, "adaptive.npz"))
    for i in range(4):
        for kind, fwd in (("manifold_fwd", 1), ("manifold_bwd", -1)):
            y0 = a[f"{kind}/{i}/y0"]
            t = a[f"{kind}/{i}/t"]
            S = a[f"{kind}/{i}/states"]
            ev = gpu.EventSpec(index=0, offset=1 - MU, direction=0, max_hits=1)
            r = gpu.propagate_dop853(y0[None], 0.0, 8.0, MU, fwd=fwd, flip=(0, 6), event=ev)
            if int(_np(r.n_hits)[0]):
                assert abs(_np(r.hit_t)[0, 0] * fwd - t[-1]) <= 1e-9
                assert rowwise_rel(_np(r.hit_y)[0, :1], S[-1:]) <= 1e-9
            else:
                assert rowwise_rel(_np(r.y_end), S[-1:]) <= 1e-9


def test_step_control_edges_match_oracle(gpu, shape, dev_oracle):
    """The kernels' step control compares bit patterns (loop test, step
    clamps, endpoint, acceptance, PI factor guards, event signs); on the
    edges it must decide as the oracle's IEEE comparisons do: a start on the
    first primary (0/0 in the right-hand side) and a NaN start (a NaN step,
    every attempt rejected until max_steps), an active max_step clamp, an
    active min_step clamp, a span at negative times and an empty span."""
    y0 = W.section_states(14, seed=21)
    y0[3] = [-MU, 0.0, 0.0, 0.0, 0.3, 0.0]
    y0[7, 4] = np.nan
    ev = gpu.EventSpec(index=1, offset=0.0, direction=0, max_hits=2)
    cases = [(0.0, 1.5, 0.02, None), (0.0, 1.5, 1e4, 0.03), (-2.0, -0.5, 1e4, None), (0.7, 0.7, 1e4, None)]
    for t0, tmax, max_step, min_step in cases:
        res = gpu.propagate_dop853(y0, t0, tmax, MU, rtol=1e-11, atol=1e-11, max_step=max_step, min_step=min_step,
                                   max_steps=300, event=ev)
        ref = dev_oracle.dop853_event_batch(y0, t0, tmax, MU, 1, 0.0, 0, 2, rtol=1e-11, atol=1e-11,
                                            max_step=max_step, min_step=min_step, max_steps=300)
        case = (t0, tmax, max_step, min_step)
        assert np.array_equal(_np(res.status), ref["status"]), case
        assert np.array_equal(_np(res.n_accept), ref["n_accept"]), case
        assert np.array_equal(_np(res.n_reject), ref["n_reject"]), case
        assert np.array_equal(_np(res.t_end), ref["t_end"]), case
        assert np.array_equal(_np(res.y_end), ref["y_end"], equal_nan=True), case
        n_hits = _np(res.n_hits)
        assert np.array_equal(n_hits, ref["n_hits"]), case
        for i, k in enumerate(n_hits):
            assert np.array_equal(_np(res.hit_t)[i, :k], ref["hit_t"][i, :k]), case
            assert np.array_equal(_np(res.hit_y)[i, :k], ref["hit_y"][i, :k]), case
    # the start states that never leave t0 keep their values and count every attempt as a rejection
    assert int(_np(res.n_accept)[3]) == 0 and int(_np(res.n_accept)[7]) == 0


@pytest.mark.parametrize("lanes42", [7, 14, 12, 18])
def test_step_control_edges_42_match_oracle(gpu, dev_oracle, lanes42):
    """The same edges on the 42-dim (state + STM) DOP853 kernels: the 7- and
    14-lane groups, the paired and the three-warp layouts."""
    x = W.stm_fixed_batch(1024, seed=0)[:9, 36:]
    y0 = np.array([stm_state(v) for v in x])
    y0[2, 36:] = [-MU, 0.0, 0.0, 0.0, 0.3, 0.0]
    y0[5, 40] = np.nan
    for t0, tmax, max_step, min_step in [(0.0, 1.2, 0.02, None), (0.0, 1.2, 1e4, 0.03), (0.9, 0.9, 1e4, None)]:
        with gpu.tuning(lanes_d42=lanes42):
            res = gpu.propagate_dop853(y0, t0, tmax, MU, rtol=1e-11, atol=1e-11, max_step=max_step,
                                       min_step=min_step, max_steps=300, n_samples=2)
        out = _np(res.samples)
        for i in range(len(y0)):
            ref, na, nr, st = dev_oracle.dop853_dense(y0[i], np.array([t0, tmax]), MU, rtol=1e-11, atol=1e-11,
                                                      max_step=max_step, min_step=min_step, max_steps=300)
            case = (t0, tmax, max_step, min_step, i)
            assert np.array_equal(out[:, i], ref, equal_nan=True), case
            assert int(_np(res.n_accept)[i]) == na and int(_np(res.n_reject)[i]) == nr, case
            assert int(_np(res.status)[i]) == st, case


def test_max_steps_status(gpu):
    y0 = W.section_states(5, seed=2)
    res = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, max_steps=3)
    assert np.all(_np(res.status) == 1)
    assert np.all(_np(res.n_accept) + _np(res.n_reject) == 3)


@pytest.mark.parametrize("scheduled", [False, None], ids=["single-pass-refill", "default-plan"])
def test_lane_refill_matches_oracle(gpu, shape, dev_oracle, scheduled):
    """More trajectories than resident lanes: finished lanes take new ones
    (single pass), or the default plan for a batch this wide (scheduled)."""
    y0 = W.section_states(60000, seed=4)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=2)
    res = gpu.propagate_dop853(y0, 0.0, 0.6, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=scheduled)
    idx = np.random.default_rng(0).choice(60000, 300, replace=False)
    ref = dev_oracle.dop853_event_batch(y0[idx], 0.0, 0.6, MU, 1, 0.0, -1, 2, rtol=1e-11, atol=1e-11,
                                        max_step=1e4)
    assert np.array_equal(_np(res.y_end)[idx], ref["y_end"])
    assert np.array_equal(_np(res.n_accept)[idx], ref["n_accept"])
    assert np.array_equal(_np(res.n_hits)[idx], ref["n_hits"])


def test_inline_and_pooled_refinement_agree(gpu):
    """A record pool over the size limit makes the single-pass call refine
    crossings inline: the same bits as the pooled refinement."""
    y0 = W.section_states(300, seed=21)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=6)
    pooled = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=False)
    with gpu.tuning(refine_pool_mb=0):
        inline = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=False)
    for f in ("y_end", "n_hits", "n_accept", "status"):
        assert np.array_equal(_np(getattr(pooled, f)), _np(getattr(inline, f)))
    n = _np(pooled.n_hits)
    assert n.max() >= 2
    for i, k in enumerate(n):
        assert np.array_equal(_np(pooled.hit_t)[i, :k], _np(inline.hit_t)[i, :k])
        assert np.array_equal(_np(pooled.hit_y)[i, :k], _np(inline.hit_y)[i, :k])
