"""Segmented DOP853 (bounded steps per launch, live trajectories compacted
between launches, state carried in the outputs and the workspace) must give
the same bits as the single-pass kernel, and so as the oracle, for every
launch shape, segment length and number of segments per call (which forces
host-side resumes)."""
import numpy as np
import pytest

from helpers import stm_state
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM

SEGS = [(1, 1), (3, 2), (16, 8), (64, 1), (100000, 1)]


def _np(t):
    return t.detach().cpu().numpy()


def _same(a, b, with_event=False, samples=False):
    assert np.array_equal(_np(a.y_end), _np(b.y_end))
    assert np.array_equal(_np(a.t_end), _np(b.t_end))
    assert np.array_equal(_np(a.n_accept), _np(b.n_accept))
    assert np.array_equal(_np(a.n_reject), _np(b.n_reject))
    assert np.array_equal(_np(a.status), _np(b.status))
    if with_event:
        assert np.array_equal(_np(a.n_hits), _np(b.n_hits))
        nh = _np(a.n_hits)
        ha, hb = _np(a.hit_t), _np(b.hit_t)
        ya, yb = _np(a.hit_y), _np(b.hit_y)
        for i, k in enumerate(nh):
            assert np.array_equal(ha[i, :k], hb[i, :k])
            assert np.array_equal(ya[i, :k], yb[i, :k])
    if samples:
        assert np.array_equal(_np(a.samples), _np(b.samples))


@pytest.mark.parametrize("lanes", [1, 2, 6])
@pytest.mark.parametrize("seg_steps,max_segments", SEGS)
def test_segmented_manifold_event(gpu, lanes, seg_steps, max_segments):
    rng = np.random.default_rng(11)
    y0 = W.HALO_L1_AZ02_X0 + rng.uniform(-1e-5, 1e-5, (77, 6))
    ev = gpu.EventSpec(index=0, offset=1 - MU, direction=0, max_hits=1)
    with gpu.tuning(lanes_d6=lanes, block=32):
        ref = gpu.propagate_dop853(y0, 0.0, 8.0, MU, fwd=-1, flip=(0, 6), event=ev)
        seg = gpu.propagate_dop853(y0, 0.0, 8.0, MU, fwd=-1, flip=(0, 6), event=ev, segmented=True,
                                   seg_steps=seg_steps, max_segments=max_segments)
    _same(ref, seg, with_event=True)


@pytest.mark.parametrize("seg_steps,max_segments", SEGS[:3])
def test_segmented_multihit_ragged_tmax(gpu, seg_steps, max_segments):
    y0 = W.section_states(70, seed=9)
    tmax = np.linspace(2.0, 20.0, 70)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=5)
    with gpu.tuning(lanes_d6=2, block=64):
        ref = gpu.propagate_dop853(y0, 0.0, tmax, MU, rtol=1e-11, atol=1e-11, event=ev)
        seg = gpu.propagate_dop853(y0, 0.0, tmax, MU, rtol=1e-11, atol=1e-11, event=ev, segmented=True,
                                   seg_steps=seg_steps, max_segments=max_segments)
    _same(ref, seg, with_event=True)


@pytest.mark.parametrize("lanes42", [7, 14])
@pytest.mark.parametrize("last_only", [False, True])
@pytest.mark.parametrize("seg_steps,max_segments", [(1, 3), (5, 2), (40, 8)])
def test_segmented_stm_dense(gpu, dev_oracle, last_only, seg_steps, max_segments, lanes42):
    x0 = W.HALO_L1_AZ02_X0
    y0 = np.array([stm_state(x0 + d) for d in np.linspace(-1e-4, 1e-4, 9)[:, None] * np.eye(6)[0]])
    T = W.HALO_L1_AZ02_T
    with gpu.tuning(lanes_d42=lanes42):
        seg = gpu.propagate_dop853(y0, 0.0, T, MU, fwd=-1, flip=(36, 42), n_samples=40,
                                   sample_last_only=last_only, segmented=True, seg_steps=seg_steps,
                                   max_segments=max_segments)
    with gpu.tuning(lanes_d42=7):
        ref = gpu.propagate_dop853(y0, 0.0, T, MU, fwd=-1, flip=(36, 42), n_samples=40, sample_last_only=last_only)
    _same(ref, seg, samples=True)
    if not last_only:
        out = _np(seg.samples)
        r, na, nr, st = dev_oracle.dop853_dense(y0[4], np.linspace(0.0, T, 40), MU, fwd=-1, flip=(36, 42))
        assert np.array_equal(out[:, 4], r)


def test_segmented_max_steps_and_empty(gpu):
    y0 = W.section_states(40, seed=3)
    ref = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, max_steps=7)
    seg = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, max_steps=7, segmented=True,
                               seg_steps=2, max_segments=1)
    _same(ref, seg)
    assert np.all(_np(seg.status) == 1)
    empty = gpu.propagate_dop853(np.zeros((0, 6)), 0.0, 1.0, MU, segmented=True)
    assert empty.y_end.shape == (0, 6)


@pytest.fixture(scope="module")
def dev_oracle(oracle):
    oracle.set_mode(oracle.MODE_DEVICE)
    yield oracle
    oracle.set_mode(oracle.MODE_PYTHON)


@pytest.mark.parametrize("seg_steps", [1, 4, 16])
@pytest.mark.parametrize("lanes", [0, 1, 2, 6])
def test_scheduled_layout_switching(gpu, seg_steps, lanes):
    """A batch wide enough that the automatic policy passes through every
    layout (1 -> 2 -> 6 lanes) as trajectories finish; bits as single pass."""
    rng = np.random.default_rng(5)
    n = 12000 if seg_steps > 1 else 3500
    y0 = W.HALO_L1_AZ02_X0 + rng.uniform(-1e-4, 1e-4, (n, 6)) * np.logspace(-3, 0, n)[:, None]
    tmax = rng.uniform(1.0, 8.0, n)
    ev = gpu.EventSpec(index=0, offset=1 - MU, direction=0, max_hits=1)
    ref = gpu.propagate_dop853(y0, 0.0, tmax, MU, fwd=-1, flip=(0, 6), event=ev)
    with gpu.tuning(lanes_d6=lanes, seg_steps=seg_steps):
        sch = gpu.propagate_dop853(y0, 0.0, tmax, MU, fwd=-1, flip=(0, 6), event=ev, scheduled=True)
    _same(ref, sch, with_event=True)


def test_scheduled_stm_dense_and_max_steps(gpu):
    x0 = W.HALO_L1_AZ02_X0
    y0 = np.array([stm_state(x0 + d) for d in np.linspace(-1e-4, 1e-4, 9)[:, None] * np.eye(6)[0]])
    T = W.HALO_L1_AZ02_T
    ref = gpu.propagate_dop853(y0, 0.0, T, MU, fwd=-1, flip=(36, 42), n_samples=40)
    with gpu.tuning(seg_steps=3):
        sch = gpu.propagate_dop853(y0, 0.0, T, MU, fwd=-1, flip=(36, 42), n_samples=40, scheduled=True)
    _same(ref, sch, samples=True)
    y6 = W.section_states(40, seed=3)
    ref = gpu.propagate_dop853(y6, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, max_steps=7)
    with gpu.tuning(seg_steps=2):
        sch = gpu.propagate_dop853(y6, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, max_steps=7, scheduled=True)
    _same(ref, sch)
    assert np.all(_np(sch.status) == 1)


def test_single_call_partial_state(gpu):
    """finish=False: one segmented call, then return.  With every slot in one
    wave each trajectory has attempted at most seg_steps steps; the unfinished
    ones report HG_RUNNING and the finished ones equal a complete run."""
    from hiten_gb300 import _lib
    y0 = W.section_states(300, seed=4)
    tmax = np.where(np.arange(300) % 2 == 0, 0.02, 3.0)  # half finish within a few steps
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=2)
    full = gpu.propagate_dop853(y0, 0.0, tmax, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=False)
    part = gpu.propagate_dop853(y0, 0.0, tmax, MU, rtol=1e-11, atol=1e-11, event=ev, scheduled=False,
                                segmented=True, seg_steps=20, max_segments=1, finish=False)
    att = _np(part.n_accept) + _np(part.n_reject)
    st = _np(part.status)
    assert att.max() <= 20
    assert np.any(st == _lib.HG_RUNNING)
    done = st != _lib.HG_RUNNING
    assert np.any(done)
    assert np.array_equal(_np(part.y_end)[done], _np(full.y_end)[done])
    assert np.array_equal(_np(part.t_end)[done], _np(full.t_end)[done])
    assert np.array_equal(att[done], (_np(full.n_accept) + _np(full.n_reject))[done])
