"""A captured DOP853 batch (CUDA graph of the segmented driver over static
buffers) replays new inputs with the same bits as direct calls, including
trajectories that outlive the captured segments (finished by resumed calls)."""
import numpy as np
import pytest

from helpers import stm_state
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def _np(t):
    return t.detach().cpu().numpy()


def _same(a, b, event=False, samples=False):
    for f in ("y_end", "t_end", "n_accept", "n_reject", "status"):
        assert np.array_equal(_np(getattr(a, f)), _np(getattr(b, f))), f
    if event:
        assert np.array_equal(_np(a.n_hits), _np(b.n_hits))
        for i, k in enumerate(_np(a.n_hits)):
            assert np.array_equal(_np(a.hit_t)[i, :k], _np(b.hit_t)[i, :k])
            assert np.array_equal(_np(a.hit_y)[i, :k], _np(b.hit_y)[i, :k])
    if samples:
        assert np.array_equal(_np(a.samples), _np(b.samples))


@pytest.mark.parametrize("segments,seg_steps", [(2, 16), (8, 32)])
def test_captured_manifold_batch_replays(gpu, segments, seg_steps):
    from hiten_gb300.graphs import CapturedDop853
    ev = gpu.EventSpec(index=0, offset=1 - MU, direction=0, max_hits=1)
    cap = CapturedDop853(77, 6, 0.0, 8.0, MU, fwd=-1, flip=(0, 6), event=ev, segments=segments, seg_steps=seg_steps)
    for seed in (11, 12):
        rng = np.random.default_rng(seed)
        y0 = W.HALO_L1_AZ02_X0 + rng.uniform(-1e-5, 1e-5, (77, 6))
        ref = gpu.propagate_dop853(y0, 0.0, 8.0, MU, fwd=-1, flip=(0, 6), event=ev)
        _same(cap.run(y0), ref, event=True)


def test_captured_stm_dense_last(gpu):
    from hiten_gb300.graphs import CapturedDop853
    x0 = W.HALO_L1_AZ02_X0
    T = W.HALO_L1_AZ02_T
    cap = CapturedDop853(9, 42, 0.0, T, MU, fwd=-1, flip=(36, 42), n_samples=500, sample_last_only=True,
                         segments=3, seg_steps=8)
    for scale in (1e-4, 3e-4):
        y0 = np.array([stm_state(x0 + d) for d in np.linspace(-scale, scale, 9)[:, None] * np.eye(6)[0]])
        ref = gpu.propagate_dop853(y0, 0.0, T, MU, fwd=-1, flip=(36, 42), n_samples=500, sample_last_only=True)
        _same(cap.run(y0), ref, samples=True)


def test_captured_shape_is_fixed(gpu):
    from hiten_gb300.graphs import CapturedDop853
    cap = CapturedDop853(4, 6, 0.0, 1.0, MU)
    with pytest.raises(ValueError):
        cap.run(np.zeros((5, 6)))
