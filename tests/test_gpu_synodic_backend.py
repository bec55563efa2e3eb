"""The synodic detection backend drop-in (hiten_gb300.synodic.
GpuSynodicDetectionBackend, the methods and request / response fields of
poincare/synodic/backend.py:662-887) on ragged batches of sampled
trajectories: every trajectory's hits equal the oracle's (DEVICE mode) bit for
bit, in order, with the trajectory indices, caps and flattening of the
reference's `run`."""
import numpy as np
import pytest

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def _trajectories(gpu, lengths, seed):
    y0 = W.section_states(len(lengths), seed=seed)
    r = gpu.propagate_dop853(y0, 0.0, 10.0, MU, rtol=1e-11, atol=1e-11, n_samples=max(lengths))
    S = r.samples.cpu().numpy()  # (m, N, 6)
    t = np.linspace(0.0, 10.0, max(lengths))
    return [(t[:n].copy(), S[:n, i, :].copy()) for i, n in enumerate(lengths)]


@pytest.mark.parametrize("interp", ["linear", "cubic"])
@pytest.mark.parametrize("cap", [None, 3])
def test_backend_run_matches_oracle_on_ragged_batches(gpu, oracle, interp, cap):
    from hiten_gb300.synodic import GpuSynodicDetectionBackend, SynodicRequest
    rng = np.random.default_rng(5)
    lengths = list(rng.choice([150, 220, 301], size=36)) + [2, 1, 301, 150]
    trajs = _trajectories(gpu, lengths, seed=17)
    idx = list(range(100, 100 + len(trajs)))
    normal = np.eye(6)[1]
    req = SynodicRequest(trajectories=trajs, normal=normal, trajectory_indices=idx, offset=0.0,
                         plane_coords=("x", "vx"), interp_kind=interp, segment_refine=50, tol_on_surface=1e-6,
                         dedup_time_tol=1e-9, dedup_point_tol=1e-6, max_hits_per_traj=cap, newton_max_iter=10,
                         direction=-1)
    backend = GpuSynodicDetectionBackend(initial_cap=2)  # small first cap: the relaunch path runs
    res = backend.run(req)
    oracle.set_mode(oracle.MODE_DEVICE)
    try:
        flat_t = []
        for k, (t, s) in enumerate(trajs):
            hits = res.hits[k]
            if t.size < 2:
                assert hits == []
                continue
            rt, ry = oracle.section_detect(t, s, 1, 0.0, -1, (0, 3), segment_refine=50, cubic=(interp == "cubic"),
                                           newton_max_iter=10, max_hits=64 if cap is None else cap)
            assert len(hits) == len(rt), k
            for h, tt, yy in zip(hits, rt, ry):
                assert h.time == tt and np.array_equal(h.state, yy) and h.trajectory_index == idx[k]
                assert h.point2d[0] == yy[0] and h.point2d[1] == yy[3]
            flat_t.extend(rt)
    finally:
        oracle.set_mode(oracle.MODE_PYTHON)
    assert sum(len(h) for h in res.hits) > len(trajs)  # several crossings per trajectory on average
    assert np.array_equal(res.times, np.asarray(flat_t))
    assert res.points.shape == (len(flat_t), 2) and res.states.shape == (len(flat_t), 6)
    assert list(res.trajectory_indices) == [h.trajectory_index for hs in res.hits for h in hs]
    one = backend.detect_on_trajectory(*trajs[0], normal=normal, plane_coords=("x", "vx"), interp_kind=interp,
                                       segment_refine=50, tol_on_surface=1e-6, dedup_point_tol=1e-6,
                                       max_hits_per_traj=cap, newton_max_iter=10, direction=-1,
                                       trajectory_index=idx[0])
    assert [h.time for h in one] == [h.time for h in res.hits[0]]
