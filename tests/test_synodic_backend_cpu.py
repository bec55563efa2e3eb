"""Argument rules of the synodic detection backend drop-in (no device needed:
they are checked before any launch)."""
import numpy as np
import pytest

from hiten_gb300.synodic import GpuSynodicDetectionBackend, SynodicRequest


def _req(**kw):
    t = np.linspace(0.0, 1.0, 5)
    s = np.zeros((5, 6))
    base = dict(trajectories=[(t, s)], normal=np.eye(6)[1], trajectory_indices=[0], segment_refine=50)
    base.update(kw)
    return SynodicRequest(**base)


@pytest.mark.parametrize("normal", [np.array([0, 2.0, 0, 0, 0, 0]), np.array([1.0, 1.0, 0, 0, 0, 0]),
                                    np.array([0, -1.0, 0, 0, 0, 0]), np.ones(3)])
def test_non_axis_normals_are_refused(normal):
    with pytest.raises(ValueError, match="axis-aligned"):
        GpuSynodicDetectionBackend().run(_req(normal=normal))


def test_unrefined_path_is_refused():
    with pytest.raises(ValueError, match="segment_refine"):
        GpuSynodicDetectionBackend().run(_req(segment_refine=0))


def test_shapes_and_indices_are_checked():
    with pytest.raises(ValueError, match="interp_kind"):
        GpuSynodicDetectionBackend().run(_req(interp_kind="quintic"))
    with pytest.raises(ValueError, match="index"):
        GpuSynodicDetectionBackend().run(_req(trajectory_indices=[0, 1]))
    t = np.linspace(0.0, 1.0, 5)
    with pytest.raises(ValueError, match="trajectory is"):
        GpuSynodicDetectionBackend().run(_req(trajectories=[(t, np.zeros((4, 6)))]))


def test_empty_request_returns_the_empty_response():
    r = GpuSynodicDetectionBackend().run(_req(trajectories=[], trajectory_indices=[]))
    assert r.hits == [] and r.times is None and r.points.shape == (0, 2) and r.states.shape == (0, 6)
    assert r.trajectory_indices.shape == (0,)
