"""The connections host logic (hiten_gb300/connections.py) with the CPU
oracle of its two all-pairs searches reproduces the reference's own
_ConnectionsBackend.run results bit for bit (tests/golden/connections.npz:
four seeded section clouds, one with duplicate points and distance ties,
one with a single unstable-side point)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLDEN, "connections.npz"))


def _check(res, meta, gold, c):
    n = len(gold[f"{c}/dv"])
    assert len(res) == n
    assert meta.get("pairs_considered", 0) == int(gold[f"{c}/pairs_considered"])
    if n == 0:
        return
    assert np.array_equal(np.array([r.kind == "ballistic" for r in res]), gold[f"{c}/kind"])
    assert np.array_equal(np.array([r.delta_v for r in res]), gold[f"{c}/dv"])
    assert np.array_equal(np.array([r.point2d for r in res]), gold[f"{c}/point"])
    assert np.array_equal(np.array([r.state_u for r in res]), gold[f"{c}/state_u"])
    assert np.array_equal(np.array([r.state_s for r in res]), gold[f"{c}/state_s"])
    idx = np.array([[r.index_u, r.index_s, r.trajectory_index_u, r.trajectory_index_s] for r in res])
    assert np.array_equal(idx, gold[f"{c}/index"])


@pytest.mark.parametrize("c", [0, 1, 2, 3])
def test_connections_reproduce_reference(gold, c):
    from oracle.connect import OracleSectionMatcher
    from hiten_gb300.connections import find_connections
    eps, dvt, bt = gold[f"{c}/params"]
    res, meta = find_connections(gold[f"{c}/pu"], gold[f"{c}/ps"], gold[f"{c}/Xu"], gold[f"{c}/Xs"],
                                 gold[f"{c}/tu"], gold[f"{c}/ts"], eps=eps, dv_tol=dvt, bal_tol=bt,
                                 matcher=OracleSectionMatcher())
    _check(res, meta, gold, c)


def test_velocity_jumps_equal_per_row_norm():
    """The batched |dv| is the per-row np.linalg.norm bit for bit (the
    reference takes the norm of each pair's 3-vector)."""
    from hiten_gb300.connections import velocity_jumps
    rng = np.random.default_rng(3)
    for scale in (1e-9, 1e-3, 1.0, 1e7):
        v = rng.normal(0, scale, (20000, 3)) * np.exp(rng.normal(0, 2, (20000, 1)))
        v[:5] = [[0, 0, 0], [1e-300, 0, 0], [3, 4, 0], [np.inf, 0, 1], [-0.0, 2, -2]]
        ref = np.array([np.linalg.norm(r) for r in v])
        assert np.array_equal(velocity_jumps(v), ref)


def test_batch_closest_points_equal_scalar_form():
    """The vectorised closest points of two 2-D segments equal the
    reference-shaped scalar function bit for bit, degenerate segments included
    (zero length, parallel, collinear, touching, crossing)."""
    from hiten_gb300.connections import closest_points_on_segments_2d, closest_points_on_segments_2d_batch
    rng = np.random.default_rng(8)
    n = 4000
    a0, a1, b0, b1 = (rng.uniform(-1, 1, (n, 2)) for _ in range(4))
    k = n // 8
    a1[:k] = a0[:k]                                   # zero-length first segment
    b1[k:2 * k] = b0[k:2 * k]                         # zero-length second segment
    d = rng.uniform(-1, 1, (k, 2))
    b0[2 * k:3 * k] = a0[2 * k:3 * k] + [0.0, 0.5]    # parallel, offset
    b1[2 * k:3 * k] = b0[2 * k:3 * k] + (a1[2 * k:3 * k] - a0[2 * k:3 * k])
    b0[3 * k:4 * k] = a0[3 * k:4 * k] + 2.0 * (a1[3 * k:4 * k] - a0[3 * k:4 * k])  # collinear, disjoint
    b1[3 * k:4 * k] = a0[3 * k:4 * k] + 3.0 * (a1[3 * k:4 * k] - a0[3 * k:4 * k])
    b0[4 * k:5 * k] = a1[4 * k:5 * k]                 # touching end to start
    b1[4 * k:5 * k] = a1[4 * k:5 * k] + d
    batch = closest_points_on_segments_2d_batch(a0[:, 0], a0[:, 1], a1[:, 0], a1[:, 1], b0[:, 0], b0[:, 1],
                                                 b1[:, 0], b1[:, 1])
    for i in range(n):
        ref = closest_points_on_segments_2d(a0[i, 0], a0[i, 1], a1[i, 0], a1[i, 1], b0[i, 0], b0[i, 1], b1[i, 0],
                                            b1[i, 1])
        got = tuple(float(x[i]) for x in batch)
        assert np.array_equal(np.array(got), np.array(ref), equal_nan=True), (i, got, ref)
