"""The benchmark workloads at their full sizes through the CUDA path.

The oracle checks a seeded sample of each batch bit for bit (the whole batch
would take the CPU minutes); the whole batch is held to properties that do not
depend on its size: permuting the states permutes every result bit for bit (no
lane, group or refill order leaks into a trajectory), every execution plan
gives the same bits, crossing times of a trajectory increase.  Empty batches
go through every entry point."""
import numpy as np
import pytest

from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM
FIELDS = ("y_end", "t_end", "n_accept", "n_reject", "n_hits", "status")


def _np(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def dev_oracle(oracle):
    oracle.set_mode(oracle.MODE_DEVICE)
    yield oracle
    oracle.set_mode(oracle.MODE_PYTHON)


def _hits(res):
    """(hit_t, hit_y) with the entries past each trajectory's n_hits zeroed."""
    k = _np(res.n_hits)
    ht, hy = _np(res.hit_t).copy(), _np(res.hit_y).copy()
    live = np.arange(ht.shape[1])[None, :] < k[:, None]
    ht[~live] = 0.0
    hy[~live] = 0.0
    return ht, hy


def _same(a, b, perm=None):
    """Results a and b are identical (b computed from the states permuted by perm)."""
    for f in FIELDS:
        x, y = _np(getattr(a, f)), _np(getattr(b, f))
        assert np.array_equal(x if perm is None else x[perm], y), f
    for x, y in zip(_hits(a), _hits(b)):
        assert np.array_equal(x if perm is None else x[perm], y)


def _vs_oracle(res, idx, ref):
    for f in ("y_end", "t_end", "n_accept", "n_reject", "n_hits"):
        assert np.array_equal(_np(getattr(res, f))[idx], ref[f]), f
    ht, hy = _hits(res)
    for j, i in enumerate(idx):
        k = int(ref["n_hits"][j])
        assert np.array_equal(ht[i, :k], ref["hit_t"][j, :k])
        assert np.array_equal(hy[i, :k], ref["hit_y"][j, :k])


def test_manifold_16384_full(gpu, dev_oracle):
    """Stable manifold of the L1 halo Az = 0.2: 512 phases x 32 displacements,
    DOP853 1e-12 to t = -8 with the terminal x = 1 - mu crossing."""
    from hiten_gb300 import manifold as M
    times, PHI = M.stm_grid(W.HALO_L1_AZ02_X0, W.HALO_L1_AZ02_T, MU, steps=2000, forward=-1)
    v = M.stable_eigvec(PHI[-1, :36].reshape(6, 6), stable=True)
    phases, disp = W.manifold_grid(512, 32, seed=0)
    s = M.seeds(times, PHI, W.HALO_L1_AZ02_T, phases, disp, v, direction=1)
    assert s.shape == (16384, 6)
    sched = M.propagate_to_plane(s, MU, tf=8.0, forward=-1, scheduled=True)
    single = M.propagate_to_plane(s, MU, tf=8.0, forward=-1, scheduled=False)
    _same(sched, single)
    perm = np.random.default_rng(0).permutation(len(s))
    _same(sched, M.propagate_to_plane(s[perm], MU, tf=8.0, forward=-1, scheduled=True), perm)
    idx = np.sort(np.random.default_rng(1).choice(len(s), 2048, replace=False))
    ref = dev_oracle.dop853_event_batch(s[idx], 0.0, 8.0, MU, 0, 1 - MU, 0, 1, max_step=1e4, fwd=-1, flip=(0, 6))
    _vs_oracle(sched, idx, ref)


def test_unstable_manifold_16384_full(gpu, dev_oracle):
    """The other leg of the manifold's t = +-8: the unstable manifold of the
    same halo (forward STM grid, the largest real eigenvalue's eigenvector),
    16384 seeds propagated forward to t = +8 with the terminal x = 1 - mu
    crossing; single pass and scheduled plans, permutation invariance, and a
    seeded 2048-seed sample against the oracle."""
    from hiten_gb300 import manifold as M
    times, PHI = M.stm_grid(W.HALO_L1_AZ02_X0, W.HALO_L1_AZ02_T, MU, steps=2000, forward=1)
    v = M.stable_eigvec(PHI[-1, :36].reshape(6, 6), stable=False)
    phases, disp = W.manifold_grid(512, 32, seed=0)
    s = M.seeds(times, PHI, W.HALO_L1_AZ02_T, phases, disp, v, direction=1)
    assert s.shape == (16384, 6)
    sched = M.propagate_to_plane(s, MU, tf=8.0, forward=1, scheduled=True)
    single = M.propagate_to_plane(s, MU, tf=8.0, forward=1, scheduled=False)
    _same(sched, single)
    perm = np.random.default_rng(6).permutation(len(s))
    _same(sched, M.propagate_to_plane(s[perm], MU, tf=8.0, forward=1, scheduled=True), perm)
    na = _np(sched.n_accept)
    assert na.min() < na.max()  # uneven lengths
    idx = np.sort(np.random.default_rng(7).choice(len(s), 2048, replace=False))
    ref = dev_oracle.dop853_event_batch(s[idx], 0.0, 8.0, MU, 0, 1 - MU, 0, 1, max_step=1e4, fwd=1, flip=(0, 6))
    _vs_oracle(sched, idx, ref)


def test_section_65536_full(gpu, dev_oracle):
    """65536 section states, DOP853 1e-11 to t = 20, up to 8 crossings of y = 0 (direction -1)."""
    y0 = W.section_states(65536, seed=0)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
    kw = dict(rtol=1e-11, atol=1e-11, event=ev)
    sched = gpu.propagate_dop853(y0, 0.0, 20.0, MU, scheduled=True, **kw)
    perm = np.random.default_rng(2).permutation(len(y0))
    _same(sched, gpu.propagate_dop853(y0[perm], 0.0, 20.0, MU, scheduled=False, **kw), perm)
    k = _np(sched.n_hits)
    ht, _ = _hits(sched)
    assert k.max() <= 8 and k.max() >= 2
    for j in range(1, 8):
        on = k > j
        assert np.all(ht[on, j] > ht[on, j - 1])
    idx = np.sort(np.random.default_rng(3).choice(len(y0), 1024, replace=False))
    ref = dev_oracle.dop853_event_batch(y0[idx], 0.0, 20.0, MU, 1, 0.0, -1, 8, rtol=1e-11, atol=1e-11,
                                        max_step=1e4)
    _vs_oracle(sched, idx, ref)


def test_fixed_rk8_stm_1024_full(gpu, dev_oracle):
    """RK8 with the 42-dim variational system, 1024 states x 3000 steps over [0, 3], every 100th state."""
    y0 = W.stm_fixed_batch(1024, seed=0)
    t = np.linspace(0.0, 3.0, 3001)
    out = _np(gpu.propagate_fixed(y0, t, MU, order=8, out_every=100))
    assert out.shape == (31, 1024, 42)
    perm = np.random.default_rng(4).permutation(len(y0))
    assert np.array_equal(out[:, perm], _np(gpu.propagate_fixed(y0[perm], t, MU, order=8, out_every=100)))
    idx = np.sort(np.random.default_rng(5).choice(len(y0), 64, replace=False))
    ref, st = dev_oracle.fixed_rk_batch(8, y0[idx], t, MU, out_every=100)
    assert st == 0
    assert np.array_equal(out[:, idx], ref.transpose(1, 0, 2))


def test_empty_batches(gpu):
    """N = 0 through every propagation entry point: empty results, no launch."""
    from hiten_gb300 import manifold as M
    t = np.linspace(0.0, 1.0, 11)
    assert _np(gpu.propagate_fixed(np.zeros((0, 6)), t, MU, order=8)).shape == (11, 0, 6)
    assert _np(gpu.propagate_fixed(np.zeros((0, 42)), t, MU, order=4, out_every=5)).shape == (3, 0, 42)
    ev = gpu.EventSpec(index=1, offset=0.0, direction=0, max_hits=3)
    for kw in (dict(), dict(scheduled=True), dict(scheduled=False, event=ev), dict(n_samples=5)):
        r = gpu.propagate_dop853(np.zeros((0, 6)), 0.0, 1.0, MU, **kw)
        assert _np(r.y_end).shape == (0, 6) and _np(r.n_accept).shape == (0,)
    r = gpu.propagate_dop853(np.zeros((0, 42)), 0.0, 1.0, MU, n_samples=4)
    assert _np(r.y_end).shape == (0, 42)
    r = M.propagate_to_plane(np.zeros((0, 6)), MU, tf=1.0)
    assert _np(r.n_hits).shape == (0,)


def test_empty_detection_filters_connections(gpu):
    """N = 0 through the sample-based section detection, the manifold filters
    and the connection search."""
    import torch
    from hiten_gb300 import connections as CN
    from hiten_gb300 import manifold as M
    from hiten_gb300 import synodic as S
    times = torch.linspace(0.0, 1.0, 9, dtype=torch.float64, device="cuda")
    samples = torch.zeros((9, 0, 6), dtype=torch.float64, device="cuda")
    ht, hy, nh = S.detect(times, samples, section_axis="y", plane_coords=("x", "vx"), direction=-1)
    assert tuple(nh.shape) == (0,)
    r1, r2, de = M.trajectory_filters(samples, MU)
    assert tuple(r1.shape) == (0,) and tuple(de.shape) == (0,)
    res, meta = CN.find_connections(np.zeros((0, 2)), np.ones((3, 2)), np.zeros((0, 6)), np.zeros((3, 6)))
    assert res == [] and meta == {}
