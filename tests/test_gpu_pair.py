"""Paired-warp 42-dim layout (a state warp with the shared Hessian and an STM
warp per five trajectories, shared-memory hand-off per stage): bit-identical
to the CPU oracle and to the single-warp layouts, for every order, ragged
batch sizes, both launch shapes (one block per SM while the blocks fit, plain
blocks beyond) and every flip range, including the STM components."""
import numpy as np
import pytest

from hiten_gb300 import _lib
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


@pytest.mark.parametrize("lanes", [12, 18])
@pytest.mark.parametrize("order", [4, 6, 8])
@pytest.mark.parametrize("n", [1, 7, 10, 23])
@pytest.mark.parametrize("fwd,flip", [(1, None), (-1, (36, 42)), (-1, (0, 42)), (-1, (30, 40))])
def test_pair_fixed_matches_oracle(gpu, dev_oracle, lanes, order, n, fwd, flip):
    y0 = W.stm_fixed_batch(64, seed=3)[:n]
    t = np.linspace(0.0, 0.8, 121)
    with gpu.tuning(lanes_d42=lanes):
        out, st = gpu.propagate_fixed(y0, t, MU, order=order, out_every=7, fwd=fwd, flip=flip, return_status=True)
    ref, rst = dev_oracle.fixed_rk_batch(order, y0, t, MU, out_every=7, fwd=fwd, flip=flip)
    assert rst == 0
    assert np.all(_np(st) == _lib.HG_OK)
    assert np.array_equal(_np(out), ref.transpose(1, 0, 2))


def test_pair_many_blocks_equals_single_warp_layouts(gpu, dev_oracle):
    # 2003 trajectories: 201 blocks of two pairs, more than one per SM, so
    # the launch runs without the one-block-per-SM reservation; the last
    # block is ragged (three trajectories in its first pair, none in its second)
    y0 = W.stm_fixed_batch(2003, seed=5)
    t = np.linspace(0.0, 0.5, 51)
    outs = {}
    for lanes in (12, 7, 14, 18):
        with gpu.tuning(lanes_d42=lanes):
            outs[lanes] = _np(gpu.propagate_fixed(y0, t, MU, order=8, out_every=5))
    assert np.array_equal(outs[12], outs[7])
    assert np.array_equal(outs[12], outs[14])
    assert np.array_equal(outs[12], outs[18])
    idx = np.array([0, 4, 5, 999, 2000, 2002])
    ref, rst = dev_oracle.fixed_rk_batch(8, y0[idx], t, MU, out_every=5)
    assert rst == 0
    assert np.array_equal(outs[12][:, idx], ref.transpose(1, 0, 2))


def test_pair_nonfinite_status_per_trajectory(gpu):
    # trajectory 6 starts on the first primary (r1 = 0): its state and STM turn
    # non-finite; its neighbours in the same pair are unaffected
    y0 = W.stm_fixed_batch(64, seed=7)[:12].copy()
    y0[6, 36:] = [-MU, 0.0, 0.0, 0.0, 0.0, 0.0]
    t = np.linspace(0.0, 0.2, 21)
    res = {}
    for lanes in (12, 7, 18):
        with gpu.tuning(lanes_d42=lanes):
            out, st = gpu.propagate_fixed(y0, t, MU, order=8, out_every=4, return_status=True)
        res[lanes] = (_np(out), _np(st))
    st = res[12][1]
    assert st[6] == _lib.HG_NONFINITE
    assert np.all(np.delete(st, 6) == _lib.HG_OK)
    ok = np.delete(np.arange(12), 6)
    for lanes in (7, 18):
        assert np.array_equal(res[12][1], res[lanes][1])
        assert np.array_equal(res[12][0][:, ok], res[lanes][0][:, ok])


# ------------------------------------------------------------------ DOP853 (42-dim, paired warps)
def _dop(gpu, lanes, y0, t0, tf, **kw):
    with gpu.tuning(lanes_d42=lanes):
        return gpu.propagate_dop853(y0, t0, tf, MU, flip=(36, 42) if kw.get("fwd", 1) == -1 else None, **kw)


@pytest.mark.parametrize("lanes", [12, 18])
@pytest.mark.parametrize("n", [1, 6, 11])
@pytest.mark.parametrize("fwd", [1, -1])
@pytest.mark.parametrize("m,last", [(2, False), (37, False), (500, True)])
def test_pair_dop853_dense_matches_oracle(gpu, dev_oracle, lanes, n, fwd, m, last):
    # 12: paired warps; 18: three warps (state + two half-column STM warps)
    y0 = W.stm_fixed_batch(64, seed=11)[:n]
    tf = np.linspace(0.4, 1.6, n)  # per-trajectory spans
    res = _dop(gpu, lanes, y0, 0.0, tf, rtol=1e-11, atol=1e-11, fwd=fwd, n_samples=m, sample_last_only=last)
    out = _np(res.samples)
    assert np.all(_np(res.status) == _lib.HG_OK)
    for i in range(n):
        ref, na, nr, st = dev_oracle.dop853_dense(y0[i], np.linspace(0.0, tf[i], m), MU, rtol=1e-11, atol=1e-11,
                                                  fwd=fwd, flip=(36, 42) if fwd == -1 else None)
        assert st == 0
        assert np.array_equal(out[:, i], ref[-1:] if last else ref)
        assert int(_np(res.n_accept)[i]) == na and int(_np(res.n_reject)[i]) == nr
    # the end state and time (not part of the dense output) as the single-warp kernel
    r7 = _dop(gpu, 7, y0, 0.0, tf, rtol=1e-11, atol=1e-11, fwd=fwd, n_samples=m, sample_last_only=last)
    assert np.array_equal(_np(res.y_end), _np(r7.y_end))
    assert np.array_equal(_np(res.t_end), _np(r7.t_end))


def test_pair_dop853_many_equals_single_warp_layouts(gpu):
    # 1003 trajectories (201 pairs, ragged last group), uneven spans and step counts
    y0 = W.stm_fixed_batch(1003, seed=12)
    tf = np.random.default_rng(3).uniform(0.2, 2.0, len(y0))
    fields = ("y_end", "t_end", "n_accept", "n_reject", "status", "samples")
    res = {lanes: _dop(gpu, lanes, y0, 0.0, tf, n_samples=25) for lanes in (12, 18, 7, 14)}
    for f in fields:
        assert np.array_equal(_np(getattr(res[12], f)), _np(getattr(res[7], f))), f
        assert np.array_equal(_np(getattr(res[12], f)), _np(getattr(res[14], f))), f
        assert np.array_equal(_np(getattr(res[18], f)), _np(getattr(res[7], f))), f


def test_pair_dop853_step_budget_status(gpu):
    # trajectory 4 starts on the first primary: its field is not finite, every
    # attempt is rejected and it runs out of steps like the single-warp kernel
    y0 = W.stm_fixed_batch(64, seed=13)[:9].copy()
    y0[4, 36:] = [-MU, 0.0, 0.0, 0.0, 0.0, 0.0]
    for max_steps in (7, 2000):
        r12 = _dop(gpu, 12, y0, 0.0, 1.0, max_steps=max_steps)
        r18 = _dop(gpu, 18, y0, 0.0, 1.0, max_steps=max_steps)
        r7 = _dop(gpu, 7, y0, 0.0, 1.0, max_steps=max_steps)
        for f in ("status", "n_accept", "n_reject", "t_end"):
            assert np.array_equal(_np(getattr(r12, f)), _np(getattr(r7, f))), f
            assert np.array_equal(_np(getattr(r18, f)), _np(getattr(r7, f))), f
        ok = _np(r12.status) == _lib.HG_OK
        assert np.array_equal(_np(r12.y_end)[ok], _np(r7.y_end)[ok])
        st = _np(r12.status)
        assert st[4] == _lib.HG_MAX_STEPS
        if max_steps == 7:
            assert np.all(st == _lib.HG_MAX_STEPS)
        else:
            assert np.all(np.delete(st, 4) == _lib.HG_OK)


def test_bounded_inter_warp_wait_runs_out_and_reports(gpu):
    """The hand-off waits of the paired layouts are bounded: a wait that
    nothing satisfies gives up after its limit (no hang, the context stays
    usable) and a satisfied one completes."""
    import ctypes as C
    import torch
    dev = torch.device("cuda", 0)
    out = torch.full((3,), -1, dtype=torch.int32, device=dev)
    H = _lib.handle(0)
    H.check(H.lib.hg_selftest_bounded_wait(H.ptr, 50, C.c_void_p(out.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    ran_out, completed, ns = (int(v) for v in out.cpu())
    assert ran_out == 1 and completed == 1
    assert 50_000_000 <= ns < 1_000_000_000
    # the context is still usable
    y0 = W.stm_fixed_batch(8, seed=1)
    out2 = _np(gpu.propagate_fixed(y0, np.linspace(0.0, 0.1, 11), MU, order=8))
    assert np.all(np.isfinite(out2))
