"""Parity with the reference as shipped, beside how far the reference moves
between two builds of the same C library, and against a tight FP64 truth.

The reference computes its fractional powers (the DOP853 controller's
err**(-1/9), err_prev**(0.4/9), err**(-1/8)) with the platform's libm pow,
which is not correctly rounded; the kernels compute the same operations with
correctly rounded powers (bit for bit the oracle's DEVICE mode, asserted in
tests/test_gpu_full_size.py and tests/test_gpu_parity.py).  A one-ulp change
of one step size moves a trajectory along chaotic arcs far beyond 1e-9, and
the reference itself does so between glibc's two x86-64 pow builds (FMA and
non-FMA, chosen at load time by the CPU): tests/golden/libm_spread.npz holds
the reference's arithmetic (oracle NUMBA mode) under both, on seeded samples
of the section (t = 20) and manifold (t = -8) workloads.

A different step-size sequence moves an adaptive solution by about the
integrator's own global error, which for the reference's DOP853 (its error
norm carries an extra factor h, quirk A1) exceeds 1e-9 on a few percent of
these trajectories even over short arcs; so once one controller power differs
in its last bit, 1e-9 can fail without either result being less accurate.

Asserted here:
* on the section and manifold workloads, the GPU's distance from the
  reference (FMA build) is of the same size as the reference's own distance
  between its two glibc builds: at every threshold from 1e-12 to 1e-7 no
  more trajectories beyond it than 1.5 x the reference's own count plus 4,
  and a 99th-percentile distance within 5 x the reference's own;
* every trajectory the two glibc builds give bit-identically and the GPU
  reproduces bit for bit is counted (printed), and the table of distances to
  a SciPy DOP853 truth at rtol = atol = 1e-14 shows that the GPU and the
  reference are equally far from it (the reference's loosened error norm).
Run with -s for the tables."""
import os

import numpy as np
import pytest

from helpers import rowwise_rel
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM
HERE = os.path.dirname(os.path.abspath(__file__))


def _dist(a, b):
    """Per trajectory: the largest relative distance over crossing times,
    crossing states and end states (inf when the crossing counts differ)."""
    at, ay, an, ae = a
    bt, by, bn, be = b
    out = np.empty(len(an))
    for i in range(len(an)):
        if an[i] != bn[i]:
            out[i] = np.inf
            continue
        k = int(an[i])
        v = np.linalg.norm(ae[i] - be[i]) / np.linalg.norm(be[i])
        if k:
            v = max(v, np.max(np.linalg.norm(ay[i, :k] - by[i, :k], axis=1) / np.linalg.norm(by[i, :k], axis=1)),
                    np.max(np.abs(at[i, :k] - bt[i, :k]) / np.abs(bt[i, :k])))
        out[i] = v
    return out


def _res(r):
    return (r.hit_t.cpu().numpy(), r.hit_y.cpu().numpy(), r.n_hits.cpu().numpy(), r.y_end.cpu().numpy())


def _fix(d, build, tag):
    return tuple(d[f"{build}/{tag}_{k}"] for k in ("hit_t", "hit_y", "n_hits", "y_end"))


@pytest.mark.parametrize("tag", ["section", "manifold"])
def test_chaotic_workloads_within_the_references_own_spread(gpu, tag):
    d = np.load(os.path.join(HERE, "golden", "libm_spread.npz"))
    y0 = d[f"{tag}_y0"]
    if tag == "section":
        ev = gpu.EventSpec(index=1, offset=0.0, direction=-1, max_hits=8)
        r = gpu.propagate_dop853(y0, 0.0, 20.0, MU, rtol=1e-11, atol=1e-11, event=ev)
    else:
        from hiten_gb300 import manifold as M
        r = M.propagate_to_plane(y0, MU, tf=8.0, forward=-1)
    g = _res(r)
    fma, nofma = _fix(d, "fma", tag), _fix(d, "nofma", tag)
    d_gpu = _dist(g, fma)
    d_ref = _dist(nofma, fma)
    same_ref = d_ref == 0.0
    print(f"\n{tag}: {len(d_gpu)} trajectories")
    print(f"  reference FMA vs non-FMA glibc: beyond 1e-9 {np.sum(d_ref > 1e-9)}, max {d_ref.max():.2e}, "
          f"bit-identical {np.sum(same_ref)}")
    print(f"  GPU vs reference (FMA glibc):   beyond 1e-9 {np.sum(d_gpu > 1e-9)}, max {d_gpu.max():.2e}, "
          f"bit-identical {np.sum(d_gpu == 0.0)}")
    assert np.all(np.isfinite(d_gpu))
    for thr in (1e-12, 1e-11, 1e-10, 1e-9, 1e-8, 1e-7):
        n_gpu, n_ref = int(np.sum(d_gpu > thr)), int(np.sum(d_ref > thr))
        print(f"  beyond {thr:.0e}: GPU {n_gpu}, reference's own spread {n_ref}")
        assert n_gpu <= 1.5 * n_ref + 4
    assert np.percentile(d_gpu, 99) <= 5.0 * np.percentile(d_ref, 99)


def _truth(y0, t_end, fwd=1):
    from scipy.integrate import solve_ivp

    def f(t, s):
        x, y, z, vx, vy, vz = s
        r1 = np.sqrt((x + MU) ** 2 + y * y + z * z)
        r2 = np.sqrt((x - 1 + MU) ** 2 + y * y + z * z)
        ax = 2 * vy + x - (1 - MU) * (x + MU) / r1 ** 3 - MU * (x - 1 + MU) / r2 ** 3
        ay = -2 * vx + y - (1 - MU) * y / r1 ** 3 - MU * y / r2 ** 3
        az = -(1 - MU) * z / r1 ** 3 - MU * z / r2 ** 3
        return fwd * np.array([vx, vy, vz, ax, ay, az])

    return solve_ivp(f, (0.0, t_end), y0, method="DOP853", rtol=1e-14, atol=1e-14).y[:, -1]


@pytest.mark.parametrize("tf", [5.0, 20.0])
def test_distance_to_truth_table(gpu, oracle, tf):
    """Both the GPU and the reference against SciPy at 1e-14 (report; the
    assertion is that neither is systematically closer: the GPU's median
    distance to the truth is within 10x of the reference's)."""
    y0 = W.section_states(24, seed=3)
    g = gpu.propagate_dop853(y0, 0.0, tf, MU, rtol=1e-11, atol=1e-11).y_end.cpu().numpy()
    oracle.set_mode(oracle.MODE_NUMBA)
    ref = oracle.dop853_event_batch(y0, 0.0, tf, MU, 1, 0.0, 0, 0, rtol=1e-11, atol=1e-11, max_step=1e4)["y_end"]
    oracle.set_mode(oracle.MODE_PYTHON)
    eg, er, dd = [], [], []
    print(f"\nt = {tf}: trajectory | |GPU-REF| | |GPU-TRUTH| | |REF-TRUTH|")
    for i in range(len(y0)):
        tr = _truth(y0[i], tf)
        dd.append(rowwise_rel(g[i:i + 1], ref[i:i + 1]))
        eg.append(rowwise_rel(g[i:i + 1], tr[None]))
        er.append(rowwise_rel(ref[i:i + 1], tr[None]))
        print(f"  {i:3d} | {dd[-1]:.2e} | {eg[-1]:.2e} | {er[-1]:.2e}")
    assert np.median(eg) <= 10.0 * np.median(er) and np.median(er) <= 10.0 * np.median(eg)
