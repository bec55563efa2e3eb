"""Reference-shaped API on the GPU vs the reference's golden outputs and the
oracle (DEVICE mode, bit-exact)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import rowwise_rel
from hiten_gb300 import dynamics as D
from hiten_gb300 import integrators as I
from hiten_gb300 import workloads as W

pytestmark = pytest.mark.gpu
MU = W.MU_EM


def test_propagate_dynsys_fixed_and_compute_stm(gpu, oracle):
    f = np.load(os.path.join(GOLDEN, "fixed.npz"))
    y0 = f["rk8_42/0/y0"]
    sol = D.propagate_dynsys(D.CR3BPSystem(MU, 42), y0, 0.0, 3.0, steps=3001, method="fixed", order=8)
    assert rowwise_rel(sol.states[::100], f["rk8_42/0/states"]) <= 1e-12
    oracle.set_mode(oracle.MODE_DEVICE)
    ref, _ = oracle.fixed_rk(8, y0, np.linspace(0.0, 3.0, 3001), MU)
    assert np.array_equal(sol.states, ref)
    x0 = f["rk8_42_bwd/0/y0"]
    x, t, phiT, PHI = D.compute_stm(D.CR3BPSystem(MU, 42), x0, 2.0, steps=401, forward=-1, method="fixed")
    assert rowwise_rel(PHI[::50], f["rk8_42_bwd/0/states"]) <= 1e-12
    assert np.array_equal(t, -np.linspace(0.0, 2.0, 401)) and np.array_equal(phiT, PHI[-1, :36].reshape(6, 6))
    oracle.set_mode(oracle.MODE_PYTHON)


def test_adaptive_dense_and_stm_vs_golden(gpu, oracle):
    a = np.load(os.path.join(GOLDEN, "adaptive.npz"))
    for i in range(4):
        y0 = a[f"dense6/{i}/y0"]
        sol = D.propagate_dynsys(D.CR3BPSystem(MU, 6), y0, 0.0, 4.0, steps=101, rtol=1e-11, atol=1e-11)
        oracle.set_mode(oracle.MODE_DEVICE)
        ref, _, _, _ = oracle.dop853_dense(y0, np.linspace(0.0, 4.0, 101), MU, rtol=1e-11, atol=1e-11)
        assert np.array_equal(sol.states, ref)
        # The golden run is the reference without numba: its x**3 is libm pow,
        # numba's (the reference as shipped, and this kernel) is x*(x*x).  On an
        # unstable arc that last-bit difference grows, so the bar is the
        # reference's own run-mode spread: numba-mode vs pure-Python reference.
        oracle.set_mode(oracle.MODE_NUMBA)
        numba, _, _, _ = oracle.dop853_dense(y0, np.linspace(0.0, 4.0, 101), MU, rtol=1e-11, atol=1e-11)
        spread = rowwise_rel(numba, a[f"dense6/{i}/states"])
        assert rowwise_rel(sol.states, a[f"dense6/{i}/states"]) <= max(1e-9, 4.0 * spread)
        assert rowwise_rel(sol.states, numba) <= max(1e-9, 4.0 * spread)
    for i, fwd in ((0, 1), (1, -1)):
        x, t, phiT, PHI = D.compute_stm(D.CR3BPSystem(MU, 42), a[f"stm_halo/{i}/y0"], W.HALO_L1_AZ02_T, steps=40,
                                        forward=fwd)
        assert rowwise_rel(PHI, a[f"stm_halo/{i}/states"]) <= 1e-9
    oracle.set_mode(oracle.MODE_PYTHON)


def test_event_path_and_integrator_objects(gpu):
    a = np.load(os.path.join(GOLDEN, "adaptive.npz"))
    for i in range(4):
        for kind, fwd in (("manifold_fwd", 1), ("manifold_bwd", -1)):
            y0 = a[f"{kind}/{i}/y0"]
            sol = D.propagate_dynsys(D.CR3BPSystem(MU, 6), y0, 0.0, 8.0, forward=fwd, steps=2,
                                     flip_indices=slice(0, 6), event_fn=D.PlaneEvent(0, 1 - MU),
                                     event_cfg=D.EventConfig(direction=0, terminal=True))
            assert abs(sol.times[-1] - a[f"{kind}/{i}/t"][-1]) <= 1e-9
            assert rowwise_rel(sol.states[-1:], a[f"{kind}/{i}/states"][-1:]) <= 1e-9
    # integrator objects agree with the propagation functions
    y0 = W.section_states(3, seed=2)
    t = np.linspace(0.0, 2.0, 51)
    s1 = I.RungeKutta(853, rtol=1e-12, atol=1e-12, max_step=1e4).integrate(D.CR3BPSystem(MU, 6), y0, t)
    s2 = D.propagate_dynsys(D.CR3BPSystem(MU, 6), y0, 0.0, 2.0, steps=51)
    assert np.array_equal(s1.states, s2.states)
    s3 = I.RungeKutta(8).integrate(D.CR3BPSystem(MU, 6), y0, t)
    s4 = D.propagate_dynsys(D.CR3BPSystem(MU, 6), y0, 0.0, 2.0, steps=51, method="fixed")
    assert np.array_equal(s3.states, s4.states)


def test_manifold_compute_filters(gpu):
    from hiten_gb300 import manifold as M
    ys, dys, states, times, ok, att = M.compute(W.HALO_L1_AZ02_X0, W.HALO_L1_AZ02_T, MU, stable=True, step=0.25,
                                                dt=0.01, safe_r1=2e-6, safe_r2=2e-6)
    assert att == 4 and ok == len(states) and ok >= 1
    for S, t in zip(states, times):
        assert S.shape == (len(t), 6) and t[-1] == -0.75 * 2 * np.pi
        x, y, z, vx, vy, vz = S.T
        r1 = np.sqrt((x + MU) * (x + MU) + y * y + z * z)
        C = (x * x + y * y) + 2.0 * ((1 - MU) / r1 + MU / np.sqrt(((x - (1 - MU)) * (x - (1 - MU)) + y * y)
                                                                   + z * z)) - ((vx * vx + vy * vy) + vz * vz)
        assert np.max(np.abs(C - C[0]) / abs(C[0])) <= 1e-6
