"""Seeded synthetic inputs with the shapes and distributions of the
benchmark configurations (Earth-Moon CR3BP, mu = 0.012150585609624).

* ``stm_fixed_batch``   -- 42-dim STM states for fixed-step RK8 over t in [0, 3]
                           (3000 equal steps): x~U[0.82,0.86], y=0, z~U[0,0.08],
                           vx=0, vy~U[-0.05,0.05], vz~U[-0.2,0.2], Phi0 = I.
* ``manifold_seeds``    -- stable-manifold seeds of the L1 southern halo with
                           Az=0.2: phases x log-uniform displacements.
* ``section_states``    -- Jacobi-constant-matched states near L1/L2 for the
                           synodic section map (C~U[3.00,3.17]).
* ``halo_guess_params`` -- (libration point, Az, zenith) for batched correction.

No reference data is read; every array is generated from a numpy seed.
"""
import numpy as np

MU_EM = 0.012150585609624
# collinear libration points of the Earth-Moon system above (x coordinate)
X_L1 = 0.8369151257724081
X_L2 = 1.1556821654448837
# L1 southern halo, Az = 0.2, corrected by the reference's orbit.correct()
HALO_L1_AZ02_X0 = np.array([0.8234486451988118, 0.0, 0.032462917618892674, 0.0, 0.1421513197820747, 0.0])
HALO_L1_AZ02_T = 2.749936405299241


def identity_stm_state(x6):
    """Reference 42-vector layout: Phi (row-major) first, then the state."""
    x6 = np.atleast_2d(np.asarray(x6, dtype=np.float64))
    out = np.zeros((x6.shape[0], 42))
    out[:, :36] = np.eye(6).ravel()
    out[:, 36:] = x6
    return out


def stm_fixed_batch(n=1024, seed=0):
    """(n, 42) initial STM states for the fixed-step RK8 workload."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.82, 0.86, n)
    z = rng.uniform(0.0, 0.08, n)
    vy = rng.uniform(-0.05, 0.05, n)
    vz = rng.uniform(-0.2, 0.2, n)
    s = np.zeros((n, 6))
    s[:, 0] = x
    s[:, 2] = z
    s[:, 4] = vy
    s[:, 5] = vz
    return identity_stm_state(s)


def effective_potential(x, y, z, mu=MU_EM):
    r1 = np.sqrt((x + mu) ** 2 + y ** 2 + z ** 2)
    r2 = np.sqrt((x - 1 + mu) ** 2 + y ** 2 + z ** 2)
    return 0.5 * (x * x + y * y) + (1 - mu) / r1 + mu / r2


def section_states(n=65536, seed=0, mu=MU_EM):
    """(n, 6) states: L1 or L2 (50/50), position jitter U[-0.03,0.03]^3,
    vx = vz = 0, vy = +-sqrt(2*Omega - C) with C~U[3.00,3.17] (resampled
    until 2*Omega > C)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 6))
    filled = 0
    while filled < n:
        m = (n - filled) * 2
        which = rng.integers(0, 2, m)
        c = rng.uniform(3.00, 3.17, m)
        pos = rng.uniform(-0.03, 0.03, (m, 3))
        sign = np.where(rng.integers(0, 2, m) == 0, -1.0, 1.0)
        x = np.where(which == 0, X_L1, X_L2) + pos[:, 0]
        y = pos[:, 1]
        z = pos[:, 2]
        v2 = 2.0 * effective_potential(x, y, z, mu) - c
        ok = v2 > 0
        k = min(int(ok.sum()), n - filled)
        idx = np.nonzero(ok)[0][:k]
        out[filled:filled + k, 0] = x[idx]
        out[filled:filled + k, 1] = y[idx]
        out[filled:filled + k, 2] = z[idx]
        out[filled:filled + k, 4] = sign[idx] * np.sqrt(v2[idx])
        filled += k
    return out


def manifold_grid(n_phase=512, n_disp=32, seed=0, lo=1e-7, hi=1e-5):
    """Phases uniform in [0,1) and displacements log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    phases = np.arange(n_phase) / n_phase
    disp = np.exp(rng.uniform(np.log(lo), np.log(hi), n_disp))
    return phases, disp


def halo_guess_params(n=2048, seed=0):
    """(point index in {1,2}, Az~U[0.01,0.4], zenith in {'northern','southern'})."""
    rng = np.random.default_rng(seed)
    point = np.where(np.arange(n) < n // 2, 1, 2)
    az = rng.uniform(0.01, 0.4, n)
    zen = np.where(rng.integers(0, 2, n) == 0, "northern", "southern")
    return point, az, zen
