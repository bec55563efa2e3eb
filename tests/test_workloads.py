"""Seeded synthetic inputs have the benchmark configurations' shapes and ranges."""
import numpy as np

from hiten_gb300 import workloads as W


def test_stm_fixed_batch():
    y = W.stm_fixed_batch(1024, seed=0)
    assert y.shape == (1024, 42)
    assert np.array_equal(y[:, :36], np.tile(np.eye(6).ravel(), (1024, 1)))
    x, z, vy, vz = y[:, 36], y[:, 38], y[:, 40], y[:, 41]
    assert x.min() >= 0.82 and x.max() <= 0.86 and z.min() >= 0 and z.max() <= 0.08
    assert np.all(y[:, 37] == 0) and np.all(y[:, 39] == 0)
    assert np.abs(vy).max() <= 0.05 and np.abs(vz).max() <= 0.2
    assert np.array_equal(y, W.stm_fixed_batch(1024, seed=0))


def test_section_states_jacobi():
    s = W.section_states(4096, seed=0)
    x, y, z, vy = s[:, 0], s[:, 1], s[:, 2], s[:, 4]
    C = 2 * W.effective_potential(x, y, z) - vy ** 2
    assert np.all((C >= 3.0 - 1e-9) & (C <= 3.17 + 1e-9))
    near1 = np.abs(x - W.X_L1) <= 0.03 + 1e-12
    near2 = np.abs(x - W.X_L2) <= 0.03 + 1e-12
    assert np.all(near1 | near2) and 0.4 < near1.mean() < 0.6
    assert np.all(s[:, 3] == 0) and np.all(s[:, 5] == 0)


def test_manifold_grid_and_halo_params():
    ph, d = W.manifold_grid(512, 32, seed=0)
    assert ph.shape == (512,) and ph.min() == 0.0 and ph.max() < 1.0
    assert d.shape == (32,) and d.min() >= 1e-7 and d.max() <= 1e-5
    p, az, zen = W.halo_guess_params(2048, seed=0)
    assert (p == 1).sum() == 1024 and az.min() >= 0.01 and az.max() <= 0.4
    assert set(zen) == {"northern", "southern"}
