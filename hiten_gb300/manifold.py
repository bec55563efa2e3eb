"""Manifold seeding and batched manifold propagation on the GPU.

Follows algorithms/types/services/manifold.py: the STM grid of the periodic
orbit (_compute_stm with steps=2000 and the manifold's direction, :215-245),
the NN-th real stable or unstable eigenvector of the monodromy as the
manifold service chooses it (eigen-decomposition of the discrete system
with delta = 1e-6, pivot-normalised complex eigenvectors, :347-367 and
algorithms/linalg/backend.py:196-260), seeds
x0W = x(t_k) + (d / |(dir * Phi(t_k) v)[0:3]|) * Re(dir * Phi(t_k) v) at the
grid time nearest to fraction * T (:470-573), then DOP853 propagation of all
seeds at once with the flip of components 0:6 for backward time (:396-409).
"""
import numpy as np
import torch

from . import propagate as P
from . import stability
from .workloads import identity_stm_state


def stm_grid(x0, period, mu, steps=2000, forward=1, rtol=1e-12, atol=1e-12, device=None):
    """(times, PHI) of _compute_stm: PHI (steps, 42) at linspace(0, T, steps), times signed."""
    y0 = identity_stm_state(np.asarray(x0, dtype=np.float64))
    r = P.propagate_dop853(y0, 0.0, float(period), mu, rtol=rtol, atol=atol, max_step=1e4, fwd=forward,
                           flip=(36, 42), n_samples=int(steps), device=device)
    PHI = r.samples[:, 0, :].cpu().numpy()
    times = forward * np.linspace(0.0, float(period), int(steps))
    return times, PHI


def stable_eigvec(phi_T, stable=True, NN=1, delta=1e-6):
    """The NN-th real stable (or unstable) eigenvector of the monodromy, as
    the manifold service picks it: complex128, pivot-normalised (first entry
    of modulus >= 1e-14 equal to 1, real vectors with a positive pivot),
    among the eigenvalues with |lambda| < 1 - delta (> 1 + delta) that
    np.isreal accepts, in numpy eig's order (services/manifold.py:347-367)."""
    sn, un, _, Ws, Wu, _ = stability.eigenvalue_decomposition(np.asarray(phi_T), delta)
    _, vecs = stability.real_eigenvectors(Ws, sn) if stable else stability.real_eigenvectors(Wu, un)
    col = NN - 1
    if col < 0 or vecs.shape[1] <= col:
        kind = "stable" if stable else "unstable"
        raise ValueError(f"Requested {kind} eigenvector {NN} not available. "
                         f"Only {vecs.shape[1]} real {kind} eigenvectors found.")
    return vecs[:, col]


def seeds(times, PHI, period, fractions, displacements, eigvec, direction=1):
    """Seeds for every (fraction, displacement) pair (fraction-major), in the
    operation order of _compute_manifold_section (services/manifold.py:470-537)."""
    tt = np.abs(times)
    xx = PHI[:, 36:42]
    out = np.empty((len(fractions) * len(displacements), 6))
    n = 0
    for f in fractions:
        k = int(np.argmin(np.abs(f * period - tt)))
        phi = PHI[k, :36].reshape((6, 6))
        man = direction * (phi @ eigvec)
        mag = np.linalg.norm(man[0:3])
        if mag < 1e-14:
            mag = 1.0
        for disp in displacements:
            d = disp / mag
            x = (xx[k, :].copy() + d * man.real).flatten()
            if abs(x[2]) < 1.0e-15:
                x[2] = 0.0
            if abs(x[5]) < 1.0e-15:
                x[5] = 0.0
            out[n] = x
            n += 1
    return out


def trajectory_filters(samples, mu, device=None):
    """(min r1, min r2, max relative Jacobi drift) of every sampled trajectory
    (samples (m, N, 6)), on the GPU (types/services/manifold.py:412-432,
    common/energy.py:26-74)."""
    import ctypes as C

    from . import _lib
    dev = P._device(device)
    S = torch.as_tensor(samples, dtype=torch.float64, device=dev)
    m, N, _ = S.shape
    soa = S.permute(0, 2, 1).contiguous()
    out = torch.empty((3, max(N, 1)), dtype=torch.float64, device=dev)
    rc = _lib.load().hg_trajectory_filters(N, m, C.c_void_p(soa.data_ptr()), N, float(mu),
                                           C.c_void_p(out[0].data_ptr()), C.c_void_p(out[1].data_ptr()),
                                           C.c_void_p(out[2].data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if rc != _lib.HG_OK:
        raise _lib.HitenGpuError(rc, "hg_trajectory_filters")
    return out[0, :N], out[1, :N], out[2, :N]


def compute(x0, period, mu, stable=True, direction=1, step=0.02, integration_fraction=0.75, NN=1,
            displacement=1e-6, dt=1e-3, method="adaptive", order=8, energy_tol=1e-6, safe_r1=0.0, safe_r2=0.0,
            displacements=None, device=None):
    """Manifold.compute / _ManifoldDynamicsService._run_compute
    (types/services/manifold.py:293-442), with every seed propagated in one
    batched GPU call instead of a Python loop.

    forward = -1 for the stable manifold; seeds at fractions arange(0, 1, step)
    of the period (times the optional `displacements` array for a grid of
    displacement magnitudes); trajectories sampled at
    linspace(0, tf, max(int(tf/dt)+1, 100)) with tf = integration_fraction*2*pi;
    rejected when they come within safe_r1/safe_r2 of a primary or drift in
    Jacobi constant by more than energy_tol.  Returns the reference's tuple
    (ysos, dysos, states_list, times_list, successes, attempts)."""
    if method != "adaptive" or order != 8:
        raise NotImplementedError("manifold propagation on the GPU path is DOP853")
    forward = -1 if stable else 1
    times, PHI = stm_grid(x0, period, mu, steps=2000, forward=forward, device=device)
    eigvec = stable_eigvec(PHI[-1, :36].reshape(6, 6), stable=stable, NN=NN)
    fractions = np.arange(0.0, 1.0, step)
    disps = np.atleast_1d(displacement if displacements is None else displacements)
    seeds_arr = seeds(times, PHI, period, fractions, disps, eigvec, direction=direction)
    tf = integration_fraction * 2 * np.pi
    steps = max(int(abs(tf) / dt) + 1, 100)
    r = P.propagate_dop853(seeds_arr, 0.0, tf, mu, rtol=1e-12, atol=1e-12, max_step=1e4, fwd=forward,
                           flip=(0, 6), n_samples=steps, device=device)
    r1, r2, de = trajectory_filters(r.samples, mu, device=device)
    ok = ((r1 >= safe_r1) & (r2 >= safe_r2) & (de <= energy_tol) & (r.status == 0)).cpu().numpy()
    S = r.samples.permute(1, 0, 2).cpu().numpy()
    t_signed = forward * np.linspace(0.0, tf, steps)
    states_list = [S[i] for i in np.nonzero(ok)[0]]
    times_list = [t_signed.copy() for _ in states_list]
    return [], [], states_list, times_list, int(ok.sum()), len(seeds_arr)


def propagate_to_plane(seeds_arr, mu, tf=8.0, forward=-1, plane_index=0, plane_offset=None, rtol=1e-12,
                       atol=1e-12, max_hits=1, device=None, **kw):
    """DOP853 from every seed to |t| = tf or the first crossing of
    y[plane_index] = plane_offset (default x = 1 - mu), as a terminal event."""
    if plane_offset is None:
        plane_offset = 1.0 - mu
    ev = P.EventSpec(index=plane_index, offset=float(plane_offset), direction=0, max_hits=max_hits)
    return P.propagate_dop853(seeds_arr, 0.0, float(tf), mu, rtol=rtol, atol=atol, max_step=1e4, fwd=forward,
                              flip=(0, 6), event=ev, device=device, **kw)
