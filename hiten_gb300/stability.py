"""Eigen-analysis of monodromy matrices on the host, and the batched
monodromy (Floquet) stability of many periodic orbits.

The spectrum routines restate hiten's linear-algebra backend
(algorithms/linalg/backend.py) operation for operation, so that the same
matrix gives the same eigenvalues, eigenvectors and indices:

* ``eigenvalue_decomposition``: _LinalgBackend.eigenvalue_decomposition
  (:196-260) -- numpy eig, imaginary parts below 1e-14 zeroed, every
  eigenvector divided by its first entry of modulus >= 1e-14, entries below
  1e-14 zeroed, real vectors signed so that the pivot is positive
  (_sort_eigenvalues :360-392, _remove_infinitesimals_in_place :497-531);
  then split into stable / unstable / center by |lambda| against 1 -+ delta
  (discrete system, _classify_eigenvalue :300-345), in input order;
* ``real_eigenvectors``: StabilityPipeline.get_real_eigenvectors
  (algorithms/linalg/base.py:116-142), the columns whose eigenvalue
  np.isreal accepts;
* ``stability_indices``: _LinalgBackend.stability_indices (:262-300) --
  the spectrum cleaned at 1e-12, normalised as above, then the unit-modulus
  pair first and reciprocal pairs after it (_compute_nu_from_eigvals
  :420-470), nu = (lambda + 1/lambda) / 2, padded with NaN.

``compute_stability`` is orbit.compute_stability()
(types/services/orbits.py:664-687) for K orbits at once: one batched
42-dimensional DOP853 propagation of the variational system over each
orbit's period on the GPU (_compute_stm with its defaults: 2000 dense
samples, the last of which is the monodromy), then the indices per orbit.
"""
import numpy as np

from . import propagate as P
from .workloads import identity_stm_state


def _zero_small_imag(ev, tol):
    """_zero_small_imag_part: the imaginary part below tol becomes +0."""
    if abs(ev.imag) < tol:
        return complex(ev.real, 0.0)
    return ev


def _remove_infinitesimals(vec, tol):
    """_remove_infinitesimals_array on a copy (real and imaginary parts below tol zeroed)."""
    v = vec.copy()
    for i in range(len(v)):
        re = v[i].real
        im = v[i].imag
        if abs(re) < tol:
            re = 0.0
        if abs(im) < tol:
            im = 0.0
        v[i] = re + 1j * im
    return v


def _normalize(eigvals, eigvecs):
    """_sort_eigenvalues: cleaned eigenvalues and pivot-normalised eigenvectors (order kept)."""
    vals = np.array([_zero_small_imag(ev, 1e-14) for ev in eigvals])
    vecs = eigvecs.astype(np.complex128)
    for k in range(vecs.shape[1]):
        vec = vecs[:, k]
        p = 0
        while p < vec.shape[0] and abs(vec[p]) < 1e-14:
            p += 1
        if p < vec.shape[0]:
            pivot = vec[p]
            if abs(pivot) > 1e-14:
                vec = vec / pivot
                vecs[:, k] = vec
        vecs[:, k] = _remove_infinitesimals(vecs[:, k], 1e-14)
        if np.max(np.abs(vecs[:, k].imag)) < 1e-14 and p < vecs.shape[0]:
            if vecs[p, k].real < 0:
                vecs[:, k] = -vecs[:, k]
    return vals, vecs


def eigenvalue_decomposition(A, delta=1e-4):
    """(sn, un, cn, Ws, Wu, Wc) of a monodromy matrix (discrete system):
    |lambda| < 1 - delta stable, > 1 + delta unstable, else center."""
    try:
        w, V = np.linalg.eig(A)
    except np.linalg.LinAlgError:
        n = A.shape[0]
        e = np.array([], dtype=np.complex128)
        z = np.zeros((n, 0), dtype=np.complex128)
        return e, e, e, z, z, z
    vals, vecs = _normalize(w, V)
    s, u, c, ws, wu, wc = [], [], [], [], [], []
    for val, vec in zip(vals, vecs.T):
        mag = abs(val)
        if mag < 1 - delta:
            s.append(val)
            ws.append(vec)
        elif mag > 1 + delta:
            u.append(val)
            wu.append(vec)
        else:
            c.append(val)
            wc.append(vec)
    n = A.shape[0]

    def stack(cols):
        return np.column_stack(cols) if cols else np.zeros((n, 0), dtype=np.complex128)
    return (np.array(s, dtype=np.complex128), np.array(u, dtype=np.complex128), np.array(c, dtype=np.complex128),
            stack(ws), stack(wu), stack(wc))


def real_eigenvectors(vectors, values):
    """(real eigenvalues, their eigenvectors): the columns np.isreal keeps."""
    mask = np.isreal(values)
    vals = values[mask].astype(np.complex128)
    vecs = vectors[:, mask] if np.any(mask) else np.zeros((vectors.shape[0], 0), dtype=np.complex128)
    return vals, vecs


def _nu(ev):
    return (ev + 1.0 / ev) / 2.0


def stability_indices(M, tol=1e-8):
    """(nu (3,), eigenvalues (6,), eigenvectors (6, 6)) of a 6x6 monodromy matrix."""
    M = np.asarray(M)
    if M.shape != (6, 6):
        raise ValueError(f"monodromy matrix has shape {M.shape}, expected (6, 6)")
    try:
        w, V = np.linalg.eig(M)
    except np.linalg.LinAlgError:
        w, V = np.array([], dtype=np.complex128), np.zeros((6, 0), dtype=np.complex128)
    w = np.array([_zero_small_imag(ev, 1e-12) for ev in w])
    vals, vecs = _normalize(w, V)
    used = np.zeros(vals.shape[0], dtype=bool)
    nu = []
    unit = [i for i, ev in enumerate(vals) if not used[i] and np.isclose(abs(ev), 1.0, rtol=tol, atol=tol)]
    if len(unit) >= 2:
        nu.append(_nu(vals[unit[0]]))
        used[unit[0]] = True
        used[unit[1]] = True
    elif len(unit) == 1:
        nu.append(_nu(vals[unit[0]]))
        used[unit[0]] = True
    n = vals.shape[0]
    for i in range(n):
        if used[i]:
            continue
        ev = vals[i]
        if abs(ev) < tol * tol:
            used[i] = True
            continue
        target = 1.0 / ev
        match = -1
        for j in range(i + 1, n):
            if used[j]:
                continue
            if np.isclose(vals[j], target, rtol=tol, atol=tol):
                match = j
                break
        used[i] = True
        if match >= 0:
            nu.append(_nu(ev))
            used[match] = True
        if len(nu) >= 3:
            break
    while len(nu) < 3:
        nu.append(np.nan + 0j)
    return np.array(nu, dtype=np.complex128), vals, vecs


def monodromy_batch(x0, periods, mu, steps=2000, rtol=1e-12, atol=1e-12, device=None):
    """Phi(T_k) of every orbit (K, 6, 6): one batched 42-dimensional DOP853
    propagation of the variational system from Phi = I over each orbit's
    period, the last of `steps` dense samples (dynamics/rtbp.py:258-340)."""
    x0 = np.atleast_2d(np.asarray(x0, dtype=np.float64))
    T = np.atleast_1d(np.asarray(periods, dtype=np.float64))
    r = P.propagate_dop853(identity_stm_state(x0), 0.0, T, mu, rtol=rtol, atol=atol, max_step=1e4, flip=(36, 42),
                           n_samples=int(steps), sample_last_only=True, device=device)
    return r.samples[0, :, :36].cpu().numpy().reshape(-1, 6, 6)


def compute_stability(x0, periods, mu, tol=1e-8, device=None):
    """orbit.compute_stability() for K orbits: (nu (K, 3), eigenvalues (K, 6),
    eigenvectors (K, 6, 6), monodromy (K, 6, 6))."""
    Phi = monodromy_batch(x0, periods, mu, device=device)
    nus, vals, vecs = [], [], []
    for M in Phi:
        nu, w, V = stability_indices(M, tol)
        nus.append(nu)
        vals.append(w)
        vecs.append(V)
    return np.array(nus), np.array(vals), np.array(vecs), Phi
