"""Reference-shaped propagation drop-ins (dynamics/base.py:346-458,
dynamics/rtbp.py:258-378), batched over a leading trajectory axis.

`CR3BPSystem` stands in for the reference's `_RTBPRHS` / `_VarEqRHS`
dynamical systems (rtbp.py:425-616): it carries `mu`, the dimension (6 or
42) and, for backward integration, the direction and flipped components of
`_DirectedSystem` (base.py:186-343).  Events are plane events (`PlaneEvent`),
the form every hot-path caller uses (singlehit `_g_y0`, the manifold's
x = 1 - mu plane, section planes); they run on the GPU inside the integrator.
"""
from dataclasses import dataclass

import numpy as np

from . import propagate as P


@dataclass
class CR3BPSystem:
    """CR3BP vector field: dim 6 (state) or 42 (STM + state)."""

    mu: float
    dim: int = 6
    fwd: int = 1
    flip: tuple = None

    def __post_init__(self):
        if self.dim not in (6, 42):
            raise ValueError(f"dim must be 6 or 42, got {self.dim}")

    @property
    def var(self):
        return CR3BPSystem(self.mu, 42)


@dataclass
class PlaneEvent:
    """g(t, y) = y[index] - offset (poincare/singlehit/backend.py:35-68)."""

    index: int
    offset: float = 0.0


@dataclass
class EventConfig:
    """types/configs.py:180-201."""

    direction: int = 0
    terminal: bool = True

    def __post_init__(self):
        if self.direction not in (-1, 0, 1):
            raise ValueError(f"Invalid direction: {self.direction}")


@dataclass
class EventOptions:
    """types/options.py:265-288."""

    xtol: float = 1e-12
    gtol: float = 1e-12

    def __post_init__(self):
        if self.xtol <= 0 or self.gtol <= 0:
            raise ValueError("xtol and gtol must be positive")


@dataclass
class Solution:
    """integrators/types.py:30-72, with an optional leading trajectory axis:
    times (m,) or (N, m) when event times differ per trajectory;
    states (m, dim) or (N, m, dim)."""

    times: np.ndarray
    states: np.ndarray
    derivatives: np.ndarray = None


def validate_initial_state(state0, dim):
    """dynamics/base.py:461-493: (dim,) or (N, dim) float64."""
    s = np.asarray(state0, dtype=np.float64)
    if s.shape[-1] != dim or s.ndim not in (1, 2):
        raise ValueError(f"Initial state dimension {s.shape[-1]} != system dimension {dim}")
    return s


def propagate_dynsys(dynsys, state0, t0, tf, forward=1, steps=1000, method="adaptive", order=8, flip_indices=None,
                     **kwargs):
    """_propagate_dynsys on the GPU.  `dynsys`: CR3BPSystem.  kwargs: rtol,
    atol, max_step (adaptive defaults 1e-12, 1e-12, 1e4), event_fn
    (PlaneEvent), event_cfg (EventConfig), event_options (EventOptions)."""
    if method == "symplectic":
        raise ValueError("Symplectic method requires a _HamiltonianSystem")
    if method not in ("fixed", "adaptive"):
        raise ValueError(f"unknown method {method!r}")
    s0 = validate_initial_state(state0, dynsys.dim)
    single = s0.ndim == 1
    Y0 = s0[None] if single else s0
    fwd = 1 if forward >= 0 else -1
    flip = _flip_range(flip_indices, dynsys.dim)
    t_eval = np.linspace(t0, tf, steps)
    event_fn = kwargs.get("event_fn")
    if steps >= 2 and np.isclose(t_eval[0], t_eval[-1]):
        states = np.repeat(Y0[:, None, :], len(t_eval), axis=1)
        return Solution(fwd * t_eval, states[0] if single else states)
    if event_fn is not None:
        cfg = kwargs.get("event_cfg") or EventConfig()
        opt = kwargs.get("event_options") or EventOptions()
        ev = P.EventSpec(index=int(event_fn.index), offset=float(event_fn.offset), direction=int(cfg.direction),
                         max_hits=1, xtol=float(opt.xtol), gtol=float(opt.gtol))
        if method == "fixed":
            out, ht, hy, nh = P.propagate_fixed_event(Y0, t_eval, dynsys.mu, ev, order=order, fwd=fwd, flip=flip)
            hit = nh.cpu().numpy() > 0
            times = np.stack([np.full(len(Y0), t_eval[0]), np.where(hit, ht.cpu().numpy(), t_eval[-1])], axis=1)
            last = np.where(hit[:, None], hy.cpu().numpy(), out[-1].cpu().numpy())
            states = np.stack([Y0, last], axis=1)
            times = times * fwd
            return Solution(times[0] if single else times, states[0] if single else states)
        r = P.propagate_dop853(Y0, float(t_eval[0]), float(t_eval[-1]), dynsys.mu, rtol=kwargs.get("rtol", 1e-12),
                               atol=kwargs.get("atol", 1e-12), max_step=kwargs.get("max_step", 1e4), fwd=fwd,
                               flip=flip, event=ev)
        hit = r.n_hits.cpu().numpy() > 0
        t_hit = r.hit_t[:, 0].cpu().numpy()
        times = np.stack([np.full(len(Y0), t_eval[0]), np.where(hit, t_hit, t_eval[-1])], axis=1) * fwd
        last = np.where(hit[:, None], r.hit_y[:, 0, :].cpu().numpy(), r.y_end.cpu().numpy())
        states = np.stack([Y0, last], axis=1)
        return Solution(times[0] if single else times, states[0] if single else states)
    if method == "fixed":
        out = P.propagate_fixed(Y0, t_eval, dynsys.mu, order=order, fwd=fwd, flip=flip)  # (m, N, dim)
        states = out.permute(1, 0, 2).cpu().numpy()
    else:
        if order != 8:
            raise NotImplementedError("the adaptive GPU path is DOP853 (order 8)")
        r = P.propagate_dop853(Y0, float(t_eval[0]), float(t_eval[-1]), dynsys.mu, rtol=kwargs.get("rtol", 1e-12),
                               atol=kwargs.get("atol", 1e-12), max_step=kwargs.get("max_step", 1e4), fwd=fwd,
                               flip=flip, n_samples=len(t_eval))
        states = r.samples.permute(1, 0, 2).cpu().numpy()
    return Solution(fwd * t_eval, states[0] if single else states)


def _flip_range(flip_indices, dim):
    if flip_indices is None:
        return (0, dim)
    if isinstance(flip_indices, slice):
        return (0 if flip_indices.start is None else flip_indices.start,
                dim if flip_indices.stop is None else flip_indices.stop)
    idx = sorted(int(i) for i in flip_indices)
    if idx and idx != list(range(idx[0], idx[-1] + 1)):
        raise ValueError("flip_indices must be a contiguous range")
    return (idx[0], idx[-1] + 1) if idx else (0, 0)


def compute_stm(var_dynsys, x0, tf, steps=2000, forward=1, method="adaptive", order=8, **kwargs):
    """_compute_stm (dynamics/rtbp.py:258-340): Phi0 = I, flip of 36:42 only.
    Returns (x (steps, 6), times, phi_T (6, 6), PHI (steps, 42)); batched
    x0 (N, 6) gives (N, ...) arrays."""
    x0 = np.asarray(x0, dtype=np.float64)
    single = x0.ndim == 1
    X = x0[None] if single else x0
    PHI0 = np.zeros((len(X), 42))
    PHI0[:, :36] = np.eye(6).ravel()
    PHI0[:, 36:] = X
    sol = propagate_dynsys(var_dynsys if var_dynsys.dim == 42 else var_dynsys.var, PHI0, 0.0, tf, forward=forward,
                           steps=steps, method=method, order=order, flip_indices=slice(36, 42), **kwargs)
    PHI = sol.states
    x = PHI[..., 36:42]
    phi_T = PHI[..., -1, :36].reshape(PHI.shape[:-2] + (6, 6))
    if single:
        return x[0], sol.times, phi_T[0], PHI[0]
    return x, sol.times, phi_T, PHI


def compute_monodromy(var_dynsys, x0, period):
    """_compute_monodromy (rtbp.py:343-378): Phi(T)."""
    _, _, M, _ = compute_stm(var_dynsys, x0, period)
    return M


def stability_indices(monodromy):
    """_stability_indices (rtbp.py:381-420), host numpy as the reference."""
    eigs = np.linalg.eigvals(monodromy)
    eigs = sorted(eigs, key=abs, reverse=True)
    nu1 = 0.5 * (eigs[2] + 1 / eigs[2])
    nu2 = 0.5 * (eigs[4] + 1 / eigs[4])
    return (nu1, nu2), eigs
