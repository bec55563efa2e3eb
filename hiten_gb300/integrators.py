"""Integrator objects with the reference's `integrate` contract
(integrators/base.py:75-262, integrators/rk.py:2871-2979), batched.

`RungeKutta(order)` mirrors the reference factory: 4, 6, 8 -> fixed step;
853 -> adaptive DOP853 (45/RK45 is not on the GPU path).  `integrate(system,
y0, t_vals, event_fn=None, event_cfg=None, event_options=None)` validates as
the reference does (dimension, >= 2 nodes, strictly monotone or all-equal,
zero-span short-circuit) and returns a `dynamics.Solution`.
"""
import numpy as np

from . import propagate as P
from .dynamics import EventConfig, EventOptions, Solution, validate_initial_state

EPS = float(np.finfo(float).eps)


class _GpuIntegrator:
    def __init__(self, name, **options):
        self.name = name
        self.options = options

    def validate_inputs(self, system, y0, t_vals):
        """integrators/base.py:148-191."""
        if not hasattr(system, "mu") or not hasattr(system, "dim"):
            raise ValueError(f"System must provide 'mu' and 'dim' for {self.name}")
        y0 = validate_initial_state(y0, system.dim)
        t_vals = np.asarray(t_vals, dtype=np.float64)
        if len(t_vals) < 2:
            raise ValueError("Must provide at least 2 time points")
        dt = np.diff(t_vals)
        if np.all(dt == 0.0):
            return y0, t_vals
        if not (np.all(dt > 0) or np.all(dt < 0)):
            raise ValueError("Time values must be strictly monotonic (either increasing or decreasing)")
        return y0, t_vals

    @staticmethod
    def _constant(y0, t_vals):
        """integrators/base.py:199-234 (states repeated; derivatives omitted)."""
        if t_vals.size >= 2 and np.isclose(t_vals[0], t_vals[-1]):
            Y = np.atleast_2d(y0)
            st = np.repeat(Y[:, None, :], t_vals.size, axis=1)
            return Solution(times=t_vals.copy(), states=st[0] if y0.ndim == 1 else st)
        return None

    @staticmethod
    def _dir(system):
        fwd = getattr(system, "fwd", 1)
        flip = getattr(system, "flip", None)
        return fwd, flip


class GpuFixedRK(_GpuIntegrator):
    def __init__(self, order=8, **options):
        if order not in (4, 6, 8):
            raise ValueError("RK order must be 4, 6, or 8")
        super().__init__(f"_RK{order}", **options)
        self.order = order

    def integrate(self, system, y0, t_vals, *, event_fn=None, event_cfg=None, event_options=None, **kwargs):
        y0, t_vals = self.validate_inputs(system, y0, t_vals)
        c = self._constant(y0, t_vals)
        if c is not None:
            return c
        fwd, flip = self._dir(system)
        Y = np.atleast_2d(y0)
        if event_fn is not None:
            cfg = event_cfg or EventConfig()
            opt = event_options or EventOptions()
            ev = P.EventSpec(index=int(event_fn.index), offset=float(event_fn.offset), direction=int(cfg.direction),
                             max_hits=1, xtol=float(opt.xtol), gtol=float(opt.gtol))
            out, ht, hy, nh = P.propagate_fixed_event(Y, t_vals, system.mu, ev, order=self.order, fwd=fwd, flip=flip)
            hit = nh.cpu().numpy() > 0
            times = np.stack([np.full(len(Y), t_vals[0]), np.where(hit, ht.cpu().numpy(), t_vals[-1])], axis=1)
            last = np.where(hit[:, None], hy.cpu().numpy(), out[-1].cpu().numpy())
            states = np.stack([Y, last], axis=1)
            if y0.ndim == 1:
                return Solution(times=times[0], states=states[0])
            return Solution(times=times, states=states)
        out = P.propagate_fixed(Y, t_vals, system.mu, order=self.order, fwd=fwd, flip=flip).permute(1, 0, 2)
        st = out.cpu().numpy()
        return Solution(times=t_vals.copy(), states=st[0] if y0.ndim == 1 else st)


class GpuDOP853(_GpuIntegrator):
    """AdaptiveRK(order=8): rtol = atol = 1e-13 and max_step = inf by
    default (integrators/rk.py:786-838), min_step = 10 eps."""

    def __init__(self, rtol=1e-13, atol=1e-13, max_step=np.inf, min_step=None, **options):
        super().__init__("_DOP853", **options)
        self.rtol, self.atol, self.max_step = float(rtol), float(atol), float(max_step)
        self.min_step = 10.0 * EPS if min_step is None else float(min_step)

    def integrate(self, system, y0, t_vals, *, event_fn=None, event_cfg=None, event_options=None, **kwargs):
        y0, t_vals = self.validate_inputs(system, y0, t_vals)
        c = self._constant(y0, t_vals)
        if c is not None:
            return c
        fwd, flip = self._dir(system)
        Y = np.atleast_2d(y0)
        if event_fn is not None:
            cfg = event_cfg or EventConfig()
            opt = event_options or EventOptions()
            ev = P.EventSpec(index=int(event_fn.index), offset=float(event_fn.offset), direction=int(cfg.direction),
                             max_hits=1, xtol=float(opt.xtol), gtol=float(opt.gtol))
            r = P.propagate_dop853(Y, float(t_vals[0]), float(t_vals[-1]), system.mu, rtol=self.rtol, atol=self.atol,
                                   max_step=self.max_step, min_step=self.min_step, fwd=fwd, flip=flip, event=ev)
            hit = r.n_hits.cpu().numpy() > 0
            t_end = np.where(hit, r.hit_t[:, 0].cpu().numpy(), t_vals[-1])
            last = np.where(hit[:, None], r.hit_y[:, 0, :].cpu().numpy(), r.y_end.cpu().numpy())
            times = np.stack([np.full(len(Y), t_vals[0]), t_end], axis=1)
            states = np.stack([Y, last], axis=1)
            if y0.ndim == 1:
                return Solution(times=times[0], states=states[0])
            return Solution(times=times, states=states)
        if not np.array_equal(t_vals, np.linspace(t_vals[0], t_vals[-1], len(t_vals))):
            raise NotImplementedError("dense output is produced on linspace(t0, tf, n) grids")
        r = P.propagate_dop853(Y, float(t_vals[0]), float(t_vals[-1]), system.mu, rtol=self.rtol, atol=self.atol,
                               max_step=self.max_step, min_step=self.min_step, fwd=fwd, flip=flip,
                               n_samples=len(t_vals))
        st = r.samples.permute(1, 0, 2).cpu().numpy()
        return Solution(times=t_vals.copy(), states=st[0] if y0.ndim == 1 else st)


def RungeKutta(order=4, **opts):
    """integrators/rk.py:2945-2979."""
    if order in (4, 6, 8):
        return GpuFixedRK(order, **opts)
    if order == 853:
        return GpuDOP853(**opts)
    raise ValueError("Runge-Kutta order not supported")


def FixedRK(order=4, **opts):
    return GpuFixedRK(order, **opts)


def AdaptiveRK(order=8, **opts):
    if order != 8:
        raise ValueError("Adaptive RK order not supported")
    return GpuDOP853(**opts)
