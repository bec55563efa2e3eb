"""Halo-family continuation, many families at once.

The reference continues one family at a time (continuation/backends/pc.py:
42-166): from the last accepted member a stepper predicts the next
representation (the orbit's initial state), ``orbit.correct()`` corrects it,
and the step is kept on success or shrunk on failure.  Here K independent
families advance in lock step: every round predicts the next member of every
family still running and corrects all predictions in ONE batched
``corrector.correct_halo`` call on the GPU; each family's accept / reject
bookkeeping is the reference's, per family, so each family's sequence of
members is the one the reference computes on its own.

Steppers (continuation/stepping/):
* ``natural`` (np/base.py): prediction = last + step on the continued state
  components;
* ``secant`` (sc/base.py, support.py; the halo default,
  types/services/orbits.py:964-977): prediction = last + tangent * |step|,
  the tangent seeded from the first natural prediction and replaced after
  every accepted member by the unit difference of the last two members.
On rejection the step is halved (or ``shrink_policy`` applied); steps are
clamped to [step_min, step_max] in magnitude (stepping/base.py).  As in the
reference, a member beyond ``target`` does not stop the family: the inner
loop's target test only ends the attempt, so families run until
``max_members`` or until a member fails ``max_retries_per_step`` times.
"""
from dataclasses import dataclass, field

import numpy as np

from . import corrector as Cr


@dataclass
class ContinuationOptions:
    """continuation/options.py:148-186 and config.py:74-167 (halo defaults)."""

    step: tuple = (0.01,)
    target: tuple = None             # kept for the reference's signature; see the module docstring
    max_members: int = 100
    max_retries_per_step: int = 50
    step_min: float = 1e-10
    step_max: float = 1.0
    shrink_policy: object = None
    stepper: str = "secant"
    state_indices: tuple = (2,)      # SynodicState.Z
    correction: Cr.HaloCorrectionOptions = field(default_factory=Cr.HaloCorrectionOptions)


@dataclass
class FamilyResult:
    family: list                  # accepted representations (initial states), the seed first
    periods: list                 # period of every member (seed: as given)
    parameter_values: tuple       # continued components of every member
    accepted_count: int = 1
    rejected_count: int = 0
    iterations: int = 0

    @property
    def success_rate(self):
        return self.accepted_count / max(self.accepted_count + self.rejected_count, 1)


class _Family:
    def __init__(self, seed, period, o):
        self.o = o
        self.idx = np.asarray(o.state_indices, dtype=int)
        self.members = [np.asarray(seed, dtype=float).copy()]
        self.periods = [float(period) if period is not None else float("nan")]
        self.params = [self.members[0][self.idx].copy()]
        self.acc, self.rej, self.iters = 1, 0, 0
        self.step = np.asarray(o.step, dtype=float).copy()
        self.attempt = 0
        self.done = self.acc >= int(o.max_members)
        self.tangent = None
        if o.stepper == "secant":
            # make_secant_stepper: tangent from the natural predictor's first step
            diff = (self._natural(self.members[0], self.step) - self.members[0]).ravel()
            nrm = float(np.linalg.norm(diff))
            self.tangent = None if nrm == 0.0 else diff / nrm
        elif o.stepper != "natural":
            raise ValueError(f"unknown stepper {o.stepper!r}")

    def _natural(self, last, step):
        out = np.asarray(last, dtype=float).copy()
        for i, d in zip(self.idx, np.asarray(step, dtype=float)):
            out[i] += d
        return out

    def predict(self):
        last = self.members[-1]
        if self.o.stepper == "natural":
            return self._natural(last, self.step)
        ds = float(self.step) if np.ndim(self.step) == 0 else float(np.linalg.norm(self.step))
        if self.tangent is None:
            n = last.copy()
            n[0] = n[0] + ds
            return n
        return last + self.tangent.reshape(last.shape) * ds

    def _clamp(self, vec):
        mag = np.clip(np.abs(vec), self.o.step_min, self.o.step_max)
        return np.sign(vec) * mag

    def accept(self, x, period):
        prev = self.members[-1]
        self.members.append(np.asarray(x, dtype=float).copy())
        self.periods.append(float(period))
        self.params.append(self.members[-1][self.idx].copy())
        self.acc += 1
        if self.o.stepper == "secant":
            d = (self.members[-1] - prev).ravel()
            nrm = float(np.linalg.norm(d))
            self.tangent = None if nrm == 0.0 else d / nrm
        self.step = self._clamp(self.step)
        self.attempt = 0
        if self.acc >= int(self.o.max_members):
            self.done = True

    def reject(self):
        self.rej += 1
        self.attempt += 1
        if self.o.shrink_policy is not None:
            try:
                new = self.o.shrink_policy(self.step)
            except Exception:
                new = self.step * 0.5
        else:
            new = self.step * 0.5
        self.step = self._clamp(new)
        if self.attempt > int(self.o.max_retries_per_step):
            self.done = True

    def result(self):
        return FamilyResult(family=self.members, periods=self.periods, parameter_values=tuple(self.params),
                            accepted_count=self.acc, rejected_count=self.rej, iterations=self.iters)


def continue_halo_families(seeds, seed_periods, mu, options=None, backend=None, device=None):
    """Continue K halo families from corrected seeds (K, 6); `options` is one
    ContinuationOptions for all or a list of K.  Returns K FamilyResults."""
    seeds = np.atleast_2d(np.asarray(seeds, dtype=float))
    K = seeds.shape[0]
    opts = options if isinstance(options, (list, tuple)) else [options or ContinuationOptions()] * K
    periods = np.broadcast_to(np.asarray(seed_periods, dtype=float), (K,))
    fams = [_Family(seeds[k], periods[k], opts[k]) for k in range(K)]
    while True:
        live = [f for f in fams if not f.done]
        if not live:
            break
        preds = np.array([f.predict() for f in live])
        # families with different correction options are corrected in groups
        groups = {}
        for j, f in enumerate(live):
            groups.setdefault(id(f.o.correction), []).append(j)
        for js in groups.values():
            res = Cr.correct_halo(preds[js], mu, options=live[js[0]].o.correction, backend=backend, device=device)
            for r, j in enumerate(js):
                f = live[j]
                f.iters += 1
                if res.status[r] == Cr.STATUS_OK:
                    f.accept(res.x0[r], res.period[r])
                else:
                    f.reject()
    return [f.result() for f in fams]
