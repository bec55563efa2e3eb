"""The batched Newton/Armijo bookkeeping of hiten_gb300.corrector against a
per-orbit restatement of the reference's loop (corrector/backends/newton.py:
39-143, stepping/armijo.py:58-164), on a fake shooting backend whose
residual, crossings and Jacobian are chosen so that every branch runs:
accepted full steps, halved steps, trials without a crossing, the best
trial kept at the minimum step, and line-search failures."""
import numpy as np
import pytest

from hiten_gb300 import corrector as C


class FakeBackend:
    """Residual r(p) = A (p - p*) + c |p - p*|^2 (p = (x0, vy0)); no crossing
    when x0 leaves a window; the Jacobian handed to Newton is A scaled by
    `jac_scale` (a wrong scale forces the line search to work)."""

    def __init__(self, pstar, A, c, window, jac_scale):
        self.pstar, self.A, self.c, self.window, self.jac_scale = pstar, A, c, window, jac_scale
        self.launches = 0
        self._rows = None

    def _r(self, x_full):
        p = x_full[:, [0, 4]]
        i = np.rint(x_full[:, 1] * 1e6).astype(int)  # orbit id carried in y (unused by the logic)
        d = p - self.pstar[i]
        return np.einsum("nij,nj->ni", self.A[i], d) + self.c[i][:, None] * np.sum(d * d, axis=1)[:, None], i

    def events(self, x_full):
        self.launches += 1
        r, i = self._r(x_full)
        x_ev = np.zeros_like(x_full)
        x_ev[:, 3] = r[:, 0]
        x_ev[:, 5] = r[:, 1]
        x_ev[:, 4] = 1.0
        found = np.abs(x_full[:, 0] - self.pstar[i, 0]) < self.window[i]
        return 1.0 + 0.01 * i, x_ev, found

    def stm(self, x_full, t_event):
        self.launches += 1
        _, i = self._r(x_full)
        Phi = np.zeros((x_full.shape[0], 6, 6))
        J = self.A[i] * self.jac_scale[i][:, None, None]
        Phi[:, 3, 0], Phi[:, 3, 4], Phi[:, 5, 0], Phi[:, 5, 4] = J[:, 0, 0], J[:, 0, 1], J[:, 1, 0], J[:, 1, 1]
        return Phi


def scalar_reference(be, guesses, o):
    """Per-orbit restatement of the reference's single-shooting Newton with Armijo."""
    out = []
    for n in range(guesses.shape[0]):
        base = guesses[n].copy()

        def resid(p):
            x = base.copy()
            x[[0, 4]] = p
            t, xe, f = be.events(x[None])
            r = xe[0, [3, 5]]
            return r, np.max(np.abs(r)), bool(f[0])

        p = base[[0, 4]].copy()
        r, rn, f = resid(p)
        if not f:
            out.append((C.STATUS_NO_EVENT, 0, p))
            continue
        status, it = C.STATUS_MAX_ITER, o.max_attempts
        for k in range(o.max_attempts):
            if rn < o.tol:
                status, it = C.STATUS_OK, k
                break
            x = base.copy()
            x[[0, 4]] = p
            Phi = be.stm(x[None], None)[0]
            J = Phi[[3, 5]][:, [0, 4]]
            delta = np.linalg.solve(J, -r)
            dn = np.max(np.abs(delta))
            if dn > o.max_delta:
                delta = delta * (o.max_delta / dn)
            # armijo.py: best starts at the current point (norm rn, alpha 0); a trial
            # without a crossing is a failed evaluation (smaller step, no best update)
            alpha, done = 1.0, False
            best_p, best_n, best_r, best_a = p, rn, r, 0.0
            while alpha >= o.min_alpha:
                trial = p + alpha * delta
                rt, nt, ft = resid(trial)
                if not ft:
                    alpha *= o.alpha_reduction
                    continue
                if nt <= (1.0 - o.armijo_c * alpha) * rn:
                    p, r, rn, done = trial, rt, nt, True
                    break
                if nt < best_n:
                    best_p, best_n, best_r, best_a = trial, nt, rt, alpha
                alpha *= o.alpha_reduction
            if not done:
                if best_a == 0.0:
                    status, it = C.STATUS_LINE_SEARCH, k
                    break
                p, rn, r = best_p, best_n, best_r
        else:
            status = C.STATUS_OK if rn < o.tol else C.STATUS_MAX_ITER
        out.append((status, it, p))
    return out


@pytest.mark.parametrize("trials", [None, 1, 3, 8])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_batched_armijo_matches_per_orbit_loop(seed, trials, monkeypatch):
    """trials: step fractions evaluated per round and orbit (speculative
    rounds must decide exactly as one trial per round)."""
    monkeypatch.setattr(C, "halo_quadratic_term", lambda x_ev, Phi, mu: np.zeros((x_ev.shape[0], 2, 2)))
    rng = np.random.default_rng(seed)
    n = 40
    pstar = np.c_[rng.uniform(0.8, 1.2, n), rng.uniform(-0.3, 0.3, n)]
    A = rng.normal(size=(n, 2, 2)) + 3 * np.eye(2)
    c = rng.uniform(0.0, 40.0, n)                      # strong curvature: full steps overshoot
    window = rng.uniform(2e-3, 5e-2, n)                # some trials lose the crossing
    jac_scale = rng.choice([1.0, 1.0, 0.3, -1.0], n)   # wrong or reversed Jacobians: line search fails
    guesses = np.zeros((n, 6))
    guesses[:, 0] = pstar[:, 0] + rng.uniform(-1, 1, n) * window * 0.9
    guesses[:, 4] = pstar[:, 1] + rng.uniform(-5e-3, 5e-3, n)
    guesses[:, 1] = np.arange(n) * 1e-6
    o = C.HaloCorrectionOptions(max_attempts=12, trials_per_round=trials)
    got = C.correct_halo(guesses, 0.0121505856, options=o, backend=FakeBackend(pstar, A, c, window, jac_scale))
    ref = scalar_reference(FakeBackend(pstar, A, c, window, jac_scale), guesses, o)
    statuses = set()
    for i, (st, it, p) in enumerate(ref):
        statuses.add(st)
        assert got.status[i] == st, i
        if st != C.STATUS_NO_EVENT:
            assert got.iterations[i] == it, i
            assert np.array_equal(got.x0[i, [0, 4]], p), i
    assert C.STATUS_OK in statuses and len(statuses) >= 2
