"""Oracle-backed stand-in for hiten_gb300.corrector.GpuShootingBackend: the
two propagations of single shooting (the half-period y = 0 crossing and the
STM at it) on the CPU oracle.  Test infrastructure: used by tests/ and by
bench.py's CPU baseline of the correction workload, never by the package.
Follows poincare/singlehit/backend.py:164-280 (the crossing: 1e-12
alignment, window [0, pi], undirected system) and dynamics/rtbp.py:258-340
(_compute_stm, last of 500 dense samples)."""
import numpy as np


def stm_state(x6):
    """42-vector of the variational system: Phi = I (row-major), then the state."""
    y = np.zeros(42)
    y[:36] = np.eye(6).ravel()
    y[36:] = x6
    return y


class OracleShootingBackend:
    """events()/stm() of GpuShootingBackend on the CPU oracle; counts the
    attempted steps of each leg (`attempts[6]`, `attempts[42]`)."""

    def __init__(self, hgo, mu, mode, threads=None):
        self.hgo, self.mu, self.mode = hgo, float(mu), mode
        self.threads = threads
        self.launches = 0
        self.attempts = {6: 0, 42: 0}

    def events(self, x_full):
        self.hgo.set_mode(self.mode)
        span = max(0.0, np.pi - 1e-12)
        r = self.hgo.dop853_event_batch(np.asarray(x_full), 0.0, span, self.mu, 1, 0.0, 0, 1, rtol=1e-12,
                                        atol=1e-12, max_step=np.inf, threads=self.threads)
        self.attempts[6] += int(r["n_accept"].sum() + r["n_reject"].sum())
        t_rel = r["hit_t"][:, 0]
        found = (r["n_hits"] > 0) & (t_rel < span) & (t_rel >= 0.0)
        return 1e-12 + t_rel, r["hit_y"][:, 0, :], found

    def stm(self, x_full, t_event):
        self.hgo.set_mode(self.mode)
        out = np.empty((len(x_full), 6, 6))
        for i, (x, t) in enumerate(zip(x_full, t_event)):
            y, na, nr, _ = self.hgo.dop853_dense(stm_state(x), np.linspace(0.0, t, 500), self.mu, max_step=1e4,
                                                 flip=(36, 42))
            self.attempts[42] += int(na) + int(nr)
            out[i] = y[-1, :36].reshape(6, 6)
        return out
