"""Oracle-backed stand-ins for the GPU propagation backends (tests only)."""
import numpy as np

from helpers import stm_state


class OracleShootingBackend:
    """events()/stm() of hiten_gb300.corrector.GpuShootingBackend on the CPU oracle."""

    def __init__(self, hgo, mu, mode):
        self.hgo, self.mu, self.mode = hgo, float(mu), mode
        self.launches = 0

    def events(self, x_full):
        self.hgo.set_mode(self.mode)
        span = max(0.0, np.pi - 1e-12)
        r = self.hgo.dop853_event_batch(np.asarray(x_full), 0.0, span, self.mu, 1, 0.0, 0, 1, rtol=1e-12,
                                        atol=1e-12, max_step=np.inf)
        t_rel = r["hit_t"][:, 0]
        found = (r["n_hits"] > 0) & (t_rel < span) & (t_rel >= 0.0)
        return 1e-12 + t_rel, r["hit_y"][:, 0, :], found

    def stm(self, x_full, t_event):
        self.hgo.set_mode(self.mode)
        out = np.empty((len(x_full), 6, 6))
        for i, (x, t) in enumerate(zip(x_full, t_event)):
            y, _, _, _ = self.hgo.dop853_dense(stm_state(x), np.linspace(0.0, t, 500), self.mu, max_step=1e4,
                                               flip=(36, 42))
            out[i] = y[-1, :36].reshape(6, 6)
        return out
