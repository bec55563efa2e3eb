"""CPU oracle of the two all-pairs searches of hiten_gb300.connections
(test infrastructure only: tests and nothing else use it).

Restates connections/backends.py:31-99 (_pair_counts / _radpair2d, with the
per-query minimum that _ConnectionsBackend.run takes over the pairs,
:444-460) and :174-235 (_nearest_neighbor_2d_numba) in FP64 numpy: the same
expressions (dx*dx + dy*dy, <= r^2, strict minima with the first index
winning ties)."""
import numpy as np


class OracleSectionMatcher:
    def radius_best(self, q, r, eps, coord_max=None):
        r2 = float(eps) * float(eps)
        n = q.shape[0]
        cnt = np.zeros(n, dtype=np.int64)
        bi = np.full(n, -1, dtype=np.int64)
        bd = np.zeros(n)
        for i in range(n):
            dx = q[i, 0] - r[:, 0]
            dy = q[i, 1] - r[:, 1]
            d2 = dx * dx + dy * dy
            hit = np.nonzero(d2 <= r2)[0]
            cnt[i] = hit.size
            if hit.size:
                k = hit[np.argmin(d2[hit])]
                bi[i], bd[i] = k, d2[k]
        return cnt, bi, bd

    def nearest(self, p, coord_max=None):
        n = p.shape[0]
        out = np.full(n, -1, dtype=np.int64)
        for i in range(n):
            dx = p[i, 0] - p[:, 0]
            dy = p[i, 1] - p[:, 1]
            d2 = dx * dx + dy * dy
            d2[i] = np.inf
            if n > 1:
                out[i] = int(np.argmin(d2))
        return out
