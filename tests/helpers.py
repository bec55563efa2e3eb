"""Shared comparison helpers for the parity tests."""
import numpy as np


def rowwise_rel(a, b):
    """max over rows of ||a_row - b_row||_inf / max(||b_row||_inf, 1)."""
    a = np.asarray(a, dtype=np.float64).reshape(-1, np.shape(a)[-1])
    b = np.asarray(b, dtype=np.float64).reshape(-1, np.shape(b)[-1])
    num = np.max(np.abs(a - b), axis=1)
    den = np.maximum(np.max(np.abs(b), axis=1), 1.0)
    return float(np.max(num / den)) if num.size else 0.0


def stm_state(x6):
    y = np.zeros(42)
    y[:36] = np.eye(6).ravel()
    y[36:] = x6
    return y


def truth_distances(tag, hit_t, hit_y, n_hits, y_end, truth):
    """Per trajectory, the largest distance to the exact solution of
    tests/golden/truth_mpmath.npz over crossing times, crossing states and
    (section runs that stopped before their 8th crossing) the end state;
    each as |a - b|_inf / max(|b|_inf, 1); inf when the crossing counts differ.
    hit_t (n, H), hit_y (n, H, 6), n_hits (n,), y_end (n, 6)."""
    n = len(n_hits)
    out = np.empty(n)
    for i in range(n):
        if tag == "section":
            k = int(truth["section_n_hits"][i])
            tt, ty = truth["section_hit_t"][i, :k], truth["section_hit_y"][i, :k]
            ends = (y_end[i], truth["section_y_end"][i]) if k < hit_t.shape[1] else None
        else:
            k = int(truth["manifold_hit"][i])
            tt, ty = truth["manifold_t"][i:i + 1], truth["manifold_y"][i:i + 1]
            ends = None if k else (y_end[i], truth["manifold_y"][i])
        if int(n_hits[i]) != k:
            out[i] = np.inf
            continue
        v = 0.0
        if k:
            v = max(float(np.max(np.abs(hit_t[i, :k] - tt) / np.maximum(np.abs(tt), 1.0))),
                    rowwise_rel(hit_y[i, :k], ty))
        if ends is not None:
            v = max(v, rowwise_rel(ends[0][None], ends[1][None]))
        out[i] = v
    return out
