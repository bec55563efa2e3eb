"""High-precision ground truth for the adaptive workloads (mpmath Taylor series).

For the first N states of each seeded sample in ``libm_spread.npz`` (the
synodic-section workload: DOP853 1e-11 to t = 20, up to 8 decreasing y = 0
crossings, terminal at the 8th; the stable-manifold workload: the flipped
field to tau = 8, terminal at the first x = 1 - mu crossing) this script
integrates the CR3BP with mpmath's Taylor-series ODE solver (``mp.odefun``) at
30 significant digits and a local tolerance of 1e-25, from the same binary64
initial states and the same binary64 mu (both converted exactly), and locates
the crossings by a scan at spacing 0.005 plus a bracketed root solve.  Each
solution is computed a second time at tolerance 1e-21; the largest relative
difference between the two is stored beside the truth (``check``).

The truth is the exact solution of the reference's ODE, independent of any
floating-point evaluation order, so the distances to it of the reference's
arithmetic (both glibc pow builds, in ``libm_spread.npz``), of the kernels'
arithmetic (correctly rounded powers) and of the GPU can be set side by side.

    python tests/golden/make_truth_mpmath.py      # writes truth_mpmath.npz
"""
import json
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
N = 24
DPS = 30
TOL, TOL_CHECK = 25, 21
SCAN = 0.005
MAX_HITS = 8


def _solution(y0, mu, sign, tol):
    import mpmath as mp
    mp.mp.dps = DPS
    m = mp.mpf(float(mu))

    def f(t, s):
        x, y, z, vx, vy, vz = s
        r1 = mp.sqrt((x + m) ** 2 + y ** 2 + z ** 2)
        r2 = mp.sqrt((x - 1 + m) ** 2 + y ** 2 + z ** 2)
        a = (1 - m) / r1 ** 3
        b = m / r2 ** 3
        d = [vx, vy, vz, 2 * vy + x - a * (x + m) - b * (x - 1 + m), -2 * vx + y - a * y - b * y, -a * z - b * z]
        return d if sign > 0 else [-c for c in d]

    return mp.odefun(f, 0, [mp.mpf(float(v)) for v in y0], tol=mp.mpf(10) ** (-tol)), m


def _root(sol, comp, off, lo, hi):
    import mpmath as mp
    g = lambda t: sol(t)[comp] - off  # noqa: E731
    a, b = mp.mpf(lo), mp.mpf(hi)
    ga = g(a)
    for _ in range(200):  # bisection to below 1e-27 of the bracket
        mid = (a + b) / 2
        gm = g(mid)
        if (gm > 0) == (ga > 0) and gm != 0:
            a, ga = mid, gm
        else:
            b = mid
        if b - a < mp.mpf(10) ** (-(DPS - 3)):
            break
    return (a + b) / 2


def section_task(args):
    """Decreasing y = 0 crossings up to t = 20 (terminal at the 8th)."""
    y0, mu, tol = args
    import mpmath as mp
    sol, _ = _solution(y0, mu, 1, tol)
    times, states = [], []
    k, t_prev = 0, mp.mpf(0)
    g_prev = sol(t_prev)[1]
    n_scan = int(round(20.0 / SCAN))
    while k < n_scan and len(times) < MAX_HITS:
        k += 1
        t = mp.mpf(k) * mp.mpf(SCAN) if k < n_scan else mp.mpf(20)
        g = sol(t)[1]
        if g_prev > 0 and g <= 0:
            tr = _root(sol, 1, 0, t_prev, t)
            times.append(tr)
            states.append(sol(tr))
        t_prev, g_prev = t, g
    t_end = times[-1] if len(times) == MAX_HITS else mp.mpf(20)
    y_end = states[-1] if len(times) == MAX_HITS else sol(mp.mpf(20))
    return ([float(t) for t in times], [[float(c) for c in s] for s in states], float(t_end),
            [float(c) for c in y_end])


def manifold_task(args):
    """First crossing of x = 1 - mu (either direction) of the flipped field
    within tau in (0, 8]; the end state at tau = 8 if there is none."""
    y0, mu, tol = args
    import mpmath as mp
    sol, m = _solution(y0, mu, -1, tol)
    off = 1 - m
    t_prev = mp.mpf(0)
    g_prev = sol(t_prev)[0] - off
    n_scan = int(round(8.0 / SCAN))
    for k in range(1, n_scan + 1):
        t = mp.mpf(k) * mp.mpf(SCAN) if k < n_scan else mp.mpf(8)
        g = sol(t)[0] - off
        if (g_prev > 0) != (g > 0) or g == 0:
            tr = _root(sol, 0, off, t_prev, t)
            return True, float(tr), [float(c) for c in sol(tr)]
        t_prev, g_prev = t, g
    return False, 8.0, [float(c) for c in sol(mp.mpf(8))]


def _rel(a, b):
    """Largest row-wise relative distance (a vector is one row)."""
    a, b = np.atleast_2d(np.asarray(a, float)), np.atleast_2d(np.asarray(b, float))
    if not a.size:
        return 0.0
    return float(np.max(np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)))


def main():
    sys.path.insert(0, REPO)
    from hiten_gb300 import workloads as W
    mu = W.MU_EM
    d = np.load(os.path.join(HERE, "libm_spread.npz"))
    sec_y0, man_y0 = d["section_y0"][:N], d["manifold_y0"][:N]
    with ProcessPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        sec = list(ex.map(section_task, [(y, mu, TOL) for y in sec_y0]))
        sec_c = list(ex.map(section_task, [(y, mu, TOL_CHECK) for y in sec_y0]))
        man = list(ex.map(manifold_task, [(y, mu, TOL) for y in man_y0]))
        man_c = list(ex.map(manifold_task, [(y, mu, TOL_CHECK) for y in man_y0]))
    out = {"section_y0": sec_y0, "manifold_y0": man_y0}
    out["section_n_hits"] = np.array([len(r[0]) for r in sec], np.int32)
    out["section_hit_t"] = np.full((N, MAX_HITS), np.nan)
    out["section_hit_y"] = np.full((N, MAX_HITS, 6), np.nan)
    out["section_t_end"] = np.array([r[2] for r in sec])
    out["section_y_end"] = np.array([r[3] for r in sec])
    check = 0.0
    for i, (r, c) in enumerate(zip(sec, sec_c)):
        k = len(r[0])
        assert len(c[0]) == k, f"section {i}: crossing count changes with the tolerance"
        if k:
            out["section_hit_t"][i, :k] = r[0]
            out["section_hit_y"][i, :k] = r[1]
            check = max(check, _rel(np.array(r[0])[:, None], np.array(c[0])[:, None]), _rel(r[1], c[1]))
        check = max(check, _rel(r[3], c[3]))
    out["manifold_hit"] = np.array([r[0] for r in man], np.int32)
    out["manifold_t"] = np.array([r[1] for r in man])
    out["manifold_y"] = np.array([r[2] for r in man])
    for r, c in zip(man, man_c):
        assert r[0] == c[0]
        check = max(check, _rel([[r[1]]], [[c[1]]]), _rel(r[2], c[2]))
    out["check"] = np.array(check)
    out["note"] = json.dumps({"dps": DPS, "tol": f"1e-{TOL}", "check_tol": f"1e-{TOL_CHECK}", "scan": SCAN,
                              "source": "first N states of libm_spread.npz's section and manifold samples"})
    np.savez_compressed(os.path.join(HERE, "truth_mpmath.npz"), **out)
    print(f"wrote truth_mpmath.npz; largest relative change between tolerances {check:.2e}")


if __name__ == "__main__":
    main()
