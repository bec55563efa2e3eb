"""Connections on the GPU: the reference's own results bit for bit
(tests/golden/connections.npz), and the FP32-screened all-pairs kernels equal
to the FP64 oracle on large clouds built to stress the screen: pairs within
an ulp of the radius, duplicate points, exact distance ties."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_connections_cpu import _check

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("c", [0, 1, 2, 3])
def test_gpu_connections_reproduce_reference(gpu, c):
    from hiten_gb300.connections import find_connections
    g = np.load(os.path.join(GOLDEN, "connections.npz"))
    eps, dvt, bt = g[f"{c}/params"]
    res, meta = find_connections(g[f"{c}/pu"], g[f"{c}/ps"], g[f"{c}/Xu"], g[f"{c}/Xs"], g[f"{c}/tu"],
                                 g[f"{c}/ts"], eps=eps, dv_tol=dvt, bal_tol=bt)
    _check(res, meta, g, c)


def _cloud(seed, n, m, eps):
    rng = np.random.default_rng(seed)
    pu = rng.uniform(-0.4, 0.4, (n, 2))
    ps = rng.uniform(-0.4, 0.4, (m, 2))
    k = min(n, m) // 4
    ang = rng.uniform(0, 2 * np.pi, k)
    # partners at distance eps * (1 +- a few ulps): decided by the last bits
    f = 1.0 + rng.integers(-4, 5, k) * 2.0 ** -52
    ps[:k, 0] = pu[:k, 0] + eps * f * np.cos(ang)
    ps[:k, 1] = pu[:k, 1] + eps * f * np.sin(ang)
    if min(n, m) >= 1000:
        # duplicates and exact ties (grid-aligned points)
        pu[k:k + 50] = pu[k + 50:k + 100]
        g = np.round(rng.uniform(-0.4, 0.4, (200, 2)) * 1024) / 1024
        pu[k + 100:k + 300] = g
        ps[k:k + 200] = g + np.array([eps / 2, 0.0])
    return pu, ps


@pytest.mark.parametrize("seed,n,m,eps", [(0, 20000, 18000, 1e-3), (1, 5000, 7000, 3e-2), (2, 3, 2, 1.0)])
def test_gpu_matcher_equals_fp64_oracle(gpu, seed, n, m, eps):
    from hiten_gb300.connections import GpuSectionMatcher
    from oracle.connect import OracleSectionMatcher
    pu, ps = _cloud(seed, n, m, eps)
    R = float(max(np.abs(pu).max(), np.abs(ps).max()))
    G, O = GpuSectionMatcher(), OracleSectionMatcher()
    for q, r in ((pu, ps), (ps, pu)):
        a, b = G.radius_best(q, r, eps, R), O.radius_best(q, r, eps, R)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    for p in (pu, ps):
        assert np.array_equal(G.nearest(p, R), O.nearest(p, R))


def _structured(kind):
    rng = np.random.default_rng(11)
    if kind == "grid":
        # a regular grid: every interior point has four neighbours at exactly
        # the same distance (the lowest index must win), shuffled order
        g = np.stack(np.meshgrid(np.arange(64) / 256.0, np.arange(48) / 256.0), -1).reshape(-1, 2) - 0.1
        return g[rng.permutation(g.shape[0])]
    if kind == "cluster":
        # micro-clusters below FP32 resolution of the coordinates (their FP32
        # distances collapse to 0) inside a wide cloud
        c = rng.uniform(-0.3, 0.3, (300, 2))
        pts = [c + rng.normal(0, 10.0 ** -e, c.shape) for e in (9, 11, 13)]
        return np.concatenate([rng.uniform(-0.3, 0.3, (3000, 2))] + pts)
    if kind == "large":
        # large coordinates: the FP32 screen's absolute error terms dominate
        return rng.uniform(-2e3, 2e3, (4000, 2)) * np.exp(rng.normal(0, 2, (4000, 1))) * 1e-3
    return rng.uniform(-1, 1, (int(kind), 2))


@pytest.mark.parametrize("kind", ["1", "2", "33", "grid", "cluster", "large"])
def test_gpu_nearest_structured_equals_fp64_oracle(gpu, kind):
    from hiten_gb300.connections import GpuSectionMatcher
    from oracle.connect import OracleSectionMatcher
    p = _structured(kind)
    R = float(np.abs(p).max())
    G, O = GpuSectionMatcher(), OracleSectionMatcher()
    assert np.array_equal(G.nearest(p, R), O.nearest(p, R))
    q = p[::-1].copy()
    eps = float(np.median(np.abs(np.diff(p[:, 0])))) if p.shape[0] > 1 else 0.5
    for a, b in zip(G.radius_best(p, q, eps, R), O.radius_best(p, q, eps, R)):
        assert np.array_equal(a, b)


def test_gpu_refinement_equals_host_arithmetic(gpu):
    """hg_connection_refine gives the numpy refinement's bits: the same cloud
    through the GPU matcher with and without its refine step (a wrapper that
    hides it sends find_connections down the numpy path)."""
    from hiten_gb300.connections import GpuSectionMatcher, find_connections
    rng = np.random.default_rng(21)
    n = 20000

    def curve(ph):
        s = rng.uniform(0, 1, n)
        return np.c_[0.1 * np.cos(2 * np.pi * s + ph) + rng.normal(0, 1e-4, n),
                     0.3 * np.sin(2 * np.pi * s + ph) + rng.normal(0, 1e-4, n)]

    pu, ps = curve(0.0), curve(0.3)
    Xu = np.c_[pu[:, :1] * 0 + 0.85, pu[:, 0], rng.normal(0, 1e-3, n), rng.normal(0, 1e-3, n), pu[:, 1],
               rng.normal(0, 1e-3, n)]
    Xs = np.c_[ps[:, :1] * 0 + 0.85, ps[:, 0], rng.normal(0, 1e-3, n), rng.normal(0, 1e-3, n), ps[:, 1],
               rng.normal(0, 1e-3, n)]
    g = GpuSectionMatcher()

    class SearchOnly:
        radius_best = g.radius_best
        nearest = g.nearest

    kw = dict(eps=3e-4, dv_tol=1e-2, bal_tol=1e-4, max_seg_len=1e-4)  # some segments too long: both branches
    a, ma = find_connections(pu, ps, Xu, Xs, matcher=g, **kw)
    b, mb = find_connections(pu, ps, Xu, Xs, matcher=SearchOnly(), **kw)
    assert ma == mb and len(a) == len(b) > 1000
    for x, y in zip(a, b):
        assert (x.kind, x.delta_v, x.point2d, x.index_u, x.index_s) == (y.kind, y.delta_v, y.point2d, y.index_u,
                                                                         y.index_s)
        assert np.array_equal(x.state_u, y.state_u) and np.array_equal(x.state_s, y.state_s)
