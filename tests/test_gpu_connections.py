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
