"""The FP32 screen of the connection searches (csrc/hg_connect.cu), checked
in exact rational arithmetic on the host: the FP32 distance d2_f of every pair
(float32 operations rounded to nearest, as the kernels' __fmul_rn/__fadd_rn)
stays within the stated bound e of the exact distance, and the nearest-
neighbour threshold built from the pass-0 minimum D admits every exact
minimiser (evaluated here without rounding; the kernel rounds each term
upward, so its threshold is at least this one)."""
import math
from fractions import Fraction as Fr

import numpy as np
import pytest

U = Fr(1, 2 ** 24)


def _f32_up(x):
    """The smallest float32 >= x (x a Fraction)."""
    f = np.float32(float(x))
    while Fr(float(f)) < x:
        f = np.nextafter(f, np.float32(np.inf))
    return f


def _clouds():
    rng = np.random.default_rng(17)
    yield rng.uniform(-0.4, 0.4, (120, 2))
    c = rng.uniform(-0.3, 0.3, (20, 2))  # micro-clusters below FP32 resolution
    yield np.concatenate([c + rng.normal(0, 1e-9, c.shape), c + rng.normal(0, 1e-12, c.shape),
                          rng.uniform(-0.3, 0.3, (60, 2))])
    yield rng.uniform(-3e3, 3e3, (100, 2))  # large coordinates
    g = np.stack(np.meshgrid(np.arange(10) / 64.0, np.arange(10) / 64.0), -1).reshape(-1, 2) - 0.07
    yield g  # exact ties


def _sqrt_up(x):
    """An upper bound of sqrt(x) for a non-negative Fraction."""
    s = Fr(math.sqrt(float(x)))
    while s * s < x:
        s *= 1 + Fr(1, 2 ** 50)
    return s


@pytest.mark.parametrize("k", range(4))
def test_fp32_screen_bound_and_nearest_threshold(k):
    p = list(_clouds())[k]
    n = len(p)
    coord_max = float(np.abs(p).max())
    R = Fr(float(np.nextafter(np.float32(coord_max), np.float32(np.inf))))
    R2c = Fr(float(_f32_up(Fr(2) ** -43 * Fr(coord_max) ** 2)))
    pf = p.astype(np.float32)
    ex = [(Fr(a), Fr(b)) for a, b in p]
    for i in range(n):
        dxf = (pf[i, 0] - pf[:, 0]).astype(np.float32)
        dyf = (pf[i, 1] - pf[:, 1]).astype(np.float32)
        d2f = (dxf * dxf).astype(np.float32) + (dyf * dyf).astype(np.float32)
        assert d2f.dtype == np.float32
        d2 = [(ex[i][0] - ex[j][0]) ** 2 + (ex[i][1] - ex[j][1]) ** 2 for j in range(n)]
        # the stated bound for every pair
        for j in range(n):
            e = Fr(2) ** -20 * (Fr(float(d2f[j])) + R * (abs(Fr(float(dxf[j]))) + abs(Fr(float(dyf[j]))))) + R2c
            assert abs(Fr(float(d2f[j])) - d2[j]) <= e, (i, j)
        # the nearest-neighbour threshold from the pass-0 minimum
        others = [j for j in range(n) if j != i]
        D = min(Fr(float(d2f[j])) for j in others)
        c1 = Fr(2) ** -20 * R * Fr(14142135623730952, 10 ** 16) / (1 - U)  # sqrt2 rounded up
        c0 = Fr(2) ** -82 * R + R2c
        M = D + Fr(2) ** -20 * D + c1 * _sqrt_up(D) + c0
        a = 1 - Fr(2) ** -20
        smax = (c1 + _sqrt_up(c1 * c1 + 4 * a * (c0 + M))) / (2 * a)
        thr = smax * smax
        dmin = min(d2[j] for j in others)
        for j in others:
            if d2[j] == dmin:
                assert Fr(float(d2f[j])) <= thr, (i, j)
