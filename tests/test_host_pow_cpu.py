"""hg_host_pow (the library's host loop over C pow) returns the bits of the
C pow the reference's numpy-scalar `**` calls (CPython's math.pow is that
call), for the exponents of the halo quadratic term and the step-size
controller, through the Python corrector's _libm_pow."""
import math

import numpy as np

from hiten_gb300 import corrector as Cr


def test_host_pow_matches_c_pow():
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(1e-6, 10.0, 20000), 10.0 ** rng.uniform(-30, 3, 20000)])
    for e in (2, 1.5, 2.5, -1.0 / 9.0, 0.4 / 9.0, -0.125):
        got = Cr._libm_pow(x, e)
        ref = np.array([math.pow(v, e) for v in x])
        assert np.array_equal(got, ref), e
    assert Cr._libm_pow(np.zeros((0,)), 2.0).shape == (0,)
    assert Cr._libm_pow(np.full((3, 2), 3.0), 2).shape == (3, 2)
