"""The oracle's section detection (PYTHON mode) reproduces the reference's
_SynodicDetectionBackend.detect_on_trajectory hits bit for bit, linear and
cubic interpolation, directional and any-direction planes."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = [(i, kind, name) for i in range(8) for kind in ("linear", "cubic") for name in ("y0dn", "xany")]
PLANES = {"y0dn": (1, -1, (0, 3)), "xany": (0, 0, (1, 4))}


@pytest.mark.parametrize("i,kind,name", CASES)
def test_section_detect_bit_exact(oracle, i, kind, name):
    s = np.load(os.path.join(GOLDEN, "section.npz"))
    oracle.set_mode(oracle.MODE_PYTHON)
    axis, d, plane = PLANES[name]
    ht, hy = oracle.section_detect(s[f"{i}/times"], s[f"{i}/states"], axis, float(s[f"{i}/{kind}_{name}_off"]), d,
                                   plane, cubic=(kind == "cubic"))
    assert np.array_equal(ht, s[f"{i}/{kind}_{name}_t"])
    assert np.array_equal(hy, s[f"{i}/{kind}_{name}_y"])
