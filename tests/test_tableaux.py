"""Tableau constants compiled into the kernels and the oracle are bit-identical
to the reference's coefficient arrays (tests/golden/tableaux.npz)."""
import os
import re

import numpy as np

from conftest import GOLDEN, REPO


def _parse(path, prefix):
    src = open(path).read()
    out = {}
    for m in re.finditer(r"double\s+" + prefix + r"(\w+)((?:\[\d+\])+)\s*=\s*\{(.*?)\};", src, flags=re.S):
        name, dims, body = m.group(1), m.group(2), m.group(3)
        shape = tuple(int(d) for d in re.findall(r"\[(\d+)\]", dims))
        vals = [float.fromhex(v) if ("0x" in v) else float(v)
                for v in re.findall(r"-?0x[0-9a-fA-F.]+p[+-]\d+|-?\d+\.\d+", body)]
        out[name] = np.array(vals).reshape(shape)
    return out


def test_kernel_and_oracle_tables_match_reference():
    ref = np.load(os.path.join(GOLDEN, "tableaux.npz"))
    for path, prefix in ((os.path.join(REPO, "hiten_gb300", "csrc", "hg_tableaux.h"), "HG_"),
                         (os.path.join(REPO, "oracle", "hgo_tableaux.h"), "HGO_")):
        t = _parse(path, prefix)
        for k in ref.files:
            if k == "DOP_META":
                continue
            assert k in t, (path, k)
            assert np.array_equal(t[k], ref[k]), (path, k)
