"""Emit the Runge-Kutta tableau constants as exact hex-float C literals.

The fixed-step (classical RK4, the 7-stage 6th-order scheme, the 13-stage
8th-order Prince-Dormand weights) and the adaptive Dormand-Prince 8(5,3)
coefficients must be bit-identical to the reference's
(``integrators/coefficients/{rk4,rk6,rk8,dop853}.py``) for results to
match, so they are read from those modules and written out with ``%a``
formatting, which round-trips every double exactly.

Outputs (all committed; regenerate only when the reference tree is present):

* ``hiten_gb300/csrc/hg_tableaux.h`` -- constexpr tables for the kernels;
* ``oracle/hgo_tableaux.h``          -- the same values for the CPU oracle;
* ``tests/golden/tableaux.npz``      -- the reference arrays, for tests.

Usage: ``python hiten_gb300/csrc/gen_tableaux.py /path/to/reference/src``
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _load(src, name):
    path = os.path.join(src, "hiten", "algorithms", "integrators", "coefficients", name + ".py")
    spec = importlib.util.spec_from_file_location("_coef_" + name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _hex(v):
    v = float(v)
    if v == 0.0:
        return "0.0"
    return float.hex(v)


def _arr1(name, a, qual):
    vals = ", ".join(_hex(v) for v in a)
    return f"{qual} double {name}[{len(a)}] = {{{vals}}};\n"


def _arr2(name, a, qual):
    rows = []
    for r in a:
        rows.append("  {" + ", ".join(_hex(v) for v in r) + "}")
    return f"{qual} double {name}[{a.shape[0]}][{a.shape[1]}] = {{\n" + ",\n".join(rows) + "\n};\n"


def tables(src):
    rk4 = _load(src, "rk4")
    rk6 = _load(src, "rk6")
    rk8 = _load(src, "rk8")
    dp = _load(src, "dop853")
    return {
        "RK4_A": rk4.A, "RK4_B": rk4.B, "RK4_C": rk4.C,
        "RK6_A": rk6.A, "RK6_B": rk6.B, "RK6_C": rk6.C,
        "RK8_A": rk8.A, "RK8_B": rk8.B, "RK8_C": rk8.C,
        "DOP_A": dp.A, "DOP_B": dp.B, "DOP_C": dp.C,
        "DOP_E3": dp.E3, "DOP_E5": dp.E5, "DOP_D": dp.D,
        "DOP_META": np.array([dp.N_STAGES, dp.N_STAGES_EXTENDED, dp.INTERPOLATOR_POWER], dtype=np.int64),
    }


def emit(t, guard, qual, prefix, header_note):
    out = [header_note, f"#ifndef {guard}\n#define {guard}\n\n"]
    meta = t["DOP_META"]
    out.append(f"#define {prefix}DOP_N_STAGES {int(meta[0])}\n")
    out.append(f"#define {prefix}DOP_N_STAGES_EXT {int(meta[1])}\n")
    out.append(f"#define {prefix}DOP_INTERP_POWER {int(meta[2])}\n\n")
    for k, v in t.items():
        if k == "DOP_META":
            continue
        v = np.asarray(v, dtype=np.float64)
        nm = prefix + k
        out.append(_arr2(nm, v, qual) if v.ndim == 2 else _arr1(nm, v, qual))
        out.append("\n")
    out.append(f"#endif  /* {guard} */\n")
    return "".join(out)


def main(src):
    t = tables(src)
    note = ("/* Generated by hiten_gb300/csrc/gen_tableaux.py: Runge-Kutta tableaux as exact\n"
            " * hex-float literals (classical RK4; 7-stage RK6; Prince-Dormand 13-stage RK8;\n"
            " * Dormand-Prince 8(5,3) with its 4-stage dense-output extension).\n"
            " * Values are identical to integrators/coefficients/{rk4,rk6,rk8,dop853}.py. */\n")
    with open(os.path.join(HERE, "hg_tableaux.h"), "w") as f:
        f.write(emit(t, "HG_TABLEAUX_H", "static constexpr", "HG_", note))
    with open(os.path.join(REPO, "oracle", "hgo_tableaux.h"), "w") as f:
        f.write(emit(t, "HGO_TABLEAUX_H", "static const", "HGO_", note))
    np.savez(os.path.join(REPO, "tests", "golden", "tableaux.npz"), **{k: np.asarray(v) for k, v in t.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path to the hiten source tree, the directory holding hiten/>")
    main(sys.argv[1])
