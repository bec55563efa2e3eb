"""Emit the lookup tables of the correctly rounded power function
(``hg_crmath.cuh``) as exact hex-float literals, computed with mpmath at
200-bit precision:

* log table: for F_j = 1 + j/1024, j in [LOG_JMIN, LOG_JMAX]:
  RN(1/F_j) and log(F_j) as a double-double (hi, lo);
* exp table: 2^(j/256), j in [0, 256), as a double-double (hi, lo);
* ln 2 split for the exponent term and ln2/256 split for argument reduction.

Usage: ``python hiten_gb300/csrc/gen_crmath_tables.py`` (needs mpmath).
"""
import os

import mpmath as mp

mp.mp.prec = 200
HERE = os.path.dirname(os.path.abspath(__file__))
LOG_JMIN, LOG_JMAX = -304, 428


def dd(v):
    hi = float(v)
    lo = float(v - mp.mpf(hi))
    return hi, lo


def trunc_bits(v, bits):
    """v rounded toward zero to `bits` significant bits (as a double)."""
    m, e = mp.frexp(v)
    scale = mp.mpf(2) ** bits
    return float(mp.floor(abs(m) * scale) / scale * mp.sign(m) * mp.mpf(2) ** e)


def h(x):
    return float.hex(float(x))


def main():
    out = ["/* Generated by hiten_gb300/csrc/gen_crmath_tables.py (mpmath, 200 bits). */\n",
           "#ifndef HG_CRMATH_TABLES_H\n#define HG_CRMATH_TABLES_H\n\n",
           f"#define HG_LOG_JMIN ({LOG_JMIN})\n#define HG_LOG_JMAX ({LOG_JMAX})\n",
           f"#define HG_LOG_N ({LOG_JMAX - LOG_JMIN + 1})\n\n"]
    inv, lh, ll = [], [], []
    for j in range(LOG_JMIN, LOG_JMAX + 1):
        F = mp.mpf(1) + mp.mpf(j) / 1024
        inv.append(float(1 / F))
        a, b = dd(mp.log(F))
        lh.append(a)
        ll.append(b)
    eh, el = [], []
    for j in range(256):
        a, b = dd(mp.power(2, mp.mpf(j) / 256))
        eh.append(a)
        el.append(b)

    def arr(name, vals):
        body = ",\n  ".join(", ".join(h(v) for v in vals[i:i + 4]) for i in range(0, len(vals), 4))
        return f"#define {name}_INIT {{ \\\n  " + body.replace("\n", " \\\n") + " }\n\n"

    out.append(arr("HG_LOG_INVF", inv))
    out.append(arr("HG_LOG_TH", lh))
    out.append(arr("HG_LOG_TL", ll))
    out.append(arr("HG_EXP_TH", eh))
    out.append(arr("HG_EXP_TL", el))
    ln2 = mp.log(2)
    l2hi = trunc_bits(ln2, 40)
    l2lo = float(ln2 - mp.mpf(l2hi))
    out.append(f"#define HG_LN2_HI {h(l2hi)}\n#define HG_LN2_LO {h(l2lo)}\n")
    c = ln2 / 256
    c1 = trunc_bits(c, 38)
    c2 = trunc_bits(c - mp.mpf(c1), 38)
    c3 = float(c - mp.mpf(c1) - mp.mpf(c2))
    out.append(f"#define HG_L256_1 {h(c1)}\n#define HG_L256_2 {h(c2)}\n#define HG_L256_3 {h(c3)}\n")
    out.append(f"#define HG_INV_L256 {h(256 / ln2)}\n")
    out.append("\n#endif\n")
    with open(os.path.join(HERE, "hg_crmath_tables.h"), "w") as f:
        f.write("".join(out))


if __name__ == "__main__":
    main()
