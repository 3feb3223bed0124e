"""Derive the tables of the library's table-driven double-precision exp / log.

Methods (published; restated, not copied):
  exp  P. T. P. Tang, "Table-driven implementation of the exponential function
       in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989:
       x = (64 m + j) ln2/64 + r,  exp(x) = 2^m * 2^(j/64) * exp(r),
       |r| <= ln2/128, exp(r) - 1 by its Taylor series to degree 6.
  log  P. T. P. Tang, "Table-driven implementation of the logarithm function
       in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990 (with the
       reduction by a tabulated reciprocal, r = m * invc - 1 in one fused
       multiply-add): x = 2^e m, m in [1, 2), bucket i = top 7 fraction bits,
       log(x) = e ln2 + log(1/invc_i) + log1p(r), |r| <= 2^-7,
       log1p(r) = r - r^2/2 + r^3 Q(r), Q the Taylor series to degree 6.
       Buckets 0 and 127 use invc = 1 and 1/2, so x next to 1 reduces to
       log1p(x - 1) exactly, with no cancellation.  e ln2 and log(1/invc_i)
       are split into a high part on the 2^-42 grid (their sum is exact) and
       a low part.

Running the script writes the same tables to eigenrand_gb300/csrc/gr_math_tables.h
(device) and oracle/ormath_tables.h (oracle):

    python eigenrand_gb300/csrc/derive_math_tables.py
"""
import os

import mpmath as mp

mp.mp.dps = 80
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def to_double(x):
    return float(mp.mpf(x))  # round to nearest


def hexf(x):
    return float(x).hex()


def on_grid(x, q):
    """x rounded to a multiple of 2^-q."""
    s = mp.mpf(2) ** q
    return float(mp.nint(mp.mpf(x) * s) / s)


def tables():
    ln2 = mp.log(2)
    out = {}
    # ---- exp
    out["EXP_INV_L"] = to_double(64 / ln2)
    l = ln2 / 64
    lh = to_double(l)
    out["EXP_L_HI"] = lh
    out["EXP_L_LO"] = to_double(l - mp.mpf(lh))
    th, tl = [], []
    for j in range(64):
        t = mp.mpf(2) ** (mp.mpf(j) / 64)
        h = to_double(t)
        th.append(h)
        tl.append(to_double(t - mp.mpf(h)))
    out["EXP_T_HI"], out["EXP_T_LO"] = th, tl
    out["EXP_C"] = [to_double(1 / mp.factorial(k)) for k in range(2, 7)]  # 1/2! .. 1/6!
    # ---- log
    ln2h = on_grid(ln2, 42)
    out["LOG_LN2_HI"] = ln2h
    out["LOG_LN2_LO"] = to_double(ln2 - mp.mpf(ln2h))
    invc, lch, lcl = [], [], []
    for i in range(128):
        if i == 0:
            ic = 1.0
        elif i == 127:
            ic = 0.5
        else:
            c = 1 + (mp.mpf(i) + mp.mpf("0.5")) / 128
            ic = float(mp.nint((1 / c) * mp.mpf(2) ** 40) / mp.mpf(2) ** 40)  # 1/c on the 2^-40 grid
        lc = -mp.log(mp.mpf(ic))
        h = on_grid(lc, 42) if i != 127 else ln2h
        invc.append(ic)
        lch.append(h)
        lcl.append(to_double(lc - mp.mpf(h)) if i != 127 else out["LOG_LN2_LO"])
    out["LOG_INVC"], out["LOG_C_HI"], out["LOG_C_LO"] = invc, lch, lcl
    # Q(r) = 1/3 - r/4 + r^2/5 - ... - r^5/8 + r^6/9
    out["LOG_Q"] = [to_double(mp.mpf((-1) ** k) / (k + 3)) for k in range(7)]
    return out


def emit(t, guard, prefix_comment):
    lines = [f"/* {prefix_comment}", " * Generated by eigenrand_gb300/csrc/derive_math_tables.py; do not edit. */",
             f"#ifndef {guard}", f"#define {guard}", ""]

    def scalar(name):
        lines.append(f"#define GRT_{name} {hexf(t[name])}")

    def array(name, attr):
        vals = t[name]
        lines.append(f"{attr}const double GRT_{name}[{len(vals)}] = {{")
        for i in range(0, len(vals), 4):
            lines.append("    " + ", ".join(hexf(v) for v in vals[i:i + 4]) + ",")
        lines.append("};")

    for s in ("EXP_INV_L", "EXP_L_HI", "EXP_L_LO", "LOG_LN2_HI", "LOG_LN2_LO"):
        scalar(s)
    for k, v in enumerate(t["EXP_C"]):
        lines.append(f"#define GRT_EXP_C{k + 2} {hexf(v)}")
    for k, v in enumerate(t["LOG_Q"]):
        lines.append(f"#define GRT_LOG_Q{k} {hexf(v)}")
    lines.append("")
    lines.append("#ifdef __CUDACC__")
    lines.append("#define GRT_TABLE __device__ static")
    lines.append("#else")
    lines.append("#define GRT_TABLE static")
    lines.append("#endif")
    for a in ("EXP_T_HI", "EXP_T_LO", "LOG_INVC", "LOG_C_HI", "LOG_C_LO"):
        array(a, "GRT_TABLE ")
    lines.append("")
    lines.append(f"#endif  /* {guard} */")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    t = tables()
    with open(os.path.join(HERE, "gr_math_tables.h"), "w") as f:
        f.write(emit(t, "GR_MATH_TABLES_H", "Tables of the table-driven double exp / log (device)."))
    with open(os.path.join(ROOT, "oracle", "ormath_tables.h"), "w") as f:
        f.write(emit(t, "ORMATH_TABLES_H", "ORACLE - tables of the table-driven double exp / log."))
    print("written")
