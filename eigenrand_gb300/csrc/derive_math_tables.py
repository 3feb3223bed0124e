"""Derive the tables of the library's integer-arithmetic double exp / log.

Both reduce in fixed point, evaluate a short series in Q62 and round once to
double (method notes in int_tables below and in gr_dmath.h):
  log  two reciprocal reductions (7-bit bucket, then a 2^-14 bucket of the
       remainder) to |r| < 2^-15 + 2^-21, log1p(r) = r S(r) with S the Taylor
       series to degree 4, table values in Q116;
  exp  Tang's reduction x = (64 m + j) ln2/64 + r (P. T. P. Tang, ACM TOMS
       15(2), 1989) with r exact in Q100, exp(r) by its Taylor series to
       degree 7, 2^(j/64) in Q63.

Running the script writes the same tables to eigenrand_gb300/csrc/gr_math_tables.h
(device) and oracle/ormath_tables.h (oracle):

    python eigenrand_gb300/csrc/derive_math_tables.py
"""
import os

import mpmath as mp

mp.mp.dps = 80
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def fixed(x, q):
    """Nearest integer to x * 2^q (mpmath value)."""
    return int(mp.nint(mp.mpf(x) * mp.mpf(2) ** q))


def int_tables():
    """Fixed-point tables of the integer-arithmetic double log / exp.

    log: x = 2^e m, M = m 2^52.  Stage 1: bucket i = top 7 fraction bits,
    K1_i ~ 256 / c_i (K1_0 = 256, K1_127 = 128, e + 1 absorbed by
    L1_127 = ln 2), y1 = M K1 = (1 + r1) 2^60 exactly.  Stage 2: bucket
    j = floor((r1 + 2^-15) 2^14) + J0, K2_j ~ 2^20 / (1 + (j - J0) 2^-14)
    (2^20 exactly for the bucket around 0, so x near 1 keeps r exact),
    y2 = y1 K2 = (1 + r2) 2^80 with |r2| < 2^-15 + 2^-21.
    log x = e ln2 + L1_i + L2_j + r2 S(r2), S = 1 - r/2 + r^2/3 - r^3/4 + r^4/5,
    everything summed in Q116 (int128).
    exp: n = round(64 x / ln2), r = x - n ln2/64 (Q100), exp(r) by its
    Taylor series to degree 7 in Q62, times T_j = 2^(j/64) in Q63."""
    t = {}
    ln2 = mp.log(2)
    K1 = []
    for i in range(128):
        if i == 0:
            k = 256
        elif i == 127:
            k = 128
        else:
            k = int(mp.nint(256 / (1 + (mp.mpf(i) + mp.mpf("0.5")) / 128)))
        K1.append(k)
    # range of r1 over every bucket (both ends), then the stage-2 buckets
    rmin, rmax = mp.mpf(0), mp.mpf(0)
    for i in range(128):
        lo = 1 + mp.mpf(i) / 128
        hi = 1 + mp.mpf(i + 1) / 128
        for m in (lo, hi):
            r = m * K1[i] / 256 - 1 if i != 127 else m * mp.mpf(K1[i]) / 256 - 1
            rmin, rmax = min(rmin, r), max(rmax, r)
    J0 = -int(mp.floor((rmin + mp.mpf(2) ** -15) * 2 ** 14))
    JN = int(mp.floor((rmax + mp.mpf(2) ** -15) * 2 ** 14)) + J0 + 1
    K2, L2 = [], []
    for j in range(JN):
        c = mp.mpf(j - J0) * mp.mpf(2) ** -14
        k = 1 << 20 if j == J0 else int(mp.nint(mp.mpf(2) ** 20 / (1 + c)))
        K2.append(k)
        L2.append(fixed(-mp.log(mp.mpf(k) / mp.mpf(2) ** 20), 116))
    L1 = [fixed(-mp.log(mp.mpf(k) / 256), 116) for k in K1]
    L1[127] = fixed(ln2, 116)  # cancels e * ln2 exactly for x just below 1
    t["ILOG_K1"], t["ILOG_L1"], t["ILOG_K2"], t["ILOG_L2"] = K1, L1, K2, L2
    t["ILOG_J0"], t["ILOG_JN"] = J0, JN
    t["ILOG_LN2"] = fixed(ln2, 116)
    t["ILOG_S"] = [fixed(mp.mpf(1) / 5, 62), -(1 << 60), fixed(mp.mpf(1) / 3, 62), -(1 << 61), 1 << 62]
    # exp
    t["IEXP_T"] = [fixed(mp.mpf(2) ** (mp.mpf(j) / 64), 63) for j in range(64)]
    t["IEXP_LN2_64"] = fixed(ln2 / 64, 100)
    t["IEXP_INVL"] = fixed(64 / ln2, 20)
    t["IEXP_C"] = [fixed(1 / mp.factorial(k), 62) for k in range(7, -1, -1)]  # 1/7! .. 1/0!
    return t


def emit(t, guard, prefix_comment):
    lines = [f"/* {prefix_comment}", " * Generated by eigenrand_gb300/csrc/derive_math_tables.py; do not edit. */",
             f"#ifndef {guard}", f"#define {guard}", "", "#include <stdint.h>", ""]

    lines.append("#ifdef __CUDACC__")
    lines.append("#define GRT_TABLE __device__ static")
    lines.append("#else")
    lines.append("#define GRT_TABLE static")
    lines.append("#endif")

    # integer tables: 128-bit values as (high, low) 64-bit halves, two's complement
    def i128(v):
        v &= (1 << 128) - 1
        return v >> 64, v & ((1 << 64) - 1)

    def u64(v):
        return f"0x{v & ((1 << 64) - 1):016x}ull"

    lines.append("")
    lines.append(f"#define GRT_ILOG_J0 {t['ILOG_J0']}")
    lines.append(f"#define GRT_ILOG_JN {t['ILOG_JN']}")
    h, l = i128(t["ILOG_LN2"])
    lines.append(f"#define GRT_ILOG_LN2_HI {u64(h)}")
    lines.append(f"#define GRT_ILOG_LN2_LO {u64(l)}")
    h, l = i128(t["IEXP_LN2_64"])
    lines.append(f"#define GRT_IEXP_LN2_64_HI {u64(h)}")
    lines.append(f"#define GRT_IEXP_LN2_64_LO {u64(l)}")
    lines.append(f"#define GRT_IEXP_INVL {t['IEXP_INVL']}ll")
    for k, v in enumerate(t["ILOG_S"]):
        lines.append(f"#define GRT_ILOG_S{k} ((int64_t){u64(v)})")
    for k, v in enumerate(t["IEXP_C"]):
        lines.append(f"#define GRT_IEXP_C{k} ((int64_t){u64(v)})")

    def iarr(name, vals, ctype):
        lines.append(f"GRT_TABLE const {ctype} GRT_{name}[{len(vals)}] = {{")
        for i in range(0, len(vals), 4):
            lines.append("    " + ", ".join(vals[i:i + 4]) + ",")
        lines.append("};")

    iarr("ILOG_K1", [str(v) for v in t["ILOG_K1"]], "uint32_t")
    iarr("ILOG_K2", [str(v) for v in t["ILOG_K2"]], "uint32_t")
    iarr("ILOG_L1", [u64(x) for v in t["ILOG_L1"] for x in i128(v)], "uint64_t")  # hi, lo per entry
    iarr("ILOG_L2", [u64(x) for v in t["ILOG_L2"] for x in i128(v)], "uint64_t")
    iarr("IEXP_T", [u64(v) for v in t["IEXP_T"]], "uint64_t")
    lines.append("")
    lines.append(f"#endif  /* {guard} */")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    t = int_tables()
    with open(os.path.join(HERE, "gr_math_tables.h"), "w") as f:
        f.write(emit(t, "GR_MATH_TABLES_H", "Tables of the integer-arithmetic double exp / log (device)."))
    with open(os.path.join(ROOT, "oracle", "ormath_tables.h"), "w") as f:
        f.write(emit(t, "ORMATH_TABLES_H", "ORACLE - tables of the integer-arithmetic double exp / log."))
    print("written")
