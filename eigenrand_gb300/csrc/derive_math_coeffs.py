"""Derive the polynomial coefficients used by the library's own float log/exp.

The sampling kernels and the CPU oracle evaluate log/exp with the same
operation sequence (explicit fused multiply-adds), so their results agree bit
for bit.  The coefficients below are least-squares fits on Chebyshev nodes
(near-minimax), computed in 60-digit arithmetic and rounded to the working
precision.  Running this script prints the tables that are pasted into
``gr_math.cuh`` (device) and ``oracle/ormath.c`` (oracle).

Methods:
  logf : x = 2^e * m, m in [sqrt(1/2), sqrt(2)), f = m - 1,
         log(1+f) = f - f^2/2 + f^3 * P8(f)           (Cephes-style reduction)
  expf : n = rint(x*log2(e)), r = x - n*ln2 (Cody-Waite split),
         exp(r) = 1 + r + r^2 * P5(r)
The double-precision log/exp are table-driven; their tables come from
derive_math_tables.py.
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 60


def cheb_fit(func, a, b, deg, npts=400):
    xs = [mp.mpf(a) + (mp.mpf(b) - mp.mpf(a)) * (1 - mp.cos(mp.pi * (k + 0.5) / npts)) / 2 for k in range(npts)]
    A = mp.matrix(npts, deg + 1)
    y = mp.matrix(npts, 1)
    for i, x in enumerate(xs):
        fx = func(x)
        for j in range(deg + 1):
            A[i, j] = x ** j
        y[i] = fx
    # weighted to relative error of the final result is handled by caller choice of func
    coef = mp.lu_solve(A.T * A, A.T * y)
    return [coef[j] for j in range(deg + 1)]


def logf_coeffs():
    a, b = mp.sqrt(0.5) - 1, mp.sqrt(2) - 1
    g = lambda f: (mp.log1p(f) - f + f * f / 2) / f ** 3 if f != 0 else mp.mpf(1) / 3
    c = cheb_fit(g, a, b, 8)
    return [np.float32(float(v)) for v in c]


def expf_coeffs():
    h = mp.log(2) / 2
    g = lambda r: (mp.exp(r) - 1 - r) / r ** 2 if r != 0 else mp.mpf(1) / 2
    c = cheb_fit(g, -h, h, 5)
    return [np.float32(float(v)) for v in c]


if __name__ == "__main__":
    print("logf P8 (ascending powers):")
    for v in logf_coeffs():
        print("  %.9ef" % v)
    print("expf P5 (ascending powers):")
    for v in expf_coeffs():
        print("  %.9ef" % v)
    ln2 = mp.log(2)
    c1 = np.float32(0.693359375)        # 9 significant bits: n*c1 exact for |n| < 2^15
    c2 = np.float32(float(ln2 - mp.mpf(float(c1))))
    print("expf ln2 split: %.9ef %.9ef" % (c1, c2))
    print("log2(e) float %.9ef" % np.float32(float(1 / ln2)))
