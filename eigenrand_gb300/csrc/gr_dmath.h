// Double-precision log and exp in integer arithmetic.
//
// The FP64 pipe of this part issues 2 thread-operations per clock per SM;
// the integer pipes issue dozens.  These functions reduce, evaluate and sum
// in fixed point (64- and 128-bit integers) and round once to double, so a
// call costs no FP64 instruction.  Maximum error (measured against 40-digit
// references): about 0.501 ulp for both; exp is exact at 0 and log at 1.
//
// log: x = 2^e m, M = m 2^52.  Stage 1 takes bucket i from the top 7
// fraction bits and an 8-bit reciprocal K1_i: y1 = M K1_i = (1 + r1) 2^60
// exactly.  Stage 2 takes bucket j of r1 (width 2^-14, the one around 0
// exact) and a 21-bit reciprocal K2_j: y2 = y1 K2_j = (1 + r2) 2^80 exactly,
// |r2| < 2^-15 + 2^-21.  Then log x = e ln2 + L1_i + L2_j + r2 S(r2) with
// S(r) = 1 - r/2 + r^2/3 - r^3/4 + r^4/5 (truncation below 2^-77 relative),
// S in Q62, the sum in Q116 (128-bit).  Near 1 the tables contribute exactly
// 0 and r2 is exact, so small results keep their relative precision.
//
// exp: n = round(64 x / ln2) (estimated from the top bits of x; an estimate
// one off only widens |r| slightly), r = x - n ln2/64 exactly in Q100,
// exp(r) by its Taylor series to degree 7 in Q62 (|r| < 0.0055), times
// 2^(j/64) in Q63 (j = n mod 64), scaled by 2^(n div 64) and rounded once,
// subnormal results included.
//
// Tables and coefficients: derive_math_tables.py (mpmath), emitted to
// gr_math_tables.h.  The header compiles for the host as well, so the same
// code is checked on the CPU.
#pragma once
#include <stdint.h>
#include <string.h>

#include "gr_math_tables.h"

#ifdef __CUDACC__
#define GRD_HD __host__ __device__ __forceinline__
#else
#define GRD_HD static inline
#endif

#ifdef __CUDA_ARCH__
#define GRD_LD(x) __ldg(&(x))
#else
#define GRD_LD(x) (x)
#endif

namespace gr {

typedef unsigned __int128 grd_u128;
typedef __int128 grd_i128;

GRD_HD uint64_t grd_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

GRD_HD double grd_double(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

GRD_HD int grd_clz64(uint64_t x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// high 64 bits of the signed 128-bit product
GRD_HD int64_t grd_mulhi(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (int64_t)(((grd_i128)a * b) >> 64);
#endif
}

GRD_HD grd_u128 grd_u128_of(uint64_t hi, uint64_t lo) { return ((grd_u128)hi << 64) | lo; }

GRD_HD uint64_t grd_umulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((grd_u128)a * b) >> 64);
#endif
}

// k (hi:lo) for a small signed k (|k| < 2^20), modulo 2^128: two 64-bit
// products instead of a general 128-bit one
GRD_HD grd_i128 grd_mul_small(int64_t k, uint64_t hi, uint64_t lo) {
  const uint64_t a = (uint64_t)(k < 0 ? -k : k);
  const uint64_t rl = a * lo;
  const uint64_t rh = grd_umulhi(a, lo) + a * hi;
  const grd_u128 r = grd_u128_of(rh, rl);
  return k < 0 ? -(grd_i128)r : (grd_i128)r;
}

// Round a normalized magnitude h:l (leading bit at 127) to 53 bits, nearest
// even, with binary exponent E of the leading bit; E within the normal range.
GRD_HD double grd_round_norm(uint64_t h, uint64_t l, int E, int neg) {
  uint64_t sig = h >> 11;  // 53 bits
  const uint64_t rest = h & 0x7ffull;
  if ((rest > 0x400ull) || (rest == 0x400ull && (l != 0 || (sig & 1)))) ++sig;
  if (sig >> 53) {
    sig >>= 1;
    ++E;
  }
  if (E > 1023) return grd_double(((uint64_t)neg << 63) | 0x7ff0000000000000ull);
  return grd_double(((uint64_t)neg << 63) | ((uint64_t)(E + 1023) << 52) | (sig & 0xfffffffffffffull));
}

// leading-bit normalization of A > 0: h:l = A << lz, returns lz
GRD_HD int grd_normalize(grd_u128 A, uint64_t& h, uint64_t& l) {
  const uint64_t hi = (uint64_t)(A >> 64), lo = (uint64_t)A;
  if (hi) {
    const int lz = grd_clz64(hi);
    h = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    l = lo << lz;
    return lz;
  }
  const int lz = grd_clz64(lo);
  h = lo << lz;
  l = 0;
  return 64 + lz;
}

// A 2^-q rounded to nearest even (A > 0), with the sign bit `neg`; results
// below the normal range round once to a subnormal, above it to infinity.
GRD_HD double grd_round(grd_u128 A, int q, int neg) {
  const uint64_t hi = (uint64_t)(A >> 64), lo = (uint64_t)A;
  const int p = hi ? 127 - grd_clz64(hi) : 63 - grd_clz64(lo);  // leading bit
  int E = p - q;                                                 // A 2^-q in [2^E, 2^(E+1))
  const uint64_t sgn = (uint64_t)neg << 63;
  if (E > 1023) return grd_double(sgn | 0x7ff0000000000000ull);
  // bits dropped: keep 53 significant bits, or down to 2^-1074 when subnormal
  const int sh = E >= -1022 ? p - 52 : q - 1074;
  uint64_t sig;
  if (sh <= 0) {
    sig = (uint64_t)A << -sh;
  } else if (sh >= 128) {
    sig = 0;  // far below half of the smallest subnormal
  } else {
    sig = (uint64_t)(A >> sh);
    const grd_u128 rem = A & (((grd_u128)1 << sh) - 1);
    const grd_u128 half = (grd_u128)1 << (sh - 1);
    if (rem > half || (rem == half && (sig & 1))) ++sig;
  }
  if (E >= -1022) {
    if (sig >> 53) {  // rounding carried into a new leading bit
      sig >>= 1;
      ++E;
      if (E > 1023) return grd_double(sgn | 0x7ff0000000000000ull);
    }
    return grd_double(sgn | ((uint64_t)(E + 1023) << 52) | (sig & 0xfffffffffffffull));
  }
  return grd_double(sgn | sig);  // subnormal (a carry to 2^52 gives the smallest normal)
}

GRD_HD double grd_log(double x) {
  const uint64_t ux = grd_bits(x);
  if ((ux & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return x;  // NaN
  if (ux >> 63)
    return (ux << 1) == 0 ? grd_double(0xfff0000000000000ull) : grd_double(0x7ff8000000000000ull);
  if (ux == 0) return grd_double(0xfff0000000000000ull);
  if (ux == 0x7ff0000000000000ull) return x;
  int e;
  uint64_t M;
  if (ux < 0x0010000000000000ull) {  // subnormal: move the leading bit to 52
    const int s = grd_clz64(ux) - 11;
    M = ux << s;
    e = -1022 - s;
  } else {
    e = (int)(ux >> 52) - 1023;
    M = (ux & 0xfffffffffffffull) | 0x10000000000000ull;
  }
  const int i = (int)((M >> 45) & 127);
  const uint64_t y1 = M * (uint64_t)GRD_LD(GRT_ILOG_K1[i]);  // (1 + r1) 2^60
  const int64_t r1 = (int64_t)(y1 - (1ull << 60));
  int j = (int)((r1 + (1ll << 45)) >> 46) + GRT_ILOG_J0;
  j = j < 0 ? 0 : (j > GRT_ILOG_JN - 1 ? GRT_ILOG_JN - 1 : j);  // the tables cover every r1
  const grd_u128 y2 = (grd_u128)y1 * GRD_LD(GRT_ILOG_K2[j]);    // (1 + r2) 2^80
  const int64_t r = (int64_t)((grd_i128)(y2 - ((grd_u128)1 << 80)) >> 4);  // r2 2^76
  int64_t s = GRT_ILOG_S0;  // S(r2) in Q62: Q62 x Q76 >> 64 is Q74
  s = GRT_ILOG_S1 + (grd_mulhi(s, r) >> 12);
  s = GRT_ILOG_S2 + (grd_mulhi(s, r) >> 12);
  s = GRT_ILOG_S3 + (grd_mulhi(s, r) >> 12);
  s = GRT_ILOG_S4 + (grd_mulhi(s, r) >> 12);
  // e ln2 + L1_i + L2_j + r2 S(r2), Q116
  grd_i128 v = grd_mul_small(e, GRT_ILOG_LN2_HI, GRT_ILOG_LN2_LO);
  v += (grd_i128)grd_u128_of(GRD_LD(GRT_ILOG_L1[2 * i]), GRD_LD(GRT_ILOG_L1[2 * i + 1]));
  v += (grd_i128)grd_u128_of(GRD_LD(GRT_ILOG_L2[2 * j]), GRD_LD(GRT_ILOG_L2[2 * j + 1]));
  v += ((grd_i128)r * s) >> 22;  // Q138 -> Q116
  if (v == 0) return 0.0;
  const int neg = v < 0;
  uint64_t h, l;
  const int lz = grd_normalize(neg ? (grd_u128)(-v) : (grd_u128)v, h, l);
  return grd_round_norm(h, l, 127 - lz - 116, neg);  // |log x| is within [2^-53, 745]: normal
}

GRD_HD double grd_exp(double x) {
  const uint64_t ux = grd_bits(x);
  const uint64_t ax = ux & 0x7fffffffffffffffull;
  if (ax > 0x7ff0000000000000ull) return x;                   // NaN
  if (ax >= 0x4086200000000000ull) {                          // |x| >= 708
    if (!(ux >> 63) && ax > 0x40862e42fefa39efull) return grd_double(0x7ff0000000000000ull);  // > 709.7827...
    if ((ux >> 63) && ax > 0x40874910d52d3052ull) return 0.0;                                // < -745.1332...
  }
  if (ax < 0x3c90000000000000ull) return 1.0;  // |x| < 2^-54 rounds to 1
  const int ex = (int)(ax >> 52) - 1023;       // -54 .. 9
  const uint64_t M = (ax & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sx = ex + 48;                      // x 2^100 = M 2^sx
  grd_i128 xv = sx >= 0 ? (grd_i128)((grd_u128)M << sx) : (grd_i128)(M >> -sx);
  if (ux >> 63) xv = -xv;
  // n = round(64 x / ln2) from x in Q20 (floor) times 64/ln2 in Q20
  const int64_t xq = (int64_t)(xv >> 80);
  const int64_t n = (xq * GRT_IEXP_INVL + (1ll << 39)) >> 40;
  const grd_i128 rv = xv - grd_mul_small(n, GRT_IEXP_LN2_64_HI, GRT_IEXP_LN2_64_LO);  // Q100
  const int64_t r = (int64_t)(rv >> 36);                              // Q64
  int64_t c = GRT_IEXP_C0;  // Q62 x Q64 >> 64 is Q62
  c = GRT_IEXP_C1 + grd_mulhi(c, r);
  c = GRT_IEXP_C2 + grd_mulhi(c, r);
  c = GRT_IEXP_C3 + grd_mulhi(c, r);
  c = GRT_IEXP_C4 + grd_mulhi(c, r);
  c = GRT_IEXP_C5 + grd_mulhi(c, r);
  c = GRT_IEXP_C6 + grd_mulhi(c, r);
  c = GRT_IEXP_C7 + grd_mulhi(c, r);  // exp(r) in Q62
  const int jj = (int)(n & 63);
  const int m = (int)(n >> 6);
  const grd_u128 P = (grd_u128)GRD_LD(GRT_IEXP_T[jj]) * (uint64_t)c;  // Q125, in [2^124, 2^126)
  const int top = (int)(P >> 125);                                   // leading bit at 125 or 124
  const int E = m + top - 1;
  if (E < -1022) return grd_round(P, 125 - m, 0);                    // subnormal result
  const uint64_t hi = (uint64_t)(P >> 64), lo = (uint64_t)P;
  const uint64_t h = top ? (hi << 2) | (lo >> 62) : (hi << 3) | (lo >> 61);
  const uint64_t l = top ? lo << 2 : lo << 3;
  return grd_round_norm(h, l, E, 0);
}

}  // namespace gr
