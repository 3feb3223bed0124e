/*
 * CPU ORACLE — math.  Test infrastructure only; see oracle.h.
 *
 * log/exp: the library's own implementations, restated here independently of
 * the device code.  Float: Cephes-style polynomials with the same operation
 * order, explicit fmaf() (correctly rounded), every other operation rounded
 * on its own (coefficients from eigenrand_gb300/csrc/derive_math_coeffs.py).
 * Double: integer fixed-point arithmetic with one final rounding (tables
 * from ormath_tables.h).  Either way the oracle and the CUDA kernels agree
 * bit for bit.
 *
 * sincos: EigenRand's psincos (Cephes single-precision sin/cos with the
 * "extended precision modular arithmetic" reduction), restated lane-wise
 * from EigenRand/MorePacketMath.h:297-393 (float) and :395-491 (double).
 *
 * lgamma: EigenRand's plgamma_approx, MorePacketMath.h:158-170.
 *
 * erfinv: Giles' approximation as EigenRand's perfinv evaluates it.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle.h"
#include "ormath_tables.h"

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint64_t d2u(double f) { uint64_t u; memcpy(&u, &f, 8); return u; }
static inline double u2d(uint64_t u) { double f; memcpy(&f, &u, 8); return f; }

/* ------------------------------------------------------------------ logf */
float or_logf(float x) {
  uint32_t ux = f2u(x);
  if (x != x) return x;
  if (x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return -INFINITY;
  if (ux == 0x7f800000u) return x;
  int e = 0;
  if (ux < 0x00800000u) { /* subnormal: scale by 2^23 */
    x = x * 8388608.0f;
    ux = f2u(x);
    e = -23;
  }
  e += (int)((ux >> 23) & 0xff) - 126;
  float m = u2f((ux & 0x007fffffu) | 0x3f000000u); /* [0.5, 1) */
  float f;
  if (m < 0.70710678118654752f) {
    e -= 1;
    f = (m + m) - 1.0f;
  } else {
    f = m - 1.0f;
  }
  float z = f * f;
  float p = 7.149753720e-02f;
  p = fmaf(p, f, -1.157120094e-01f);
  p = fmaf(p, f, 1.166151091e-01f);
  p = fmaf(p, f, -1.241105050e-01f);
  p = fmaf(p, f, 1.424993724e-01f);
  p = fmaf(p, f, -1.666848063e-01f);
  p = fmaf(p, f, 2.000070810e-01f);
  p = fmaf(p, f, -2.499998957e-01f);
  p = fmaf(p, f, 3.333333135e-01f);
  float fe = (float)e;
  float y = (f * z) * p;
  y = fmaf(fe, -2.121944417e-04f, y);
  y = fmaf(-0.5f, z, y);
  float r = f + y;
  r = fmaf(fe, 6.933593750e-01f, r);
  return r;
}

/* ------------------------------------------------------------------ expf */
float or_expf(float x) {
  if (x != x) return x;
  if (x > 88.72283935546875f) return INFINITY;
  if (x < -103.972084045410156f) return 0.0f;
  float n = rintf(x * 1.442695022e+00f);
  float r = fmaf(-n, 6.933593750e-01f, x);
  r = fmaf(-n, -2.121944417e-04f, r);
  float p = 1.989927550e-04f;
  p = fmaf(p, r, 1.393364393e-03f);
  p = fmaf(p, r, 8.333298378e-03f);
  p = fmaf(p, r, 4.166646674e-02f);
  p = fmaf(p, r, 1.666666716e-01f);
  p = fmaf(p, r, 5.000000000e-01f);
  float r2 = r * r;
  float y = fmaf(r2, p, r) + 1.0f;
  int ni = (int)n;
  /* scale by 2^n in two steps so that subnormal results round once */
  if (ni > 127) {
    y = y * 2.0f;
    ni -= 1;
  }
  if (ni < -126) {
    y = y * u2f((uint32_t)(ni + 126 + 127) << 23);
    return y * u2f(0x00800000u); /* 2^-126 */
  }
  return y * u2f((uint32_t)(ni + 127) << 23);
}

/* ------------------------------------------------------------- log, exp
 * Integer arithmetic: fixed-point reductions and series in 64- and 128-bit
 * integers, one final rounding to double (the method notes and tables are
 * in eigenrand_gb300/csrc/derive_math_tables.py).  Restated here in C; the
 * integer steps are exact, so the oracle and the kernels agree bit for bit.
 */
typedef unsigned __int128 u128;
typedef __int128 i128;

static inline u128 u128_of(uint64_t hi, uint64_t lo) { return ((u128)hi << 64) | lo; }
static inline int clz64(uint64_t x) { return __builtin_clzll(x); }
static inline int64_t mulhi64(int64_t a, int64_t b) { return (int64_t)(((i128)a * b) >> 64); }

/* A 2^-q (A > 0) rounded to nearest even, signed by `neg`: 53 significant
 * bits, or down to 2^-1074 below the normal range; overflow gives infinity */
static double round_fixed(u128 A, int q, int neg) {
  const uint64_t hi = (uint64_t)(A >> 64), lo = (uint64_t)A;
  const int p = hi ? 127 - clz64(hi) : 63 - clz64(lo);
  int E = p - q;
  const uint64_t sgn = (uint64_t)neg << 63;
  if (E > 1023) return u2d(sgn | 0x7ff0000000000000ull);
  const int sh = E >= -1022 ? p - 52 : q - 1074;
  uint64_t sig;
  if (sh <= 0) {
    sig = (uint64_t)A << -sh;
  } else if (sh >= 128) {
    sig = 0;
  } else {
    sig = (uint64_t)(A >> sh);
    const u128 rem = A & (((u128)1 << sh) - 1), half = (u128)1 << (sh - 1);
    if (rem > half || (rem == half && (sig & 1))) ++sig;
  }
  if (E >= -1022) {
    if (sig >> 53) {
      sig >>= 1;
      if (++E > 1023) return u2d(sgn | 0x7ff0000000000000ull);
    }
    return u2d(sgn | ((uint64_t)(E + 1023) << 52) | (sig & 0xfffffffffffffull));
  }
  return u2d(sgn | sig);
}

/* log x = e ln2 + L1_i + L2_j + r2 S(r2): two reciprocal reductions
 * (y1 = M K1_i = (1 + r1) 2^60, y2 = y1 K2_j = (1 + r2) 2^80, exact),
 * S(r) = 1 - r/2 + r^2/3 - r^3/4 + r^4/5 in Q62, the sum in Q116 */
/* Timing mode for the CPU baseline: the integer arithmetic above is exact
 * and portable but slow on a CPU, whose FP64 units are fast, while the
 * reference calls Eigen's FP64 plog / pexp.  With it on, or_log / or_exp are
 * the C library's FP64 log / exp (within an ulp; never used for parity). */
static int g_fp_math = 0;
void or_set_fp_math(int on) { g_fp_math = on; }

double or_log(double x) {
  if (g_fp_math) return log(x);
  const uint64_t ux = d2u(x);
  if ((ux & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return x; /* NaN */
  if (ux >> 63) return (ux << 1) == 0 ? -INFINITY : u2d(0x7ff8000000000000ull);
  if (ux == 0) return -INFINITY;
  if (ux == 0x7ff0000000000000ull) return x;
  int e;
  uint64_t M;
  if (ux < 0x0010000000000000ull) { /* subnormal */
    const int s = clz64(ux) - 11;
    M = ux << s;
    e = -1022 - s;
  } else {
    e = (int)(ux >> 52) - 1023;
    M = (ux & 0xfffffffffffffull) | 0x10000000000000ull;
  }
  const int i = (int)((M >> 45) & 127);
  const uint64_t y1 = M * (uint64_t)GRT_ILOG_K1[i];
  const int64_t r1 = (int64_t)(y1 - (1ull << 60));
  int j = (int)((r1 + (1ll << 45)) >> 46) + GRT_ILOG_J0;
  if (j < 0) j = 0;
  if (j > GRT_ILOG_JN - 1) j = GRT_ILOG_JN - 1;
  const u128 y2 = (u128)y1 * GRT_ILOG_K2[j];
  const int64_t r = (int64_t)((i128)(y2 - ((u128)1 << 80)) >> 4); /* Q76 */
  int64_t s = GRT_ILOG_S0;
  s = GRT_ILOG_S1 + (mulhi64(s, r) >> 12);
  s = GRT_ILOG_S2 + (mulhi64(s, r) >> 12);
  s = GRT_ILOG_S3 + (mulhi64(s, r) >> 12);
  s = GRT_ILOG_S4 + (mulhi64(s, r) >> 12);
  i128 v = (i128)e * (i128)u128_of(GRT_ILOG_LN2_HI, GRT_ILOG_LN2_LO);
  v += (i128)u128_of(GRT_ILOG_L1[2 * i], GRT_ILOG_L1[2 * i + 1]);
  v += (i128)u128_of(GRT_ILOG_L2[2 * j], GRT_ILOG_L2[2 * j + 1]);
  v += ((i128)r * s) >> 22;
  if (v == 0) return 0.0;
  return v < 0 ? round_fixed((u128)(-v), 116, 1) : round_fixed((u128)v, 116, 0);
}

/* exp x = 2^(n div 64) 2^((n mod 64)/64) exp(r), n = round(64 x / ln2)
 * estimated from x in Q20, r = x - n ln2/64 exact in Q100, exp(r) by its
 * Taylor series to degree 7 in Q62, 2^(j/64) in Q63 */
double or_exp(double x) {
  if (g_fp_math) return exp(x);
  const uint64_t ux = d2u(x), ax = ux & 0x7fffffffffffffffull;
  if (ax > 0x7ff0000000000000ull) return x;
  if (ax >= 0x4086200000000000ull) { /* |x| >= 708 */
    if (!(ux >> 63) && ax > 0x40862e42fefa39efull) return INFINITY; /* > 709.782712893384 */
    if ((ux >> 63) && ax > 0x40874910d52d3052ull) return 0.0;       /* < -745.1332191019412 */
  }
  if (ax < 0x3c90000000000000ull) return 1.0; /* |x| < 2^-54 */
  const int ex = (int)(ax >> 52) - 1023;
  const uint64_t M = (ax & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sx = ex + 48;
  i128 xv = sx >= 0 ? (i128)((u128)M << sx) : (i128)(M >> -sx);
  if (ux >> 63) xv = -xv;
  const int64_t xq = (int64_t)(xv >> 80);
  const int64_t n = (xq * GRT_IEXP_INVL + (1ll << 39)) >> 40;
  const i128 rv = xv - (i128)n * (i128)u128_of(GRT_IEXP_LN2_64_HI, GRT_IEXP_LN2_64_LO);
  const int64_t r = (int64_t)(rv >> 36);
  int64_t c = GRT_IEXP_C0;
  c = GRT_IEXP_C1 + mulhi64(c, r);
  c = GRT_IEXP_C2 + mulhi64(c, r);
  c = GRT_IEXP_C3 + mulhi64(c, r);
  c = GRT_IEXP_C4 + mulhi64(c, r);
  c = GRT_IEXP_C5 + mulhi64(c, r);
  c = GRT_IEXP_C6 + mulhi64(c, r);
  c = GRT_IEXP_C7 + mulhi64(c, r);
  const int jj = (int)(n & 63), m = (int)(n >> 6);
  return round_fixed((u128)GRT_IEXP_T[jj] * (uint64_t)c, 125 - m, 0);
}

/* --------------------------------------------------------------- sincosf */
/* MorePacketMath.h:297-393, one lane. pcast<Packet8f,Packet8i> truncates
 * (cvttps); pnew_andnot(a,b) = a & ~b. */
void or_sincosf(float x, float* s, float* c) {
  uint32_t sign_bit_sin = f2u(x) & 0x80000000u;
  x = fabsf(x);
  float y = x * (float)1.27323954473516;
  int32_t emm2 = (int32_t)y;
  emm2 = emm2 + 1;
  emm2 = emm2 & ~1;
  y = (float)emm2;
  int32_t emm4 = emm2;
  uint32_t swap_sign_bit_sin = ((uint32_t)(emm2 & 4)) << 29;
  emm2 = emm2 & 2;
  uint32_t poly_mask = (emm2 == 0) ? 0xffffffffu : 0u;
  float xmm1 = y * (float)-0.78515625;
  float xmm2 = y * (float)-2.4187564849853515625e-4;
  float xmm3 = y * (float)-3.77489497744594108e-8;
  x = x + xmm1;
  x = x + xmm2;
  x = x + xmm3;
  emm4 = emm4 - 2;
  emm4 = 4 & ~emm4;
  uint32_t sign_bit_cos = ((uint32_t)emm4) << 29;
  sign_bit_sin ^= swap_sign_bit_sin;
  float z = x * x;
  float yy = (float)2.443315711809948E-005;
  yy = yy * z;
  yy = yy + (float)-1.388731625493765E-003;
  yy = yy * z;
  yy = yy + (float)4.166664568298827E-002;
  yy = yy * z;
  yy = yy * z;
  float tmp = z * 0.5f;
  yy = yy - tmp;
  yy = yy + 1.0f;
  float y2 = (float)-1.9515295891E-4;
  y2 = y2 * z;
  y2 = y2 + (float)8.3321608736E-3;
  y2 = y2 * z;
  y2 = y2 + (float)-1.6666654611E-1;
  y2 = y2 * z;
  y2 = y2 * x;
  y2 = y2 + x;
  float ysin2 = u2f(poly_mask & f2u(y2));
  float ysin1 = u2f(f2u(yy) & ~poly_mask);
  y2 = y2 - ysin2;
  yy = yy - ysin1;
  float o1 = ysin1 + ysin2;
  float o2 = yy + y2;
  *s = u2f(f2u(o1) ^ sign_bit_sin);
  *c = u2f(f2u(o2) ^ sign_bit_cos);
}

/* ---------------------------------------------------------------- sincos */
/* MorePacketMath.h:395-491 (double packets).  pcast64 from double is the
 * floor-based magic-number conversion (arch/AVX/MorePacketMath.h:731-738);
 * arguments here are >= 0 so it equals truncation. */
void or_sincos(double x, double* s, double* c) {
  uint64_t sign_bit_sin = d2u(x) & 0x8000000000000000ull;
  x = fabs(x);
  double y = x * 1.27323954473516;
  int64_t emm2 = (int64_t)floor(y);
  emm2 = emm2 + 1;
  emm2 = emm2 & ~(int64_t)1;
  y = (double)emm2;
  int64_t emm4 = emm2;
  uint64_t swap_sign_bit_sin = ((uint64_t)(emm2 & 4)) << 61;
  emm2 = emm2 & 2;
  uint64_t poly_mask = (emm2 == 0) ? ~0ull : 0ull;
  double xmm1 = y * -0.78515625;
  double xmm2 = y * -2.4187564849853515625e-4;
  double xmm3 = y * -3.77489497744594108e-8;
  x = x + xmm1;
  x = x + xmm2;
  x = x + xmm3;
  emm4 = emm4 - 2;
  emm4 = 4 & ~emm4;
  uint64_t sign_bit_cos = ((uint64_t)emm4) << 61;
  sign_bit_sin ^= swap_sign_bit_sin;
  double z = x * x;
  double yy = 2.443315711809948E-005;
  yy = yy * z;
  yy = yy + -1.388731625493765E-003;
  yy = yy * z;
  yy = yy + 4.166664568298827E-002;
  yy = yy * z;
  yy = yy * z;
  double tmp = z * 0.5;
  yy = yy - tmp;
  yy = yy + 1.0;
  double y2 = -1.9515295891E-4;
  y2 = y2 * z;
  y2 = y2 + 8.3321608736E-3;
  y2 = y2 * z;
  y2 = y2 + -1.6666654611E-1;
  y2 = y2 * z;
  y2 = y2 * x;
  y2 = y2 + x;
  double ysin2 = u2d(poly_mask & d2u(y2));
  double ysin1 = u2d(d2u(yy) & ~poly_mask);
  y2 = y2 - ysin2;
  yy = yy - ysin1;
  double o1 = ysin1 + ysin2;
  double o2 = yy + y2;
  *s = u2d(d2u(o1) ^ sign_bit_sin);
  *c = u2d(d2u(o2) ^ sign_bit_cos);
}

/* ------------------------------------------------------- plgamma_approx */
/* lgamma(z) ~= (z+2.5)ln(z+3) - z - 3 + 0.5 ln(2pi) + 1/12/(z+3)
 *             - ln(z(z+1)(z+2)),  MorePacketMath.h:158-170 */
float or_lgamma_approxf(float x) {
  float x_3 = x + 3.0f;
  float ret = (x_3 + -0.5f) * or_logf(x_3);
  ret = ret - x_3;
  ret = ret + (float)0.9189385332046727;
  ret = ret + (float)(1 / 12.) / x_3;
  ret = ret - or_logf(((x_3 - 1.0f) * (x_3 - 2.0f)) * x);
  return ret;
}

double or_lgamma_approx(double x) {
  double x_3 = x + 3.0;
  double ret = (x_3 + -0.5) * or_log(x_3);
  ret = ret - x_3;
  ret = ret + 0.9189385332046727;
  ret = ret + (1 / 12.) / x_3;
  ret = ret - or_log(((x_3 - 1.0) * (x_3 - 2.0)) * x);
  return ret;
}

/* ---------------------------------------------------------------- erfinv */
/* M. Giles, "Approximating the erfinv function" (GPU Computing Gems, Jade
 * Edition, 2011): w = -log((1 - x)(1 + x)), then a polynomial in w - c (small
 * w) or sqrt(w) - c (large w), times x.  Evaluated as EigenRand's packet
 * perfinv does (MorePacketMath.h:499-535 float, :543-624 double): both the
 * product and the sum of each Horner step round on their own, and the region
 * is picked by w < 5 (float) or w < 6.25 / w < 16 (double). */
static const float ERFINV_F_SMALL[9] = {
    2.81022636e-08f, 3.43273939e-07f, -3.5233877e-06f, -4.39150654e-06f, 0.00021858087f,
    -0.00125372503f, -0.00417768164f, 0.246640727f, 1.50140941f};
static const float ERFINV_F_LARGE[9] = {
    -0.000200214257f, 0.000100950558f, 0.00134934322f, -0.00367342844f, 0.00573950773f,
    -0.0076224613f, 0.00943887047f, 1.00167406f, 2.83297682f};
static const double ERFINV_D_SMALL[23] = {
    -3.6444120640178196996e-21, -1.685059138182016589e-19, 1.2858480715256400167e-18,
    1.115787767802518096e-17, -1.333171662854620906e-16, 2.0972767875968561637e-17,
    6.6376381343583238325e-15, -4.0545662729752068639e-14, -8.1519341976054721522e-14,
    2.6335093153082322977e-12, -1.2975133253453532498e-11, -5.4154120542946279317e-11,
    1.051212273321532285e-09, -4.1126339803469836976e-09, -2.9070369957882005086e-08,
    4.2347877827932403518e-07, -1.3654692000834678645e-06, -1.3882523362786468719e-05,
    0.0001867342080340571352, -0.00074070253416626697512, -0.0060336708714301490533,
    0.24015818242558961693, 1.6536545626831027356};
static const double ERFINV_D_MID[19] = {
    2.2137376921775787049e-09, 9.0756561938885390979e-08, -2.7517406297064545428e-07,
    1.8239629214389227755e-08, 1.5027403968909827627e-06, -4.013867526981545969e-06,
    2.9234449089955446044e-06, 1.2475304481671778723e-05, -4.7318229009055733981e-05,
    6.8284851459573175448e-05, 2.4031110387097893999e-05, -0.0003550375203628474796,
    0.00095328937973738049703, -0.0016882755560235047313, 0.0024914420961078508066,
    -0.0037512085075692412107, 0.005370914553590063617, 1.0052589676941592334,
    3.0838856104922207635};
static const double ERFINV_D_LARGE[17] = {
    -2.7109920616438573243e-11, -2.5556418169965252055e-10, 1.5076572693500548083e-09,
    -3.7894654401267369937e-09, 7.6157012080783393804e-09, -1.4960026627149240478e-08,
    2.9147953450901080826e-08, -6.7711997758452339498e-08, 2.2900482228026654717e-07,
    -9.9298272942317002539e-07, 4.5260625972231537039e-06, -1.9681778105531670567e-05,
    7.5995277030017761139e-05, -0.00021503011930044477347, -0.00013871931833623122026,
    1.0103004648645343977, 4.8499064014085844221};

static float horner_f(const float* c, int n, float t) {
  float p = c[0];
  for (int i = 1; i < n; ++i) p = p * t + c[i];
  return p;
}
static double horner_d(const double* c, int n, double t) {
  double p = c[0];
  for (int i = 1; i < n; ++i) p = p * t + c[i];
  return p;
}

float or_erfinvf(float x) {
  const float w = -or_logf((1.0f - x) * (1.0f + x));
  const float p = w < 5.0f ? horner_f(ERFINV_F_SMALL, 9, w - 2.5f) : horner_f(ERFINV_F_LARGE, 9, sqrtf(w) - 3.0f);
  return p * x;
}

double or_erfinv(double x) {
  const double w = -or_log((1.0 - x) * (1.0 + x));
  double p;
  if (w < 6.25) p = horner_d(ERFINV_D_SMALL, 23, w - 3.125);
  else if (w < 16.0) p = horner_d(ERFINV_D_MID, 19, sqrt(w) - 3.25);
  else p = horner_d(ERFINV_D_LARGE, 17, sqrt(w) - 5.0);
  return p * x;
}

void or_vec_logf(const float* x, float* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_logf(x[i]); }
void or_vec_expf(const float* x, float* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_expf(x[i]); }
void or_vec_log(const double* x, double* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_log(x[i]); }
void or_vec_exp(const double* x, double* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_exp(x[i]); }
void or_vec_erfinvf(const float* x, float* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_erfinvf(x[i]); }
void or_vec_erfinv(const double* x, double* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_erfinv(x[i]); }
void or_vec_sincosf(const float* x, float* s, float* c, size_t n) {
  for (size_t i = 0; i < n; ++i) or_sincosf(x[i], s + i, c + i);
}
void or_vec_sincos(const double* x, double* s, double* c, size_t n) {
  for (size_t i = 0; i < n; ++i) or_sincos(x[i], s + i, c + i);
}
