/*
 * CPU ORACLE — math.  Test infrastructure only; see oracle.h.
 *
 * log/exp: the library's own published-method implementations, restated here
 * independently of the device code (double: table-driven, tables from
 * ormath_tables.h).  Same operation order, explicit fma() /
 * fmaf() (correctly rounded), every other operation rounded on its own, so
 * the oracle and the CUDA kernels agree bit for bit.  Coefficients come from
 * eigenrand_gb300/csrc/derive_math_coeffs.py.
 *
 * sincos: EigenRand's psincos (Cephes single-precision sin/cos with the
 * "extended precision modular arithmetic" reduction), restated lane-wise
 * from EigenRand/MorePacketMath.h:297-393 (float) and :395-491 (double).
 *
 * lgamma: EigenRand's plgamma_approx, MorePacketMath.h:158-170.
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
 * Table-driven (P. T. P. Tang, ACM TOMS 1989 and 1990); tables and the
 * method notes in eigenrand_gb300/csrc/derive_math_tables.py.
 */
double or_log(double x) {
  uint64_t ux = d2u(x);
  if ((ux & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return x; /* NaN */
  if (ux >> 63) return (ux << 1) == 0 ? -INFINITY : u2d(0x7ff8000000000000ull);
  if (ux == 0) return -INFINITY;
  if (ux == 0x7ff0000000000000ull) return x;
  int e = 0;
  if (ux < 0x0010000000000000ull) {
    x = x * 18014398509481984.0; /* 2^54 */
    ux = d2u(x);
    e = -54;
  }
  e += (int)(ux >> 52) - 1023;
  const int i = (int)((ux >> 45) & 127);
  const double m = u2d((ux & 0x000fffffffffffffull) | 0x3ff0000000000000ull); /* [1, 2) */
  const double r = fma(m, GRT_LOG_INVC[i], -1.0);
  const double de = (double)e;
  const double hi = fma(de, GRT_LOG_LN2_HI, GRT_LOG_C_HI[i]); /* exact: both on the 2^-42 grid */
  const double lo = fma(de, GRT_LOG_LN2_LO, GRT_LOG_C_LO[i]);
  const double r2 = r * r;
  double q = GRT_LOG_Q6;
  q = fma(q, r, GRT_LOG_Q5);
  q = fma(q, r, GRT_LOG_Q4);
  q = fma(q, r, GRT_LOG_Q3);
  q = fma(q, r, GRT_LOG_Q2);
  q = fma(q, r, GRT_LOG_Q1);
  q = fma(q, r, GRT_LOG_Q0);
  const double t = (r2 * r) * q; /* r^3 Q(r) */
  double s = lo + t;
  s = s - 0.5 * r2;
  s = s + r;
  return hi + s;
}

double or_exp(double x) {
  const uint64_t ax = d2u(x) & 0x7fffffffffffffffull;
  if (ax >= 0x4086200000000000ull) { /* |x| >= 708, inf or NaN */
    if (ax > 0x7ff0000000000000ull) return x;
    if (x > 709.782712893383973) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
  }
  const double z = fma(x, GRT_EXP_INV_L, 6755399441055744.0); /* 1.5 * 2^52 + n */
  const double n = z - 6755399441055744.0;
  const int32_t ni = (int32_t)(uint32_t)d2u(z);
  const int j = ni & 63;
  int mm = (ni - j) / 64;
  double r = fma(-n, GRT_EXP_L_HI, x);
  r = fma(-n, GRT_EXP_L_LO, r);
  double q = GRT_EXP_C6;
  q = fma(q, r, GRT_EXP_C5);
  q = fma(q, r, GRT_EXP_C4);
  q = fma(q, r, GRT_EXP_C3);
  q = fma(q, r, GRT_EXP_C2);
  const double p = fma(r * r, q, r); /* exp(r) - 1 */
  const double th = GRT_EXP_T_HI[j];
  double y = th + fma(th, p, GRT_EXP_T_LO[j]);
  if (mm < -1022) {
    y = y * u2d((uint64_t)(mm + 1022 + 1023) << 52);
    return y * u2d(0x0010000000000000ull); /* 2^-1022 */
  }
  return y * u2d((uint64_t)(mm + 1023) << 52);
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

void or_vec_logf(const float* x, float* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_logf(x[i]); }
void or_vec_expf(const float* x, float* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_expf(x[i]); }
void or_vec_log(const double* x, double* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_log(x[i]); }
void or_vec_exp(const double* x, double* y, size_t n) { for (size_t i = 0; i < n; ++i) y[i] = or_exp(x[i]); }
void or_vec_sincosf(const float* x, float* s, float* c, size_t n) {
  for (size_t i = 0; i < n; ++i) or_sincosf(x[i], s + i, c + i);
}
void or_vec_sincos(const double* x, double* s, double* c, size_t n) {
  for (size_t i = 0; i < n; ++i) or_sincos(x[i], s + i, c + i);
}
