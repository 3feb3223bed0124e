// Device math for the sampling kernels.
//
// log/exp are this library's own implementations of published methods:
//   logf/log : exponent/mantissa split with m in [sqrt(1/2), sqrt(2)),
//              logf -> f - f^2/2 + f^3*P8(f)  (Cephes-style reduction),
//              log  -> 2*atanh(s), s = f/(2+f), Taylor series in s^2;
//   expf/exp : Cody-Waite reduction by ln2, polynomial (fitted / Taylor),
//              scaling by 2^n in at most two steps.
// Coefficients are derived by derive_math_coeffs.py.  Every operation is
// rounded on its own (the library is compiled with --fmad=false) except the
// explicit fmaf/fma calls, so the same sequence evaluated on the CPU with a
// correctly rounded fma gives identical bits.  Max error measured against
// 60-digit references: <= 1 ulp.
//
// sincos is EigenRand's own psincos (Cephes single-precision sin/cos with the
// three-constant pi/4 reduction), EigenRand/MorePacketMath.h:297-491, and
// lgamma_approx is EigenRand's plgamma_approx, MorePacketMath.h:158-170.
#pragma once
#include <cstdint>

#include "gr_dmath.h"
#include "gr_math_tables.h"

namespace gr {

__device__ __forceinline__ uint32_t f2u(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ uint64_t d2u(double f) { return (uint64_t)__double_as_longlong(f); }
__device__ __forceinline__ double u2d(uint64_t u) { return __longlong_as_double((long long)u); }

__device__ __forceinline__ float logf_(float x) {
  uint32_t ux = f2u(x);
  if (x != x) return x;
  if (x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return -__int_as_float(0x7f800000);
  if (ux == 0x7f800000u) return x;
  int e = 0;
  if (ux < 0x00800000u) {
    x = x * 8388608.0f;
    ux = f2u(x);
    e = -23;
  }
  e += (int)((ux >> 23) & 0xff) - 126;
  float m = u2f((ux & 0x007fffffu) | 0x3f000000u);
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

__device__ __forceinline__ float expf_(float x) {
  if (x != x) return x;
  if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
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
  if (ni > 127) {
    y = y * 2.0f;
    ni -= 1;
  }
  if (ni < -126) {
    y = y * u2f((uint32_t)(ni + 126 + 127) << 23);
    return y * u2f(0x00800000u);
  }
  return y * u2f((uint32_t)(ni + 127) << 23);
}

// _mm_cvttps_epi32 of one lane: truncation; NaN and out of range give INT_MIN
__device__ __forceinline__ int32_t cvtt_f32(float x) {
  return (x >= -2147483648.0f && x < 2147483648.0f) ? (int32_t)x : (int32_t)0x80000000u;
}

// Double log / exp in integer arithmetic (gr_dmath.h): no FP64 instruction,
// about 0.5 ulp.
__device__ __forceinline__ double log_(double x) { return grd_log(x); }
__device__ __forceinline__ double exp_(double x) { return grd_exp(x); }

// EigenRand psincos, float lanes (MorePacketMath.h:297-393).
__device__ __forceinline__ void sincosf_(float x, float& s, float& c) {
  uint32_t sign_bit_sin = f2u(x) & 0x80000000u;
  x = fabsf(x);
  float y = x * (float)1.27323954473516;
  int32_t emm2 = __float2int_rz(y);
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
  s = u2f(f2u(o1) ^ sign_bit_sin);
  c = u2f(f2u(o2) ^ sign_bit_cos);
}

// EigenRand psincos, double lanes (MorePacketMath.h:395-491); the float-grade
// Cephes coefficients are evaluated in double arithmetic, as there.
__device__ __forceinline__ void sincos_(double x, double& s, double& c) {
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
  s = u2d(d2u(o1) ^ sign_bit_sin);
  c = u2d(d2u(o2) ^ sign_bit_cos);
}

__device__ __forceinline__ float lgamma_approxf_(float x) {
  float x_3 = x + 3.0f;
  float ret = (x_3 + -0.5f) * logf_(x_3);
  ret = ret - x_3;
  ret = ret + (float)0.9189385332046727;
  ret = ret + (float)(1 / 12.) / x_3;
  ret = ret - logf_(((x_3 - 1.0f) * (x_3 - 2.0f)) * x);
  return ret;
}

__device__ __forceinline__ double lgamma_approx_(double x) {
  double x_3 = x + 3.0;
  double ret = (x_3 + -0.5) * log_(x_3);
  ret = ret - x_3;
  ret = ret + 0.9189385332046727;
  ret = ret + (1 / 12.) / x_3;
  ret = ret - log_(((x_3 - 1.0) * (x_3 - 2.0)) * x);
  return ret;
}

}  // namespace gr
