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
// erfinv is Giles' approximation as EigenRand's perfinv evaluates it.
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

// Inverse error function: M. Giles, "Approximating the erfinv function" (GPU
// Computing Gems, Jade Edition, 2011).  w = -log((1 - x)(1 + x)); erfinv(x) =
// x * P(w - c) for small w, x * Q(sqrt(w) - c') for large w, with Giles'
// published coefficients.  The evaluation follows EigenRand's packet perfinv
// (MorePacketMath.h:499-535 float, :543-624 double): every product and sum
// rounds on its own, and the region is picked by w < 5 (float) or w < 6.25,
// w < 16 (double).  log is the library's own logf_/log_ above.
static __constant__ float kErfinvFSmall[9] = {
    2.81022636e-08f, 3.43273939e-07f, -3.5233877e-06f, -4.39150654e-06f, 0.00021858087f,
    -0.00125372503f, -0.00417768164f, 0.246640727f, 1.50140941f};
static __constant__ float kErfinvFLarge[9] = {
    -0.000200214257f, 0.000100950558f, 0.00134934322f, -0.00367342844f, 0.00573950773f,
    -0.0076224613f, 0.00943887047f, 1.00167406f, 2.83297682f};
static __constant__ double kErfinvDSmall[23] = {
    -3.6444120640178196996e-21, -1.685059138182016589e-19, 1.2858480715256400167e-18,
    1.115787767802518096e-17, -1.333171662854620906e-16, 2.0972767875968561637e-17,
    6.6376381343583238325e-15, -4.0545662729752068639e-14, -8.1519341976054721522e-14,
    2.6335093153082322977e-12, -1.2975133253453532498e-11, -5.4154120542946279317e-11,
    1.051212273321532285e-09, -4.1126339803469836976e-09, -2.9070369957882005086e-08,
    4.2347877827932403518e-07, -1.3654692000834678645e-06, -1.3882523362786468719e-05,
    0.0001867342080340571352, -0.00074070253416626697512, -0.0060336708714301490533,
    0.24015818242558961693, 1.6536545626831027356};
static __constant__ double kErfinvDMid[19] = {
    2.2137376921775787049e-09, 9.0756561938885390979e-08, -2.7517406297064545428e-07,
    1.8239629214389227755e-08, 1.5027403968909827627e-06, -4.013867526981545969e-06,
    2.9234449089955446044e-06, 1.2475304481671778723e-05, -4.7318229009055733981e-05,
    6.8284851459573175448e-05, 2.4031110387097893999e-05, -0.0003550375203628474796,
    0.00095328937973738049703, -0.0016882755560235047313, 0.0024914420961078508066,
    -0.0037512085075692412107, 0.005370914553590063617, 1.0052589676941592334,
    3.0838856104922207635};
static __constant__ double kErfinvDLarge[17] = {
    -2.7109920616438573243e-11, -2.5556418169965252055e-10, 1.5076572693500548083e-09,
    -3.7894654401267369937e-09, 7.6157012080783393804e-09, -1.4960026627149240478e-08,
    2.9147953450901080826e-08, -6.7711997758452339498e-08, 2.2900482228026654717e-07,
    -9.9298272942317002539e-07, 4.5260625972231537039e-06, -1.9681778105531670567e-05,
    7.5995277030017761139e-05, -0.00021503011930044477347, -0.00013871931833623122026,
    1.0103004648645343977, 4.8499064014085844221};

template <int N>
__device__ __forceinline__ float horner_f(const float (&c)[N], float t) {
  float p = c[0];
#pragma unroll
  for (int i = 1; i < N; ++i) p = __fadd_rn(__fmul_rn(p, t), c[i]);
  return p;
}
template <int N>
__device__ __forceinline__ double horner_d(const double (&c)[N], double t) {
  double p = c[0];
#pragma unroll
  for (int i = 1; i < N; ++i) p = __dadd_rn(__dmul_rn(p, t), c[i]);
  return p;
}

__device__ __forceinline__ float erfinvf_(float x) {
  const float w = -logf_((1.0f - x) * (1.0f + x));
  const float p = w < 5.0f ? horner_f(kErfinvFSmall, w - 2.5f) : horner_f(kErfinvFLarge, __fsqrt_rn(w) - 3.0f);
  return p * x;
}

__device__ __forceinline__ double erfinv_(double x) {
  const double w = -log_((1.0 - x) * (1.0 + x));
  double p;
  if (w < 6.25) p = horner_d(kErfinvDSmall, w - 3.125);
  else if (w < 16.0) p = horner_d(kErfinvDMid, __dsqrt_rn(w) - 3.25);
  else p = horner_d(kErfinvDLarge, __dsqrt_rn(w) - 5.0);
  return p * x;
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
