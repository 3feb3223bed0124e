// Exact integer forms of floating-point expressions of the reference, shared
// by the kernels and the host-side checks (compiles as plain C++).
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define GR_HD __host__ __device__ __forceinline__
#else
#define GR_HD inline
#endif

namespace gr {

GR_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

GR_HD double bits_to_double(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// (double)k / 2147483647.0 (BalancedGen<double>'s quotient, round to
// nearest), 0 <= k <= 2^31 - 1, with no division.  1 / (2^31 - 1) =
// 2^-31 (1 + 2^-31 + 2^-62 + ...), so for 0 < k < 2^31 - 1 the quotient is
// X 2^-62 + t with X = k (2^31 + 1) < 2^62 and 0 < t < 2^-62.  t never
// vanishes, so no quotient lies on a midpoint: rounding to nearest keeps the
// leading 53 bits of X and adds the bit after them (a carry out of the
// significand moves into the exponent).
GR_HD double div_2p31m1(uint32_t k) {
  if (k == 0u) return 0.0;
  if (k == 0x7fffffffu) return 1.0;
  const uint64_t X = (uint64_t)k * 0x80000001ull;
  const int lz = clz64(X);                 // 2 .. 32
  const uint64_t N = X << lz;              // leading bit at 63; value N 2^(-62-lz)
  const uint64_t sig = N >> 11;            // 53 bits with the leading one at bit 52
  const uint64_t rnd = (N >> 10) & 1ull;
  return bits_to_double(((uint64_t)(1023 - lz) << 52) + sig + rnd);
}

// 1 - u for u = asdouble((x & (2^52 - 1)) | 1.0) - 1 (the reference's
// uniform double, then 1 - u): both steps are exact, and the result is
// 2 - m = (2^52 - F) 2^-52 for the fraction F, built here from the integer.
GR_HD double one_minus_ur_d(uint64_t x) {
  const uint64_t F = x & 0xfffffffffffffull;
  if (F == 0) return 1.0;
  const uint64_t D = 0x10000000000000ull - F;  // 1 .. 2^52 - 1
  const int p = 63 - clz64(D);                 // leading bit, 0 .. 51
  return bits_to_double(((uint64_t)(p + 1023 - 52) << 52) | ((D << (52 - p)) & 0xfffffffffffffull));
}

// MT19937-64 tempering (PacketRandomEngine.h:295-310) and its inverse:
// each step y ^= (y >> s) & m or y ^= (y << s) & m is undone by iterating
// x = y ^ ((x >> s) & m) (or <<) until s (k + 1) >= 64.
GR_HD uint64_t mt_temper64(uint64_t r) {
  r ^= (r >> 29) & 0x5555555555555555ull;
  r ^= (r << 17) & 0x71d67fffeda60000ull;
  r ^= (r << 37) & 0xfff7eee000000000ull;
  r ^= r >> 43;
  return r;
}
GR_HD uint64_t mt_untemper64(uint64_t y) {
  y ^= y >> 43;
  y ^= (y << 37) & 0xfff7eee000000000ull;
  uint64_t x = y;
  for (int k = 0; k < 3; ++k) x = y ^ ((x << 17) & 0x71d67fffeda60000ull);
  y = x;
  for (int k = 0; k < 2; ++k) x = y ^ ((x >> 29) & 0x5555555555555555ull);
  return x;
}

// Inverse of one MT19937-64 block twist (PacketRandomEngine.h:340-404): from
// the 312 words nw of a block recover the 312 words of the block before.
// nw[i] = c_i ^ f(y_i) with y_i = (old[i] & upper) | (old[i + 1] & lower)
// (old[312] read as nw[0]), c_i = old[i + 156] below 156 and nw[i - 156]
// from 156 on, and f(y) = (y >> 1) ^ (y & 1 ? MATRIX_A : 0); since the top
// bit of MATRIX_A is set, the top bit of f(y) is y & 1, so f inverts.  The
// y_i of the upper half come from nw alone, those of the lower half from the
// recovered upper half, and old[0]'s lower bits from the twist that made
// old[311] (old[311] = old[155] ^ f((older & upper) | (old[0] & lower))).
// `idx` gives the element of a lane window (stride for lane-major layouts).
GR_HD uint64_t mt_finv(uint64_t t) {
  const uint64_t b = t >> 63;
  return ((t ^ (b ? 0xb5026f5aa96619e9ull : 0ull)) << 1) | b;
}
template <class NW, class OLD>
GR_HD void mt_untwist_block(NW&& nw, OLD&& old) {
  // MT19937-64 splits a word into its upper 33 and lower 31 bits
  constexpr uint64_t U = 0xffffffff80000000ull, L = 0x000000007fffffffull;
  // upper half: y_i for i in [156, 312) from nw only
  for (int i = 156; i < 312; ++i) {
    const uint64_t y = mt_finv(nw(i) ^ nw(i - 156));
    const uint64_t hi = y & U;
    old(i) = hi | (i > 156 ? (old(i) & L) : 0);  // lower bits of old[i] come from y_(i-1)
    if (i + 1 < 312) old(i + 1) = (old(i + 1) & U) | (y & L);
  }
  // y_155 = (old[155] & U) | (old[156] & L): nw[155] = old[311] ^ f(y_155)
  {
    const uint64_t y = mt_finv(nw(155) ^ old(311));
    old(156) = (old(156) & U) | (y & L);
    old(155) = y & U;
  }
  for (int i = 154; i >= 0; --i) {
    const uint64_t y = mt_finv(nw(i) ^ old(i + 156));
    old(i + 1) = (old(i + 1) & U) | (y & L);
    old(i) = y & U;
  }
  // lower bits of old[0]: old[311] = old[155] ^ f((older & U) | (old[0] & L))
  old(0) = (old(0) & U) | (mt_finv(old(311) ^ old(155)) & L);
}

}  // namespace gr
