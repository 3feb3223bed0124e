// MT19937-64 packet engine and fused engine+transform kernels for sm_103a.
//
// Engine: each Vmt19937_64 has 4 MT19937-64 lanes (lane l = std::mt19937_64
// seeded seed+l), EigenRand/PacketRandomEngine.h:196-426.  One CTA owns one
// engine (or one jump-ahead segment of it): the 4 x 312-word lane states sit
// in shared memory, the twist runs in two phases of 156 independent words,
// and each thread tempers the 4 lane words of one packet index and turns them
// into output samples in registers, so raw bits never reach HBM.
//
// Jump-ahead: a segment starting e packets into the call gets its lane state
// from  window(a+e) = sum_i c_i * window(a+i),  c = x^e mod P(x)  (P the
// characteristic polynomial of MT19937-64), i.e. a GF(2) correlation of the
// polynomial's coefficients with the lane's next 20k raw words (the "prefix").
#include <cuda_runtime.h>

#include <cstdint>

#include "gr_exact.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_math.cuh"
#include "../../include/gpurand.h"

namespace gr {

__device__ __forceinline__ uint64_t twist1(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t t = (a & kUpper) | (b & kLower);
  return (t >> 1) ^ ((0ull - (t & 1ull)) & kMatA) ^ c;
}

__device__ __forceinline__ uint64_t temper(uint64_t r) {
  r ^= (r >> 29) & 0x5555555555555555ull;
  r ^= (r << 17) & 0x71d67fffeda60000ull;
  r ^= (r << 37) & 0xfff7eee000000000ull;
  r ^= r >> 43;
  return r;
}

// ---------------------------------------------------------------- seeding
// MersenneTwister::seed, PacketRandomEngine.h:256-265; engine k lane l is
// seeded seed + 4k + l.
__global__ void k_seed(EngState* st, int K, uint64_t seed) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= K * kLanes) return;
  int k = t / kLanes, l = t % kLanes;
  uint64_t prev = seed + (uint64_t)kLanes * (uint64_t)k + (uint64_t)l;
  uint64_t* w = st[k].win[l];
  w[0] = prev;
  for (int i = 1; i < kN; ++i) {
    prev = (prev ^ (prev >> 62)) * kSeedF + (uint64_t)i;
    w[i] = prev;
  }
  if (l == 0) {
    st[k].half_valid = 0;
    st[k].status = 0;
    st[k].consumed = 0;
    for (int q = 0; q < kLanes; ++q) st[k].half_cache[q] = 0;
  }
}

cudaError_t launch_seed(EngState* st, int K, uint64_t seed, cudaStream_t s) {
  int n = K * kLanes;
  k_seed<<<(n + 127) / 128, 128, 0, s>>>(st, K, seed);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- prefix
// prefix[k][l][0..312) = current window, then the raw recurrence
// x[i+312] = twist(x[i], x[i+1], x[i+156]) in chunks of 156 independent words.
// Also snapshots the caches the call starts from (block lane 0).
__global__ void __launch_bounds__(160) k_prefix(const EngState* st, uint64_t* prefix, CallSnap* snap,
                                                const GenState* gen) {
  __shared__ uint64_t ring[2 * kN];
  const int k = blockIdx.x / kLanes, l = blockIdx.x % kLanes;
  const int tid = threadIdx.x;
  uint64_t* out = prefix + ((size_t)k * kLanes + l) * kPrefixLen;
  for (int i = tid; i < kN; i += blockDim.x) {
    uint64_t v = st[k].win[l][i];
    ring[i] = v;
    out[i] = v;
  }
  if (l == 0 && tid == 0) {
    snap[k].half_valid = st[k].half_valid;
    for (int q = 0; q < kLanes; ++q) snap[k].half_cache[q] = st[k].half_cache[q];
    snap[k].gen_valid = gen ? gen[k].s[0].valid : 0;
    for (int q = 0; q < 16; ++q) snap[k].gen_cache[q] = gen ? gen[k].s[0].cache[q] : 0u;
  }
  __syncthreads();
  for (int base = 0; base + kN < kPrefixLen; base += kM) {
    if (tid < kM) {
      int i = base + tid;  // computes x[i+312]
      uint64_t a = ring[i % (2 * kN)], b = ring[(i + 1) % (2 * kN)], c = ring[(i + kM) % (2 * kN)];
      uint64_t v = twist1(a, b, c);
      ring[(i + kN) % (2 * kN)] = v;
      out[i + kN] = v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- jump
// One CTA per (engine k, segment s >= 1, lane l).  16 warps; warp g covers
// polynomial terms i in [1248 g, 1248 g + 1248), lane q of the warp covers
// output words j in [10 q, 10 q + 10).  Per 8 terms a thread loads 8 new
// prefix words into a sliding register window and XORs them into its 10
// accumulators under the (warp-uniform) coefficient bits.
constexpr int kJumpThreads = 512;
constexpr int kJumpPer = 1248;  // terms per warp (16 * 1248 = 19968 >= 19937)

__global__ void __launch_bounds__(kJumpThreads, 1)
    k_jump(const uint64_t* prefix, const uint64_t* polys, int S, uint64_t* segwin) {
  extern __shared__ uint64_t sm[];
  uint64_t* px = sm;                  // kPrefixLen words
  uint64_t* cf = sm + kPrefixLen;     // 312 coefficient words
  const int nseg = S - 1;
  const int l = blockIdx.x % kLanes;
  const int s1 = (blockIdx.x / kLanes) % nseg;  // segment - 1
  const int k = blockIdx.x / (kLanes * nseg);
  const int tid = threadIdx.x;
  const uint64_t* src = prefix + ((size_t)k * kLanes + l) * kPrefixLen;
  for (int i = tid; i < kPrefixLen / 2; i += kJumpThreads)
    reinterpret_cast<uint4*>(px)[i] = reinterpret_cast<const uint4*>(src)[i];
  for (int i = tid; i < kN; i += kJumpThreads) cf[i] = polys[(size_t)s1 * kN + i];
  __syncthreads();

  const int g = tid >> 5, q = tid & 31;
  const int j0 = 10 * q;
  uint64_t acc[10];
#pragma unroll
  for (int jj = 0; jj < 10; ++jj) acc[jj] = 0;
  uint64_t w[17];
  const int ibeg = g * kJumpPer;
#pragma unroll
  for (int m = 0; m < 9; ++m) w[m] = px[ibeg + j0 + m];
  for (int i0 = ibeg; i0 < ibeg + kJumpPer; i0 += 8) {
#pragma unroll
    for (int m = 0; m < 8; ++m) w[9 + m] = px[i0 + j0 + 9 + m];
    const uint32_t cb = (uint32_t)(cf[i0 >> 6] >> (i0 & 63)) & 0xffu;
    if (cb) {
#pragma unroll
      for (int ii = 0; ii < 8; ++ii) {
        if (cb & (1u << ii)) {
#pragma unroll
          for (int jj = 0; jj < 10; ++jj) acc[jj] ^= w[ii + jj];
        }
      }
    }
#pragma unroll
    for (int m = 0; m < 9; ++m) w[m] = w[m + 8];
  }
  __syncthreads();
  uint64_t* red = sm;  // reuse: [16][320]
#pragma unroll
  for (int jj = 0; jj < 10; ++jj) red[g * 320 + j0 + jj] = acc[jj];
  __syncthreads();
  uint64_t* dst = segwin + (((size_t)k * nseg + s1) * kLanes + l) * kN;
  for (int j = tid; j < kN; j += kJumpThreads) {
    uint64_t v = 0;
#pragma unroll
    for (int gg = 0; gg < 16; ++gg) v ^= red[gg * 320 + j];
    dst[j] = v;
  }
}

// ---------------------------------------------------------------- transforms
__device__ __forceinline__ float ur_f(uint32_t x) { return u2f((x & 0x7fffffu) | (127u << 23)) - 1.0f; }
__device__ __forceinline__ double ur_d(uint64_t x) {
  return u2d((x & 0xfffffffffffffull) | (1023ull << 52)) - 1.0;
}

// Truncated.h inverse-CDF forms, one lane: u is UniformRealGen(phi(lower),
// phi(upper))'s value.  TruncNormalGen::packetOp (:322-331), lognormal
// (:593-598), exponential (:477-484), Cauchy (:534-543), extreme value
// (:649-656), Weibull (:709-718).
template <int KIND>
__device__ __forceinline__ float trunc32(float u, const DistParams& d) {
  if (KIND == kTruncNormalKind || KIND == kTruncLognormalKind) {
    const float x = ((float)-1.4142135623730951 * erfinvf_(1.0f - 2.0f * u)) * d.fc + d.fd;
    return KIND == kTruncLognormalKind ? expf_(x) : x;
  }
  if (KIND == kTruncExponentialKind) return -logf_(1.0f - u) * d.fc;
  if (KIND == kTruncCauchyKind) {
    float s, c;
    sincosf_((float)3.1415926535897932 * (u - 0.5f), s, c);
    return d.fc + d.fd * (s / c);
  }
  if (KIND == kTruncExtremeKind) return d.fc - d.fd * logf_(-logf_(u));
  return d.fd * expf_(logf_(-logf_(1.0f - u)) * d.fc);  // Weibull
}

template <int KIND>
__device__ __forceinline__ double trunc64(double u, const DistParams& d) {
  if (KIND == kTruncNormalKind || KIND == kTruncLognormalKind) {
    const double x = (-1.4142135623730951 * erfinv_(1.0 - 2.0 * u)) * d.dc + d.dd;
    return KIND == kTruncLognormalKind ? exp_(x) : x;
  }
  if (KIND == kTruncExponentialKind) return -log_(1.0 - u) * d.dc;
  if (KIND == kTruncCauchyKind) {
    double s, c;
    sincos_(3.1415926535897932 * (u - 0.5), s, c);
    return d.dc + d.dd * (s / c);
  }
  if (KIND == kTruncExtremeKind) return d.dc - d.dd * log_(-log_(u));
  return d.dd * exp_(log_(-log_(1.0 - u)) * d.dc);
}

// float samples from one u32 word (one lane of a Packet8f), per kind.
template <int KIND>
__device__ __forceinline__ float tf32(uint32_t w, const DistParams& d) {
  if (KIND == GR_UNIFORM_REAL) return ur_f(w);
  if (KIND == GR_UNIFORM_REAL2) return ur_f(w) * d.fa + d.fb;
  if (KIND == GR_BALANCED || KIND == GR_BALANCED2) {
    float z = (float)(int32_t)(w & 0x7fffffffu) / (float)0x7FFFFFFF;
    return KIND == GR_BALANCED ? z * 2.0f - 1.0f : z * d.fa + d.fb;
  }
  if (KIND == GR_EXPONENTIAL) return -(logf_(1.0f - ur_f(w)) / d.fa);
  if (KIND == GR_GAMMA) return d.fb * (-(logf_(1.0f - ur_f(w)) / 1.0f));
  if (KIND == GR_CAUCHY) {
    float s, c;
    sincosf_((float)3.1415926535897932 * (ur_f(w) - 0.5f), s, c);
    return d.fa + d.fb * (s / c);
  }
  if (KIND == GR_WEIBULL) return expf_(logf_(-logf_(1.0f - ur_f(w))) * d.fa) * d.fb;
  if (KIND == GR_EXTREME_VALUE) return d.fa - logf_(-logf_(ur_f(w) + 1.1920928955078125e-07f / 8)) * d.fb;
  // BernoulliGen<float>: the word of the lane, masked, compared signed
  if (KIND == GR_BERNOULLI) return ((int32_t)(w & 0x7fffffffu) < d.ia) ? 1.0f : 0.0f;
  if (KIND >= kTruncNormalKind && KIND <= kTruncWeibullKind) return trunc32<KIND>(ur_f(w) * d.fa + d.fb, d);
  return 0.0f;
}

template <int KIND>
__device__ __forceinline__ double tf64(uint64_t r, const DistParams& d) {
  if (KIND == GR_UNIFORM_REAL) return ur_d(r);
  if (KIND == GR_UNIFORM_REAL2) return ur_d(r) * d.da + d.db;
  if (KIND == GR_EXPONENTIAL) {
    const double l = log_(one_minus_ur_d(r));
    return (d.flags & kParamUnitDiv) ? -l : -(l / d.da);
  }
  if (KIND == GR_GAMMA) {
    const double l = -(log_(one_minus_ur_d(r)) / 1.0);
    return (d.flags & kParamUnitScale) ? l : d.db * l;
  }
  if (KIND == GR_CAUCHY) {
    double s, c;
    sincos_(3.1415926535897932 * (ur_d(r) - 0.5), s, c);
    return d.da + d.db * (s / c);
  }
  if (KIND == GR_WEIBULL) {
    const double w = exp_(log_(-log_(one_minus_ur_d(r))) * d.da);
    return (d.flags & kParamUnitScale) ? w : w * d.db;
  }
  if (KIND == GR_EXTREME_VALUE) return d.da - log_(-log_(ur_d(r) + 2.220446049250313e-16 / 8)) * d.db;
  // BernoulliGen<double>: the compare runs on the eight 32-bit words and the
  // blend reads each 64-bit element's sign, the compare of its high word
  if (KIND == GR_BERNOULLI) return ((int32_t)((uint32_t)(r >> 32) & 0x7fffffffu) < d.ia) ? 1.0 : 0.0;
  if (KIND >= kTruncNormalKind && KIND <= kTruncWeibullKind) return trunc64<KIND>(ur_d(r) * d.da + d.db, d);
  return 0.0;
}

// double balanced from one u32 word (rng.half() path); the quotient by
// 2^31 - 1 in integer form (gr_exact.h), bit-identical to the division
template <int KIND>
__device__ __forceinline__ double tw64(uint32_t w, const DistParams& d) {
  double z = div_2p31m1(w & 0x7fffffffu);
  return KIND == GR_BALANCED ? z * 2.0 - 1.0 : z * d.da + d.db;
}

template <int KIND>
__device__ __forceinline__ int32_t tw32(uint32_t w, const DistParams& d) {
  if (KIND == GR_RANDBITS) return (int32_t)w;
  if (KIND == GR_BERNOULLI) return ((int32_t)(w & 0x7fffffffu) < d.ia) ? 1 : 0;
  // UniformIntGen<int32_t> over a power-of-two range: (rx & bitmask) + pmin (Discrete.h:302-305)
  if (KIND == GR_UNIFORM_INT) return (int32_t)((w & d.bitmask) + (uint32_t)d.ia);
  // GeometricGen<int32_t>: pcast(ptruncate(plog(1 - u) * rlog_q)), Discrete.h:1368-1374
  if (KIND == GR_GEOMETRIC) return cvtt_f32(truncf(logf_(1.0f - ur_f(w)) * d.fa));
  // DiscreteGen<int32_t,int32_t>, Discrete.h:455-470
  if (d.ncdf > 0) {
    int32_t r = d.ncdf - 1;
    int32_t x = (int32_t)(w & 0x7fffffffu);
    for (int i = 0; i < d.ncdf - 1; ++i) r += (x < __ldg(d.prob + i)) ? -1 : 0;
    return r;
  }
  int32_t albit = (int32_t)(w & d.bitmask);
  return ((int32_t)(w >> 1) < __ldg(d.prob + albit)) ? albit : __ldg(d.alias + albit);
}

template <int KIND>
__device__ __forceinline__ float nscale32(float x, const DistParams& d) {
  if (KIND == GR_NORMAL_STD) return x;
  if (KIND == GR_NORMAL) return x * d.fb + d.fa;
  return expf_(x * d.fb + d.fa);  // lognormal
}
template <int KIND>
__device__ __forceinline__ double nscale64(double x, const DistParams& d) {
  if (KIND == GR_NORMAL_STD) return x;
  if (KIND == GR_NORMAL) return x * d.db + d.da;
  return exp_(x * d.db + d.da);
}

// ---------------------------------------------------------------- per-element forms
// The *VGen packetOp arguments of output element idx, mapped onto the
// constants the scalar-parameter transform reads: UniformRealVGen and
// BalancedVGen slope b - a, bias a (Basic.h:486-491, :660-665); NormalVGen and
// LognormalVGen mean a, stdev b (NormalExp.h:155-162, :230-235);
// ExponentialVGen lambda a (:420-426); WeibullVGen 1 / a and b (:679-685);
// ExtremeValueVGen and CauchyVGen a, b (:757-764, :879-888).  Each is the
// same packet arithmetic as the scalar generator with the lane's own values.
template <int BK>
__device__ __forceinline__ DistParams vparams32(const DistParams& d, int64_t idx) {
  const float a = (d.flags & kParamVecA) ? __ldg(static_cast<const float*>(d.vparam) + idx) : d.fe;
  const float b = (d.flags & kParamVecB) ? __ldg(static_cast<const float*>(d.vparam2) + idx) : d.ff;
  DistParams e = d;
  e.flags = 0;
  if (BK == GR_UNIFORM_REAL2 || BK == GR_BALANCED2) {
    e.fa = b - a;
    e.fb = a;
  } else if (BK == GR_WEIBULL) {
    e.fa = 1.0f / a;
    e.fb = b;
  } else {
    e.fa = a;
    e.fb = b;
  }
  return e;
}
template <int BK>
__device__ __forceinline__ DistParams vparams64(const DistParams& d, int64_t idx) {
  const double a = (d.flags & kParamVecA) ? __ldg(static_cast<const double*>(d.vparam) + idx) : d.de;
  const double b = (d.flags & kParamVecB) ? __ldg(static_cast<const double*>(d.vparam2) + idx) : d.df;
  DistParams e = d;
  e.flags = 0;
  if (BK == GR_UNIFORM_REAL2 || BK == GR_BALANCED2) {
    e.da = b - a;
    e.db = a;
  } else if (BK == GR_WEIBULL) {
    e.da = 1.0 / a;
    e.db = b;
  } else {
    e.da = a;
    e.db = b;
  }
  return e;
}

// Transforms with the output element index: a per-element kind reads its
// parameters there, the others ignore it.
template <int KIND>
__device__ __forceinline__ float tf32i(uint32_t w, const DistParams& d, int64_t idx) {
  if constexpr (KIND >= kVecBase) return tf32<KIND - kVecBase>(w, vparams32<KIND - kVecBase>(d, idx));
  else return tf32<KIND>(w, d);
}
template <int KIND>
__device__ __forceinline__ double tf64i(uint64_t r, const DistParams& d, int64_t idx) {
  if constexpr (KIND >= kVecBase) return tf64<KIND - kVecBase>(r, vparams64<KIND - kVecBase>(d, idx));
  else return tf64<KIND>(r, d);
}
template <int KIND>
__device__ __forceinline__ double tw64i(uint32_t w, const DistParams& d, int64_t idx) {
  if constexpr (KIND >= kVecBase) return tw64<KIND - kVecBase>(w, vparams64<KIND - kVecBase>(d, idx));
  else return tw64<KIND>(w, d);
}
template <int KIND>
__device__ __forceinline__ float nscale32i(float x, const DistParams& d, int64_t idx) {
  if constexpr (KIND >= kVecBase) return nscale32<KIND - kVecBase>(x, vparams32<KIND - kVecBase>(d, idx));
  else return nscale32<KIND>(x, d);
}
template <int KIND>
__device__ __forceinline__ double nscale64i(double x, const DistParams& d, int64_t idx) {
  if constexpr (KIND >= kVecBase) return nscale64<KIND - kVecBase>(x, vparams64<KIND - kVecBase>(d, idx));
  else return nscale64<KIND>(x, d);
}

// ---------------------------------------------------------------- direct kernel
// M_RAW2 / M_F32H / M_F64H: the 2-lane Vmt19937_64 (SSE / NEON profile,
// Pmt19937_64<Packet4i>): its packets are the first two lanes of the 4-lane
// engine with the same seed, a Packet4f (4 floats) or Packet2d (2 doubles)
// per packet; the other two lanes are made and left unused.
enum Mode { M_RAW, M_F32, M_F64, M_W32, M_W64, M_N32, M_N64, M_RAW0, M_RAW2, M_F32H, M_F64H };

template <int MODE>
struct ModeInfo {
  static constexpr int OPP = (MODE == M_RAW || MODE == M_RAW0) ? 4 : MODE == M_F32 ? 8 : MODE == M_F64 ? 4 : MODE == M_N32 ? 8 : MODE == M_N64 ? 4
                           : MODE == M_RAW2 ? 2 : MODE == M_F32H ? 4 : MODE == M_F64H ? 2 : 8;
  static constexpr bool kHalfCache = MODE == M_W64;  // randbits handled separately below
  static constexpr int kCacheOut = MODE == M_N32 ? 8 : MODE == M_N64 ? 4 : (MODE == M_W32 || MODE == M_W64) ? 4 : 0;
};

__device__ __forceinline__ void st16(void* p, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  *reinterpret_cast<uint4*>(p) = make_uint4(a, b, c, d);
}

template <int MODE, int KIND>
__global__ void __maxnreg__(64) k_direct(Plan p, DistParams d, const CallSnap* snap) {
  __shared__ uint64_t raw[2][kLanes][kN];
  const int k = blockIdx.x / p.S, s = blockIdx.x % p.S;
  const int tid = threadIdx.x;
  EngState* st = p.eng + k;
  GenState* gs = p.gen ? p.gen + k : nullptr;

  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;

  // --- caches the call starts from
  // int32 kinds whose packets are rng.half() words leave raw words in the
  // engine's half cache; DiscreteGen caches its own computed results
  constexpr bool kHalfKind =
      KIND == GR_RANDBITS || KIND == GR_BERNOULLI || KIND == GR_GEOMETRIC || KIND == GR_UNIFORM_INT;
  constexpr bool kUsesHalf = (MODE == M_W64) || (MODE == M_W32 && kHalfKind);
  constexpr bool kUsesGen = (MODE == M_N32) || (MODE == M_N64) || (MODE == M_W32 && KIND == GR_DISCRETE);
  int cvalid = 0;
  const uint32_t* cwords = nullptr;
  if (kUsesHalf) {
    cvalid = p.S > 1 ? snap[k].half_valid : st->half_valid;
    cwords = p.S > 1 ? snap[k].half_cache : st->half_cache;
  } else if (kUsesGen) {
    cvalid = p.S > 1 ? snap[k].gen_valid : gs->s[0].valid;
    cwords = p.S > 1 ? snap[k].gen_cache : gs->s[0].cache;
  }
  constexpr int CO = ModeInfo<MODE>::kCacheOut;
  const int64_t Q0 = (cvalid && CO) ? min((int64_t)CO, n) : 0;
  const int64_t r = n - Q0;
  constexpr int OPP = ModeInfo<MODE>::OPP;  // outputs per packet (N modes: per packet of a 2-packet unit)
  const int64_t Np = (MODE == M_N32 || MODE == M_N64) ? 2 * ((r + 2 * OPP - 1) / (2 * OPP)) : (r + OPP - 1) / OPP;
  const int64_t pbeg = (int64_t)s * p.J;
  const int64_t pend = min(pbeg + p.J, Np);
  const bool last = (pbeg < Np && Np <= pbeg + p.J) || (Np == 0 && s == 0);
  if (pbeg >= Np && !(Np == 0 && s == 0)) return;

  // --- prefix outputs served from the cache (segment 0 only)
  if (s == 0 && tid < Q0) {
    const int i = tid;
    if (MODE == M_W64) reinterpret_cast<double*>(p.out)[off + i] = tw64i<KIND>(cwords[i], d, off + i);
    if (MODE == M_W32)
      reinterpret_cast<int32_t*>(p.out)[off + i] = kHalfKind ? tw32<KIND>(cwords[i], d) : (int32_t)cwords[i];
    if (MODE == M_N32) reinterpret_cast<float*>(p.out)[off + i] = nscale32i<KIND>(u2f(cwords[i]), d, off + i);
    if (MODE == M_N64) {
      uint64_t b = (uint64_t)cwords[2 * i] | ((uint64_t)cwords[2 * i + 1] << 32);
      reinterpret_cast<double*>(p.out)[off + i] = nscale64i<KIND>(u2d(b), d, off + i);
    }
  }

  // --- lane windows.  With several segments the last one rewrites st->win,
  // so segment 0 reads the copy the prefix kernel made at call start.
  if (s == 0 && p.S > 1) {
    for (int i = tid; i < kLanes * kN; i += blockDim.x)
      (&raw[0][0][0])[i] = p.prefix[((size_t)k * kLanes + i / kN) * kPrefixLen + i % kN];
  } else {
    const uint64_t* w0 = (s == 0) ? &st->win[0][0] : p.segwin + ((size_t)k * (p.S - 1) + (s - 1)) * kLanes * kN;
    for (int i = tid; i < kLanes * kN; i += blockDim.x) (&raw[0][0][0])[i] = w0[i];
  }
  __syncthreads();

  const int64_t obase = off + Q0;
  const int64_t oend = off + n;
  int cur = 0;
  int64_t base = pbeg;
  for (; base < pend; base += kN) {
    uint64_t(*old)[kN] = raw[cur];
    uint64_t(*nw)[kN] = raw[cur ^ 1];
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
      const int i = ph * kM + tid;
      uint64_t pk[kLanes];
      const bool act = tid < kM;
      if (act) {
#pragma unroll
        for (int l = 0; l < kLanes; ++l) {
          uint64_t b = (i + 1 < kN) ? old[l][i + 1] : nw[l][0];
          uint64_t c = (ph == 0) ? old[l][i + kM] : nw[l][i - kM];
          uint64_t v = twist1(old[l][i], b, c);
          nw[l][i] = v;
          pk[l] = temper(v);
        }
      } else {
#pragma unroll
        for (int l = 0; l < kLanes; ++l) pk[l] = 0;
      }
      const int64_t pidx = base + i;
      const bool valid = act && pidx < pend;
      // ---- emit
      if (MODE == M_RAW) {
        if (valid && p.out) {  // p.out == nullptr: discard
          uint64_t* o = reinterpret_cast<uint64_t*>(p.out) + obase + pidx * 4;
          reinterpret_cast<ulonglong2*>(o)[0] = make_ulonglong2(pk[0], pk[1]);
          reinterpret_cast<ulonglong2*>(o)[1] = make_ulonglong2(pk[2], pk[3]);
        }
      } else if (MODE == M_RAW2) {
        if (valid && p.out)
          reinterpret_cast<ulonglong2*>(reinterpret_cast<uint64_t*>(p.out) + obase + pidx * 2)[0] =
              make_ulonglong2(pk[0], pk[1]);
      } else if (MODE == M_F32H) {
        if (valid) {
          float* o = reinterpret_cast<float*>(p.out) + obase + pidx * 4;
          const int64_t ib = obase + pidx * 4;
          reinterpret_cast<float4*>(o)[0] =
              make_float4(tf32i<KIND>((uint32_t)pk[0], d, ib), tf32i<KIND>((uint32_t)(pk[0] >> 32), d, ib + 1),
                          tf32i<KIND>((uint32_t)pk[1], d, ib + 2), tf32i<KIND>((uint32_t)(pk[1] >> 32), d, ib + 3));
        }
      } else if (MODE == M_F64H) {
        if (valid) {
          double* o = reinterpret_cast<double*>(p.out) + obase + pidx * 2;
          const int64_t ib = obase + pidx * 2;
          reinterpret_cast<double2*>(o)[0] = make_double2(tf64i<KIND>(pk[0], d, ib), tf64i<KIND>(pk[1], d, ib + 1));
        }
      } else if (MODE == M_RAW0) {
        // a scalar draw takes the engine's whole packet and keeps its first
        // element (StdUniformRealGen::operator(), Dists/Basic.h:533-540)
        if (valid) reinterpret_cast<uint64_t*>(p.out)[obase / 4 + pidx] = pk[0];
      } else if (MODE == M_F32) {
        if (valid) {
          float* o = reinterpret_cast<float*>(p.out) + obase + pidx * 8;
          float v[8];
          if (KIND == kBernoulliVKind) {
            // BernoulliVGen<float>: p = cvttps(a * 2^31), compared signed with
            // the masked word (Basic.h:735-745)
            const float4* pv = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(d.vparam) + obase + pidx * 8);
            const float4 q0 = pv[0], q1 = pv[1];
            const float pa[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const uint32_t w = (q & 1) ? (uint32_t)(pk[q >> 1] >> 32) : (uint32_t)pk[q >> 1];
              v[q] = ((int32_t)(w & 0x7fffffffu) < cvtt_f32(pa[q] * 2147483648.0f)) ? 1.0f : 0.0f;
            }
          } else {
#pragma unroll
            for (int l = 0; l < kLanes; ++l) {
              v[2 * l] = tf32i<KIND>((uint32_t)pk[l], d, obase + pidx * 8 + 2 * l);
              v[2 * l + 1] = tf32i<KIND>((uint32_t)(pk[l] >> 32), d, obase + pidx * 8 + 2 * l + 1);
            }
          }
          reinterpret_cast<float4*>(o)[0] = make_float4(v[0], v[1], v[2], v[3]);
          reinterpret_cast<float4*>(o)[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
      } else if (MODE == M_F64) {
        if (valid) {
          double* o = reinterpret_cast<double*>(p.out) + obase + pidx * 4;
          double v[4];
#pragma unroll
          for (int l = 0; l < kLanes; ++l) v[l] = tf64i<KIND>(pk[l], d, obase + pidx * 4 + l);
          reinterpret_cast<double2*>(o)[0] = make_double2(v[0], v[1]);
          reinterpret_cast<double2*>(o)[1] = make_double2(v[2], v[3]);
        }
      } else if (MODE == M_W32 || MODE == M_W64) {
        if (valid) {
          const int64_t ob = obase + pidx * 8;
          uint32_t wd[8];
#pragma unroll
          for (int l = 0; l < kLanes; ++l) {
            wd[2 * l] = (uint32_t)pk[l];
            wd[2 * l + 1] = (uint32_t)(pk[l] >> 32);
          }
          const bool full = ob + 8 <= oend;
          if (MODE == M_W32) {
            int32_t v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = tw32<KIND>(wd[q], d);
            int32_t* o = reinterpret_cast<int32_t*>(p.out) + ob;
            st16(o, v[0], v[1], v[2], v[3]);
            if (full) st16(o + 4, v[4], v[5], v[6], v[7]);
            else if (gs || kHalfKind) {
              // leftover half: rng.half() kinds leave raw words in the engine's
              // half() cache; DiscreteGen caches its computed upper 4 results
              uint32_t* cdst = kHalfKind ? st->half_cache : gs->s[0].cache;
#pragma unroll
              for (int q = 0; q < 4; ++q) cdst[q] = kHalfKind ? wd[4 + q] : (uint32_t)v[4 + q];
            }
          } else {
            double v[8];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = tw64i<KIND>(wd[q], d, ob + q);
            double* o = reinterpret_cast<double*>(p.out) + ob;
            reinterpret_cast<double2*>(o)[0] = make_double2(v[0], v[1]);
            reinterpret_cast<double2*>(o)[1] = make_double2(v[2], v[3]);
            if (full) {
#pragma unroll
              for (int q = 4; q < 8; ++q) v[q] = tw64i<KIND>(wd[q], d, ob + q);
              reinterpret_cast<double2*>(o)[2] = make_double2(v[4], v[5]);
              reinterpret_cast<double2*>(o)[3] = make_double2(v[6], v[7]);
            } else {
#pragma unroll
              for (int q = 0; q < 4; ++q) st->half_cache[q] = wd[4 + q];
            }
          }
        }
      } else if (MODE == M_N32) {
        // unit = packets (2j, 2j+1): u1 words in the even thread, u2 in the odd.
        // Even thread handles lanes i = 0..3 of the unit, odd handles 4..7.
        const bool odd = (tid & 1);
        uint32_t wd[8];
#pragma unroll
        for (int l = 0; l < kLanes; ++l) {
          wd[2 * l] = (uint32_t)pk[l];
          wd[2 * l + 1] = (uint32_t)(pk[l] >> 32);
        }
        uint32_t other[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) other[q] = __shfl_xor_sync(0xffffffffu, odd ? wd[q] : wd[4 + q], 1);
        if (valid) {
          const int64_t unit = pidx >> 1;
          const int i0 = odd ? 4 : 0;
          float sv[4], cv[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float u1 = ur_f(odd ? other[q] : wd[q]);
            const float u2 = ur_f(odd ? wd[4 + q] : other[q]);
            const float radius = sqrtf((float)-2 * logf_(1.0f - u1));
            const float theta = (float)(2 * 3.1415926535897932) * u2;
            float sn, cs;
            sincosf_(theta, sn, cs);
            sv[q] = radius * sn;
            cv[q] = radius * cs;
          }
          const int64_t ob = obase + unit * 16;
          float* o = reinterpret_cast<float*>(p.out) + ob;
          reinterpret_cast<float4*>(o + i0)[0] =
              make_float4(nscale32i<KIND>(sv[0], d, ob + i0), nscale32i<KIND>(sv[1], d, ob + i0 + 1),
                          nscale32i<KIND>(sv[2], d, ob + i0 + 2), nscale32i<KIND>(sv[3], d, ob + i0 + 3));
          if (ob + 16 <= oend) {
            reinterpret_cast<float4*>(o + 8 + i0)[0] =
                make_float4(nscale32i<KIND>(cv[0], d, ob + 8 + i0), nscale32i<KIND>(cv[1], d, ob + 9 + i0),
                            nscale32i<KIND>(cv[2], d, ob + 10 + i0), nscale32i<KIND>(cv[3], d, ob + 11 + i0));
          } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) gs->s[0].cache[i0 + q] = f2u(cv[q]);
          }
        }
      } else if (MODE == M_N64) {
        const bool odd = (tid & 1);
        uint64_t other[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          uint64_t sendv = odd ? pk[q] : pk[2 + q];
          other[q] = ((uint64_t)__shfl_xor_sync(0xffffffffu, (uint32_t)(sendv >> 32), 1) << 32) |
                     (uint64_t)__shfl_xor_sync(0xffffffffu, (uint32_t)sendv, 1);
        }
        if (valid) {
          const int64_t unit = pidx >> 1;
          const int i0 = odd ? 2 : 0;
          double sv[2], cv[2];
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const double u2 = ur_d(odd ? pk[2 + q] : other[q]);
            const double radius = sqrt(-2.0 * log_(one_minus_ur_d(odd ? other[q] : pk[q])));
            const double theta = (2 * 3.1415926535897932) * u2;
            double sn, cs;
            sincos_(theta, sn, cs);
            sv[q] = radius * sn;
            cv[q] = radius * cs;
          }
          const int64_t ob = obase + unit * 8;
          double* o = reinterpret_cast<double*>(p.out) + ob;
          reinterpret_cast<double2*>(o + i0)[0] =
              make_double2(nscale64i<KIND>(sv[0], d, ob + i0), nscale64i<KIND>(sv[1], d, ob + i0 + 1));
          if (ob + 8 <= oend) {
            reinterpret_cast<double2*>(o + 4 + i0)[0] =
                make_double2(nscale64i<KIND>(cv[0], d, ob + 4 + i0), nscale64i<KIND>(cv[1], d, ob + 5 + i0));
          } else {
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              uint64_t b = d2u(cv[q]);
              gs->s[0].cache[2 * (i0 + q)] = (uint32_t)b;
              gs->s[0].cache[2 * (i0 + q) + 1] = (uint32_t)(b >> 32);
            }
          }
        }
      }
      __syncthreads();
    }
    cur ^= 1;
  }

  // --- end-of-call state: new lane windows and cache flags
  if (last) {
    if (Np > 0) {
      const int64_t nb = (pend - pbeg + kN - 1) / kN;
      const int rr = (int)(pend - (pbeg + (nb - 1) * kN));  // packets used of the last block, 1..312
      uint64_t(*lastb)[kN] = raw[cur];
      uint64_t(*prevb)[kN] = raw[cur ^ 1];
      for (int t = tid; t < kLanes * kN; t += blockDim.x) {
        const int l = t / kN, i = t % kN;
        st->win[l][i] = (i < kN - rr) ? prevb[l][rr + i] : lastb[l][i - (kN - rr)];
      }
    }
    if (tid == 0) {
      int64_t left = 0;  // leftover outputs cached for the next call
      if (MODE == M_W32 || MODE == M_W64) left = (r % 8) ? 4 : 0;
      if (MODE == M_N32) left = (r % 16) ? 8 : 0;
      if (MODE == M_N64) left = (r % 8) ? 4 : 0;
      if (kUsesHalf) st->half_valid = left ? 1 : (Q0 ? 0 : st->half_valid);
      if (kUsesGen) gs->s[0].valid = left ? 1 : 0;
      st->consumed += (uint64_t)Np;
    }
  }
}

template <int MODE, int KIND>
static cudaError_t run_direct(const Plan& p, const DistParams& d, const CallSnap* snap, cudaStream_t s) {
  k_direct<MODE, KIND><<<p.K * p.S, 160, 0, s>>>(p, d, snap);
  return cudaGetLastError();
}

cudaError_t launch_prefix(const EngState* st, const GenState* gen, int K, uint64_t* prefix, CallSnap* snap,
                          cudaStream_t s) {
  k_prefix<<<K * kLanes, 160, 0, s>>>(st, prefix, snap, gen);
  return cudaGetLastError();
}

static constexpr size_t kJumpSmem = (size_t)(kPrefixLen + kN) * sizeof(uint64_t);

// k_jump's dynamic shared-memory limit, set once per device.
static cudaError_t jump_attr() {
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_jump, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kJumpSmem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  return cudaSuccess;
}

cudaError_t launch_jump(const uint64_t* prefix, const uint64_t* polys, int K, int S, uint64_t* segwin,
                        cudaStream_t s) {
  if (S <= 1) return cudaSuccess;
  cudaError_t e = jump_attr();
  if (e != cudaSuccess) return e;
  k_jump<<<K * (S - 1) * kLanes, kJumpThreads, kJumpSmem, s>>>(prefix, polys, S, segwin);
  return cudaGetLastError();
}

cudaError_t preload_raw_stream_kernels() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k_prefix);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_jump);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_direct<M_RAW, kRawKind>);
  if (e == cudaSuccess) e = jump_attr();
  return e;
}

// ---------------------------------------------------------------- scalar tails
// A size that is not a whole number of packets ends with n % P elements made
// by the generator's scalar operator() (Eigen's linear vectorised assignment
// loop: packets up to the last whole one, then scalars).  Each takes one draw:
// the first 64-bit lane of an engine packet (pfirst of the packet), or one
// draw of a scalar engine.  Exact bit arithmetic for these kinds:
// randBits (Basic.h:386-391), balanced (:416-420), balanced(a, b)
// (:456-460), uniformReal (:533-540, ExtractFirstUint :345-371),
// uniformReal(min, max) (:620-624), bernoulli (:689-693).
bool kind_has_exact_tail(int kind, int dtype) {
  switch (kind) {
    case GR_UNIFORM_REAL:
    case GR_UNIFORM_REAL2:
    case GR_BALANCED:
    case GR_BALANCED2:
      return dtype == GR_F32 || dtype == GR_F64;
    case GR_BERNOULLI:
      return true;
    case GR_RANDBITS:
      return dtype == GR_I32;
    default:
      return false;
  }
}

__global__ void k_tail(const uint64_t* w, void* out, int n, DistParams d, int packet_engine) {
  const int i = threadIdx.x;
  if (i >= n) return;
  const uint64_t r = w[i];
  const uint32_t lo = (uint32_t)r;
  // pfirst of an engine packet is its first 32-bit word; of a scalar engine's
  // draw, the whole 64-bit value
  const uint64_t first = packet_engine ? (uint64_t)(int64_t)(int32_t)lo : r;
  const bool f64 = d.dtype == GR_F64;
  switch (d.kind) {
    case GR_UNIFORM_REAL:
      // ExtractFirstUint: the first 32-bit word (float), the first 64-bit lane (double)
      if (f64) reinterpret_cast<double*>(out)[i] = ur_d(r);
      else reinterpret_cast<float*>(out)[i] = ur_f(lo);
      break;
    case GR_UNIFORM_REAL2:  // bias + to_ur(pfirst(rng())) * slope
      if (f64) reinterpret_cast<double*>(out)[i] = d.db + ur_d(first) * d.da;
      else reinterpret_cast<float*>(out)[i] = d.fb + ur_f(lo) * d.fa;
      break;
    case GR_BALANCED:
    case GR_BALANCED2: {
      const uint32_t k = lo & 0x7fffffffu;
      if (f64) {
        const double z = div_2p31m1(k);
        reinterpret_cast<double*>(out)[i] = d.kind == GR_BALANCED ? z * 2.0 - 1.0 : z * d.da + d.db;
      } else {
        const float z = (float)(int32_t)k / (float)0x7FFFFFFF;
        reinterpret_cast<float*>(out)[i] = d.kind == GR_BALANCED ? z * 2.0f - 1.0f : z * d.fa + d.fb;
      }
      break;
    }
    case GR_BERNOULLI: {
      const int v = ((int32_t)(lo & 0x7fffffffu) < d.ia) ? 1 : 0;
      if (d.dtype == GR_I32) reinterpret_cast<int32_t*>(out)[i] = v;
      else if (f64) reinterpret_cast<double*>(out)[i] = v;
      else reinterpret_cast<float*>(out)[i] = (float)v;
      break;
    }
    case GR_RANDBITS:
      reinterpret_cast<int32_t*>(out)[i] = (int32_t)lo;
      break;
    default:
      break;
  }
}

cudaError_t launch_tail(const uint64_t* w, void* out, int n, const DistParams& d, bool packet_engine, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_tail<<<1, 32, 0, s>>>(w, out, n, d, packet_engine ? 1 : 0);
  return cudaGetLastError();
}

int kind_granule(int kind, int dtype) {
  if (kind == kRawKind || kind == kRawLane0Kind) return 4;
  if (dtype == GR_F32) return 8;
  return 4;  // double packets and int32 packets hold 4 lanes
}

int kind_packets_per_unit(int kind, int dtype) {
  (void)dtype;
  if (kind >= kVecBase) kind -= kVecBase;
  if (kind == GR_NORMAL_STD || kind == GR_NORMAL || kind == GR_LOGNORMAL) return 2;
  return 1;
}

bool kind_is_direct(int kind, int dtype, const DistParams& d) {
  switch (kind) {
    case kRawKind:
    case kRawLane0Kind:
    case GR_UNIFORM_REAL:
    case GR_UNIFORM_REAL2:
    case GR_BALANCED:
    case GR_BALANCED2:
    case GR_NORMAL_STD:
    case GR_NORMAL:
    case GR_LOGNORMAL:
    case GR_EXPONENTIAL:
    case GR_CAUCHY:
    case GR_WEIBULL:
    case GR_EXTREME_VALUE:
      return true;
    case GR_GAMMA:
      return d.ia == 1;  // alpha == 1: beta * exponential
    case GR_BERNOULLI:
      return true;
    case kTruncNormalKind:
    case kTruncLognormalKind:
    case kTruncExponentialKind:
    case kTruncCauchyKind:
    case kTruncExtremeKind:
    case kTruncWeibullKind:
      return dtype == GR_F32 || dtype == GR_F64;
    case kBernoulliVKind:
      return dtype == GR_F32;
    case kVecBase + GR_UNIFORM_REAL2:
    case kVecBase + GR_BALANCED2:
    case kVecBase + GR_NORMAL:
    case kVecBase + GR_LOGNORMAL:
    case kVecBase + GR_EXPONENTIAL:
    case kVecBase + GR_WEIBULL:
    case kVecBase + GR_EXTREME_VALUE:
    case kVecBase + GR_CAUCHY:
      return dtype == GR_F32 || dtype == GR_F64;
    case GR_RANDBITS:
    case GR_DISCRETE:
    case GR_GEOMETRIC:
      return dtype == GR_I32;
    case GR_UNIFORM_INT:
      return dtype == GR_I32 && d.ib == 1;
    default:
      return false;
  }
}

#define GR_F32_CASE(K) \
  case K:              \
    return run_direct<M_F32, K>(p, d, snap, s);
#define GR_F64_CASE(K) \
  case K:              \
    return run_direct<M_F64, K>(p, d, snap, s);

bool kind_two_lane(int kind, int dtype) {
  if (kind == kRawKind) return true;
  switch (kind) {
    case GR_UNIFORM_REAL:
    case GR_UNIFORM_REAL2:
    case GR_EXPONENTIAL:
    case GR_CAUCHY:
    case GR_WEIBULL:
    case GR_EXTREME_VALUE:
    case GR_GAMMA:  // alpha == 1 (the caller checks)
      return dtype == GR_F32 || dtype == GR_F64;
    case GR_BALANCED:
    case GR_BALANCED2:
    case GR_BERNOULLI:
      return dtype == GR_F32;
    default:
      return false;
  }
}

#define GR_F32H_CASE(K) \
  case K:               \
    return run_direct<M_F32H, K>(p, d, snap, s);
#define GR_F64H_CASE(K) \
  case K:               \
    return run_direct<M_F64H, K>(p, d, snap, s);

cudaError_t launch_direct(const Plan& p, const DistParams& d, const CallSnap* snap, cudaStream_t s) {
  if (d.flags & kParamTwoLane) {
    if (d.kind == kRawKind) return run_direct<M_RAW2, kRawKind>(p, d, snap, s);
    if (d.dtype == GR_F32) {
      switch (d.kind) {
        GR_F32H_CASE(GR_UNIFORM_REAL)
        GR_F32H_CASE(GR_UNIFORM_REAL2)
        GR_F32H_CASE(GR_BALANCED)
        GR_F32H_CASE(GR_BALANCED2)
        GR_F32H_CASE(GR_EXPONENTIAL)
        GR_F32H_CASE(GR_CAUCHY)
        GR_F32H_CASE(GR_WEIBULL)
        GR_F32H_CASE(GR_EXTREME_VALUE)
        GR_F32H_CASE(GR_GAMMA)
        GR_F32H_CASE(GR_BERNOULLI)
        default:
          return cudaErrorNotSupported;
      }
    }
    if (d.dtype == GR_F64) {
      switch (d.kind) {
        GR_F64H_CASE(GR_UNIFORM_REAL)
        GR_F64H_CASE(GR_UNIFORM_REAL2)
        GR_F64H_CASE(GR_EXPONENTIAL)
        GR_F64H_CASE(GR_CAUCHY)
        GR_F64H_CASE(GR_WEIBULL)
        GR_F64H_CASE(GR_EXTREME_VALUE)
        GR_F64H_CASE(GR_GAMMA)
        default:
          return cudaErrorNotSupported;
      }
    }
    return cudaErrorNotSupported;
  }
  if (d.kind == kRawKind) return run_direct<M_RAW, kRawKind>(p, d, snap, s);
  if (d.kind == kRawLane0Kind) return run_direct<M_RAW0, kRawLane0Kind>(p, d, snap, s);
  if (d.dtype == GR_F32) {
    switch (d.kind) {
      GR_F32_CASE(GR_UNIFORM_REAL)
      GR_F32_CASE(GR_UNIFORM_REAL2)
      GR_F32_CASE(GR_BALANCED)
      GR_F32_CASE(GR_BALANCED2)
      GR_F32_CASE(GR_EXPONENTIAL)
      GR_F32_CASE(GR_CAUCHY)
      GR_F32_CASE(GR_WEIBULL)
      GR_F32_CASE(GR_EXTREME_VALUE)
      GR_F32_CASE(GR_GAMMA)
      GR_F32_CASE(GR_BERNOULLI)
      GR_F32_CASE(kBernoulliVKind)
      GR_F32_CASE(kTruncNormalKind)
      GR_F32_CASE(kTruncLognormalKind)
      GR_F32_CASE(kTruncExponentialKind)
      GR_F32_CASE(kTruncCauchyKind)
      GR_F32_CASE(kTruncExtremeKind)
      GR_F32_CASE(kTruncWeibullKind)
      GR_F32_CASE(kVecBase + GR_UNIFORM_REAL2)
      GR_F32_CASE(kVecBase + GR_BALANCED2)
      GR_F32_CASE(kVecBase + GR_EXPONENTIAL)
      GR_F32_CASE(kVecBase + GR_WEIBULL)
      GR_F32_CASE(kVecBase + GR_EXTREME_VALUE)
      GR_F32_CASE(kVecBase + GR_CAUCHY)
      case kVecBase + GR_NORMAL:
        return run_direct<M_N32, kVecBase + GR_NORMAL>(p, d, snap, s);
      case kVecBase + GR_LOGNORMAL:
        return run_direct<M_N32, kVecBase + GR_LOGNORMAL>(p, d, snap, s);
      case GR_NORMAL_STD:
        return run_direct<M_N32, GR_NORMAL_STD>(p, d, snap, s);
      case GR_NORMAL:
        return run_direct<M_N32, GR_NORMAL>(p, d, snap, s);
      case GR_LOGNORMAL:
        return run_direct<M_N32, GR_LOGNORMAL>(p, d, snap, s);
      default:
        return cudaErrorNotSupported;
    }
  }
  if (d.dtype == GR_F64) {
    switch (d.kind) {
      GR_F64_CASE(GR_UNIFORM_REAL)
      GR_F64_CASE(GR_UNIFORM_REAL2)
      GR_F64_CASE(GR_EXPONENTIAL)
      GR_F64_CASE(GR_CAUCHY)
      GR_F64_CASE(GR_WEIBULL)
      GR_F64_CASE(GR_EXTREME_VALUE)
      GR_F64_CASE(GR_GAMMA)
      GR_F64_CASE(GR_BERNOULLI)
      GR_F64_CASE(kTruncNormalKind)
      GR_F64_CASE(kTruncLognormalKind)
      GR_F64_CASE(kTruncExponentialKind)
      GR_F64_CASE(kTruncCauchyKind)
      GR_F64_CASE(kTruncExtremeKind)
      GR_F64_CASE(kTruncWeibullKind)
      GR_F64_CASE(kVecBase + GR_UNIFORM_REAL2)
      GR_F64_CASE(kVecBase + GR_EXPONENTIAL)
      GR_F64_CASE(kVecBase + GR_WEIBULL)
      GR_F64_CASE(kVecBase + GR_EXTREME_VALUE)
      GR_F64_CASE(kVecBase + GR_CAUCHY)
      case kVecBase + GR_BALANCED2:
        return run_direct<M_W64, kVecBase + GR_BALANCED2>(p, d, snap, s);
      case kVecBase + GR_NORMAL:
        return run_direct<M_N64, kVecBase + GR_NORMAL>(p, d, snap, s);
      case kVecBase + GR_LOGNORMAL:
        return run_direct<M_N64, kVecBase + GR_LOGNORMAL>(p, d, snap, s);
      case GR_BALANCED:
        return run_direct<M_W64, GR_BALANCED>(p, d, snap, s);
      case GR_BALANCED2:
        return run_direct<M_W64, GR_BALANCED2>(p, d, snap, s);
      case GR_NORMAL_STD:
        return run_direct<M_N64, GR_NORMAL_STD>(p, d, snap, s);
      case GR_NORMAL:
        return run_direct<M_N64, GR_NORMAL>(p, d, snap, s);
      case GR_LOGNORMAL:
        return run_direct<M_N64, GR_LOGNORMAL>(p, d, snap, s);
      default:
        return cudaErrorNotSupported;
    }
  }
  if (d.dtype == GR_I32) {
    if (d.kind == GR_RANDBITS) return run_direct<M_W32, GR_RANDBITS>(p, d, snap, s);
    if (d.kind == GR_DISCRETE) return run_direct<M_W32, GR_DISCRETE>(p, d, snap, s);
    if (d.kind == GR_BERNOULLI) return run_direct<M_W32, GR_BERNOULLI>(p, d, snap, s);
    if (d.kind == GR_GEOMETRIC) return run_direct<M_W32, GR_GEOMETRIC>(p, d, snap, s);
    if (d.kind == GR_UNIFORM_INT) return run_direct<M_W32, GR_UNIFORM_INT>(p, d, snap, s);
  }
  return cudaErrorNotSupported;
}

// ---------------------------------------------------------------- scalar engines
// Samples drawn with a scalar engine as the Urng (std::mt19937_64,
// P8_mt19937_64): the packets come from RawbitsMaker<Packet8i, Rng, uint64_t,
// scalar_fullbit> (arch/AVX/RandUtils.h:59-144) and RawbitsMaker<Packet4i,
// ...> (arch/SSE/RandUtils.h:22-65) over the engine's 64-bit words, with GCC's
// right-to-left argument evaluation:
//   S_F32U  uniform_real<Packet8f> = rawbits_34: 3 words (a, b, c) ->
//           (c.lo, c.hi, b.lo, t0, b.hi, a.lo, a.hi, t1), t0 / t1 the top
//           bytes of their half's three words (the third twice)
//   S_F32R  rawbits (zero_to_one, BernoulliGen): 4 words in order, lo / hi
//   S_F64   rawbits as 4 double lanes
//   S_F64H  rawbits_half (zero_to_one<Packet4d>): 2 words -> 4 int32 words
//   S_N32 / S_N64  StdNormalGen units of two uniform packets
//   S_I32   Packet4i rawbits: 2 words -> 4 int32
// Packet k of the call reads its words at w[k * wpp]; one thread per packet
// (per unit for the normal kinds).
enum SMode { S_F32U, S_F32R, S_F64, S_F64H, S_N32, S_N64, S_I32 };

__device__ __forceinline__ void words34(const uint64_t* w, uint32_t* v8) {
  const uint64_t a = w[0], b = w[1], c = w[2];
  const uint32_t v[6] = {(uint32_t)c, (uint32_t)(c >> 32), (uint32_t)b, (uint32_t)(b >> 32), (uint32_t)a,
                         (uint32_t)(a >> 32)};
  v8[0] = v[0];
  v8[1] = v[1];
  v8[2] = v[2];
  v8[3] = (v[0] >> 24) | ((v[1] >> 24) << 8) | ((v[2] >> 24) << 16) | ((v[2] >> 24) << 24);
  v8[4] = v[3];
  v8[5] = v[4];
  v8[6] = v[5];
  v8[7] = (v[3] >> 24) | ((v[4] >> 24) << 8) | ((v[5] >> 24) << 16) | ((v[5] >> 24) << 24);
}

template <int SM, int KIND>
__global__ void __launch_bounds__(256) k_sxform(const uint64_t* w, void* out, int64_t npk, DistParams d) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (SM == S_N32 || SM == S_N64) {
    constexpr int WPP = SM == S_N32 ? 3 : 4;
    const int64_t u = t;
    if (2 * u >= npk) return;
    const uint64_t* w1 = w + 2 * u * WPP;
    if (SM == S_N32) {
      uint32_t a[8], b[8];
      words34(w1, a);
      words34(w1 + WPP, b);
      float* o = reinterpret_cast<float*>(out) + 2 * u * 8;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float radius = sqrtf((float)-2 * logf_(1.0f - ur_f(a[q])));
        float sn, cs;
        sincosf_((float)(2 * 3.1415926535897932) * ur_f(b[q]), sn, cs);
        o[q] = nscale32<KIND>(radius * sn, d);
        if (2 * u + 1 < npk) o[8 + q] = nscale32<KIND>(radius * cs, d);
      }
    } else {
      double* o = reinterpret_cast<double*>(out) + 2 * u * 4;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double radius = sqrt(-2.0 * log_(one_minus_ur_d(w1[q])));
        double sn, cs;
        sincos_((2 * 3.1415926535897932) * ur_d(w1[WPP + q]), sn, cs);
        o[q] = nscale64<KIND>(radius * sn, d);
        if (2 * u + 1 < npk) o[4 + q] = nscale64<KIND>(radius * cs, d);
      }
    }
    return;
  }
  if (t >= npk) return;
  if (SM == S_F32U || SM == S_F32R) {
    uint32_t v[8];
    if (SM == S_F32U) {
      words34(w + 3 * t, v);
    } else {
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        v[2 * l] = (uint32_t)w[4 * t + l];
        v[2 * l + 1] = (uint32_t)(w[4 * t + l] >> 32);
      }
    }
    float r[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) r[q] = tf32<KIND>(v[q], d);
    float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(out) + 8 * t);
    o[0] = make_float4(r[0], r[1], r[2], r[3]);
    o[1] = make_float4(r[4], r[5], r[6], r[7]);
  } else if (SM == S_F64) {
    double r[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) r[l] = tf64<KIND>(w[4 * t + l], d);
    double2* o = reinterpret_cast<double2*>(reinterpret_cast<double*>(out) + 4 * t);
    o[0] = make_double2(r[0], r[1]);
    o[1] = make_double2(r[2], r[3]);
  } else if (SM == S_F64H) {
    const uint64_t a = w[2 * t], b = w[2 * t + 1];
    const uint32_t v[4] = {(uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32)};
    double2* o = reinterpret_cast<double2*>(reinterpret_cast<double*>(out) + 4 * t);
    o[0] = make_double2(tw64<KIND>(v[0], d), tw64<KIND>(v[1], d));
    o[1] = make_double2(tw64<KIND>(v[2], d), tw64<KIND>(v[3], d));
  } else {  // S_I32
    const uint64_t a = w[2 * t], b = w[2 * t + 1];
    int4* o = reinterpret_cast<int4*>(reinterpret_cast<int32_t*>(out) + 4 * t);
    o[0] = make_int4(tw32<KIND>((uint32_t)a, d), tw32<KIND>((uint32_t)(a >> 32), d), tw32<KIND>((uint32_t)b, d),
                     tw32<KIND>((uint32_t)(b >> 32), d));
  }
}

template <int SM, int KIND>
static cudaError_t run_sx(const uint64_t* w, void* out, int64_t npk, const DistParams& d, cudaStream_t s) {
  const int64_t threads = (SM == S_N32 || SM == S_N64) ? (npk + 1) / 2 : npk;
  k_sxform<SM, KIND><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(w, out, npk, d);
  return cudaGetLastError();
}

int scalar_words_per_packet(int kind, int dtype) {
  // int32 kinds on one SSE packet of two draws (rawbits / rawbits_34)
  if (dtype == GR_I32) return (kind == GR_RANDBITS || kind == GR_BERNOULLI || kind == GR_GEOMETRIC) ? 2 : 0;
  const bool bal = kind == GR_BALANCED || kind == GR_BALANCED2;
  switch (kind) {
    case GR_UNIFORM_REAL:
    case GR_UNIFORM_REAL2:
    case GR_BALANCED:
    case GR_BALANCED2:
    case GR_NORMAL_STD:
    case GR_NORMAL:
    case GR_LOGNORMAL:
    case GR_EXPONENTIAL:
    case GR_CAUCHY:
    case GR_WEIBULL:
    case GR_EXTREME_VALUE:
    case GR_GAMMA:
    case GR_BERNOULLI:
      if (dtype == GR_F32) return (bal || kind == GR_BERNOULLI) ? 4 : 3;
      return bal ? 2 : 4;
    default:
      return 0;
  }
}

#define GR_SX(SMODE, K) \
  case K:               \
    return run_sx<SMODE, K>(w, out, npk, d, s);

cudaError_t launch_scalar_xform(const uint64_t* w, void* out, int64_t npk, const DistParams& d, cudaStream_t s) {
  if (d.dtype == GR_I32) {
    if (d.kind == GR_RANDBITS) return run_sx<S_I32, GR_RANDBITS>(w, out, npk, d, s);
    if (d.kind == GR_BERNOULLI) return run_sx<S_I32, GR_BERNOULLI>(w, out, npk, d, s);
    if (d.kind == GR_GEOMETRIC) return run_sx<S_I32, GR_GEOMETRIC>(w, out, npk, d, s);
    // DiscreteGen: a Packet8i of four draws per two output packets, so packet
    // t still reads draws 2t and 2t + 1
    if (d.kind == GR_DISCRETE) return run_sx<S_I32, GR_DISCRETE>(w, out, npk, d, s);
    return cudaErrorNotSupported;
  }
  if (d.dtype == GR_F32) {
    switch (d.kind) {
      GR_SX(S_F32U, GR_UNIFORM_REAL)
      GR_SX(S_F32U, GR_UNIFORM_REAL2)
      GR_SX(S_F32U, GR_EXPONENTIAL)
      GR_SX(S_F32U, GR_CAUCHY)
      GR_SX(S_F32U, GR_WEIBULL)
      GR_SX(S_F32U, GR_EXTREME_VALUE)
      GR_SX(S_F32U, GR_GAMMA)
      GR_SX(S_F32R, GR_BALANCED)
      GR_SX(S_F32R, GR_BALANCED2)
      GR_SX(S_F32R, GR_BERNOULLI)
      GR_SX(S_N32, GR_NORMAL_STD)
      GR_SX(S_N32, GR_NORMAL)
      GR_SX(S_N32, GR_LOGNORMAL)
      default:
        return cudaErrorNotSupported;
    }
  }
  switch (d.kind) {
    GR_SX(S_F64, GR_UNIFORM_REAL)
    GR_SX(S_F64, GR_UNIFORM_REAL2)
    GR_SX(S_F64, GR_EXPONENTIAL)
    GR_SX(S_F64, GR_CAUCHY)
    GR_SX(S_F64, GR_WEIBULL)
    GR_SX(S_F64, GR_EXTREME_VALUE)
    GR_SX(S_F64, GR_GAMMA)
    GR_SX(S_F64, GR_BERNOULLI)
    GR_SX(S_F64H, GR_BALANCED)
    GR_SX(S_F64H, GR_BALANCED2)
    GR_SX(S_N64, GR_NORMAL_STD)
    GR_SX(S_N64, GR_NORMAL)
    GR_SX(S_N64, GR_LOGNORMAL)
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace gr
