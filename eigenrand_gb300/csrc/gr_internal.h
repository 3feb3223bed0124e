// Internal layouts shared by the host library code and the CUDA kernels.
#pragma once
#include <cstddef>
#include <cstdint>

namespace gr {

constexpr int kN = 312;      // MT19937-64 state words
constexpr int kM = 156;      // MT19937-64 shift
constexpr int kLanes = 4;    // Vmt19937_64 lanes under AVX2 (Pmt19937_64<Packet8i>)
constexpr int kPrefix = 20280;  // 65 blocks: >= 19937 + 312 words for a jump

constexpr uint64_t kMatA = 0xb5026f5aa96619e9ull;
constexpr uint64_t kSeedF = 6364136223846793005ull;
constexpr uint64_t kUpper = ~0ull << 31;
constexpr uint64_t kLower = ~kUpper;

// One Vmt19937_64 engine (4 MT19937-64 lanes) resident in HBM.
//   win[l][i]  : the 312 raw (untempered) words of lane l that precede the
//                next output; twisting them yields the next 312 outputs.
//                After seeding these are the seed words x_0..x_311.
//   half_*     : MersenneTwister::half() cache (the upper 128 bits of a split
//                packet), PacketRandomEngine.h:325-336.
struct EngState {
  uint64_t win[kLanes][kN];
  uint32_t half_cache[kLanes];
  int32_t half_valid;
  int32_t status;      // device-side error bits (GR_DEV_*), folded into the next sync
  uint64_t consumed;   // packets drawn since seeding
};
static_assert(sizeof(EngState) % 16 == 0, "EngState must stay 16-byte aligned");

// Caches that EigenRand keeps inside generator objects: the StdNormalGen /
// DiscreteGen packet cache (valid + cache) and the CompressMask carry
// (rest_cnt + rest).  Three slots: the generator itself and two nested ones
// (BetaGen holds two GammaGens).
struct GenSlot {
  int32_t valid;
  int32_t rest_cnt;
  uint32_t cache[16];
  uint32_t rest[16];
};
struct GenState {
  GenSlot s[3];
};

// Jump-ahead prefix: the window plus 130 chunks of 156 words per lane
// (20592 >= 19968 terms + 312 window words + register look-ahead).
constexpr int kPrefixLen = kN + 130 * kM;
constexpr int kRawKind = 100;  // internal kind id for the raw u64 stream
constexpr int kBernoulliVKind = 101;  // BernoulliVGen<float>: per-element probability (DistParams::vparam)
constexpr int kRawLane0Kind = 102;   // lane 0 of every packet only (scalar draws: pfirst of rng()), u64 each
// Truncated.h inverse-CDF forms: u = UniformRealGen(phi(lower), phi(upper))
// (slope fa/da, bias fb/db), then the base's inverse CDF with constants
// fc/dc, fd/dd
constexpr int kTruncNormalKind = 110;       // -sqrt2 erfinv(1 - 2u) * stdev(c) + mean(d)
constexpr int kTruncLognormalKind = 111;    // exp of the above
constexpr int kTruncExponentialKind = 112;  // -log(1 - u) * (1 / lambda)(c)
constexpr int kTruncCauchyKind = 113;       // a(c) + b(d) tan(pi (u - 1/2))
constexpr int kTruncExtremeKind = 114;      // a(c) - b(d) log(-log u)
constexpr int kTruncWeibullKind = 115;      // b(d) exp(log(-log(1 - u)) (1 / a)(c))
// Per-element forms (*VGen): kind kVecBase + K draws like K with parameters
// a[i], b[i] of output element i (DistParams::vparam / vparam2 when the
// kParamVecA / kParamVecB flag is set, else the scalars fe/ff, de/df)
constexpr int kVecBase = 200;

// Caches as they were when a segmented call started (written by the prefix
// kernel, read by every segment so that the last segment may update the live
// state without racing the first).
struct CallSnap {
  int32_t half_valid;
  int32_t gen_valid;
  uint32_t half_cache[kLanes];
  uint32_t gen_cache[16];
};

enum DevStatus : int32_t {
  GR_DEV_REJECT_LIMIT = 1,  // a rejection loop hit its iteration cap
  GR_DEV_BAD_INPUT = 2,
  GR_DEV_MMA_TIMEOUT = 8,   // a tensor-core kernel gave up waiting for its products
};

}  // namespace gr
