// Launch interface between the host library (gr_api.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "gr_internal.h"
#include "../../include/gpurand.h"

#include <string>

namespace gr {

// Per-call distribution constants, computed on the host exactly as the
// reference generator's constructor computes them.
struct DistParams {
  int32_t kind;   // gr_dist_kind
  int32_t dtype;  // gr_dtype
  float fa, fb, fc, fd, fe, ff, fg, fh;   // float-precision constants
  double da, db, dc, dd, de, df, dg, dh;  // double-precision constants
  int32_t ia, ib, ic;                      // integer constants (trials, counts, flags)
  uint32_t bitmask;                        // alias table mask
  int32_t ncdf;                            // CDF entries (discrete < 16 weights)
  int32_t post;                            // output transform of a beta draw: 1 = FisherFGen (fh / dh = b/a)
  int32_t flags;                           // kParamUnit*: a divisor or scale that is exactly 1 in the scalar type
  const void* vparam;                      // per-element parameter array (device), aligned with the output
  const void* vparam2;                     // second per-element parameter array (kParamVecB)
  const int32_t* prob;                     // alias table / cdf (device)
  const int32_t* alias;
};

// x / 1 and x * 1 are x in IEEE arithmetic, so a parameter that is exactly 1
// skips its division or multiplication without changing a bit.
constexpr int32_t kParamUnitDiv = 1;    // ExponentialGen: lambda == 1
constexpr int32_t kParamUnitScale = 2;  // GammaGen beta, WeibullGen b == 1
// per-element forms: parameter a / b of element i is vparam[i] / vparam2[i]
constexpr int32_t kParamVecA = 4;
constexpr int32_t kParamVecB = 8;
// the 2-lane Vmt19937_64 (SSE / NEON profile): Packet4f / Packet2d outputs
// from the first two lanes of each packet (launch_direct only)
constexpr int32_t kParamTwoLane = 16;

// Output transform of generators built on a BetaGen draw x (bits v):
// FisherFGen writes (b/a) x / (1 - x), b/a in the scalar type
// (NormalExp.h:1016-1021).
template <bool WIDE>
__device__ __forceinline__ uint64_t beta_post(uint64_t v, const DistParams& d) {
  if (d.post != 1) return v;
  if (WIDE) {
    const double x = __longlong_as_double((long long)v);
    return (uint64_t)__double_as_longlong((d.dh * x) / (1.0 - x));
  }
  const float x = __uint_as_float((uint32_t)v);
  return (uint64_t)__float_as_uint((d.fh * x) / (1.0f - x));
}

// How one call is split over sub-engines and segments.
struct Plan {
  EngState* eng;          // K engines
  GenState* gen;          // K generator states (may be null)
  const uint64_t* segwin; // jump results: [(k*(S-1) + s-1)][4][312]
  const uint64_t* prefix; // prefix buffer [k][4][kPrefixLen] (segmented calls)
  int32_t K;              // sub-engines
  int32_t S;              // segments per sub-engine
  int64_t J;              // packets (or units for 2-packet kinds) per segment
  int64_t gran_per_k;     // output granules per sub-engine ...
  int64_t gran_rem;       // ... plus one for the first gran_rem engines
  int32_t gran;           // outputs per granule
  void* out;
};

// kernels (gr_kernels.cu)
cudaError_t launch_seed(EngState* st, int K, uint64_t seed, cudaStream_t s);
cudaError_t launch_prefix(const EngState* st, const GenState* gen, int K, uint64_t* prefix, CallSnap* snap,
                          cudaStream_t s);
cudaError_t launch_jump(const uint64_t* prefix, const uint64_t* polys, int K, int S, uint64_t* segwin,
                        cudaStream_t s);
// Loads the code of k_prefix, k_jump and the raw-stream k_direct on the
// current device and sets k_jump's shared-memory limit, so that later
// launches of them load nothing.
cudaError_t preload_raw_stream_kernels();
// Fused engine + transform for kinds whose draws per output are fixed and
// packet aligned.  Returns cudaErrorNotSupported for other kinds.
cudaError_t launch_direct(const Plan& p, const DistParams& d, const CallSnap* snap, cudaStream_t s);

// Multi-packet fixed units (gr_samplers.cu): U packets (or half packets) per
// unit of P outputs, Us units per jump segment; segment s starts at packet
// s*J - delta.
cudaError_t launch_staged(const Plan& p, const DistParams& d, const CallSnap* snap, int U, int64_t Us, int delta,
                          cudaStream_t s);

// Rejection samplers resolved with CompressMask semantics (gr_samplers.cu);
// one CTA per stream.  rk: 0 gamma alpha<1 (GS), 1 gamma tan proposal,
// 2 beta with a,b < 1, 3 poisson mean >= 12, 4 binomial tan proposal.
cudaError_t launch_reject(const Plan& p, const DistParams& d, int rk, int64_t max_blocks, cudaStream_t s);

// Segmented form of launch_reject for long calls on few engines (see
// gr_samplers.cu): p.S segments of a.Ts trials per engine, windows from
// prepare_segments with J = Ts * packets per trial (one packet earlier for the
// int32 kinds).  gather_n bounds the FIFO lanes of one engine.
struct RsArgs {
  int64_t Ts;
  int64_t* cnt;    // [K * S][2]
  int64_t* start;  // [K * S][2]
  int64_t* fin;    // [K][4]
  uint64_t* lanes; // [K][lane_cap] lanes of 8 bytes (double) or 4 bytes (float / int32)
  int64_t* pos;    // [K][pos_cap]
  int64_t lane_cap, pos_cap;
  int64_t max_blocks;
};
cudaError_t launch_reject_segmented(const Plan& p, const DistParams& d, int rk, const CallSnap* snap, const RsArgs& a,
                                    int64_t gather_n, cudaStream_t s);

// PoissonGen (mean < 12) / BinomialGen (mean < 1) on few engines over S
// jump-ahead segments of J packets per engine (gr_samplers.cu): a scan per
// segment, a plan per engine, a write per segment.  Scratch per engine and
// segment; bits: words_per_seg bitmap words per segment.
constexpr int kPwEntries = 64;  // entry offsets into a segment (the step look-ahead)
struct PwArgs {
  int64_t J;                // packets per segment
  const CallSnap* snap;     // caches at call start, per engine
  int32_t* info;            // [K*S][4]: exit offset, steps, every entry merged, unused
  int32_t* ent;             // [K*S][kPwEntries][2]: steps, exit offset
  int64_t* plan;            // [K*S][3]: entry offset, first output packet, steps
  uint32_t* bits;           // [K*S][words_per_seg]
  int64_t words_per_seg;
  int64_t max_blocks;       // blocks the last segment of an engine may run to
};
cudaError_t launch_poisson_segmented(const Plan& p, const DistParams& d, const PwArgs& a, cudaStream_t s);

// Data-dependent consumption (gr_samplers.cu), one CTA per stream: k_poisson
// for PoissonGen mean < 12 and BinomialGen mean < 1 (int32), k_beta for
// BetaGen with a or b >= 1 (f32/f64; d.ia / d.ib hold (gamma branch << 8) |
// packets for the two GammaGens).
cudaError_t launch_walk(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s);

// Samples drawn with a scalar engine as the Urng (gr_kernels.cu): npk output
// packets from the engine's 64-bit words w (scalar_words_per_packet(kind,
// dtype) words per packet, two packets per StdNormalGen unit).  0 words: the
// kind has no scalar-engine form here.
int scalar_words_per_packet(int kind, int dtype);
cudaError_t launch_scalar_xform(const uint64_t* w, void* out, int64_t npk, const DistParams& d, cudaStream_t s);

// TruncGen's CompressMask filter over M base packets drawn into HBM
// (gr_trunc.cu).  Writes up to `cap` output packets, updates the carried
// lanes, and leaves in res: [0] packets emitted, [1] the base packet that
// emitted the last wanted one (-1: the chunk ran out first), [2] full base
// packets, [3] accepted lanes of partial base packets, [4] FIFO fill after
// the stop packet (or the chunk), [5] carried lanes at the start.
constexpr int64_t kTruncChunkMax = (int64_t)1 << 22;
struct TruncFilterArgs {
  const void* cand;  // M packets of P lanes (float bits P = 8, double bits P = 4)
  int64_t M;
  double lower, upper;  // the support, already in the scalar type
  GenSlot* carry;       // rest_cnt + rest: TruncGen's carried lanes
  void* out;            // output packets
  int64_t cap;          // output packets wanted
  void* queue;          // (M + 1) * P lanes
  int64_t* blk;         // 2 * ceil(M / 256)
  int64_t* grp;         // M + 1
  int64_t* res;         // 6
};
cudaError_t launch_trunc_filter(int dtype, const TruncFilterArgs& a, cudaStream_t s);

// BinomialVGen<int32_t> with per-element (trials, p) (gr_binomv.cu): one warp
// per stream, packets of 4 outputs on half-packet draws.  NULL arrays take
// the scalar operands.
struct BinomVArgs {
  const int32_t* trials;
  const float* p;
  int32_t trials0;
  float p0;
  int64_t max_blocks;
};
cudaError_t launch_binom_v(const Plan& p, const BinomVArgs& a, cudaStream_t s);
// The same on a scalar engine's pre-drawn 64-bit words (one chain): res[0] =
// packets completed, res[1] = words they consumed.
cudaError_t launch_binom_v_words(const uint64_t* w, int64_t nwords, const BinomVArgs& a, int32_t* out, int64_t npk,
                                 int64_t* res, cudaStream_t s);
// PoissonGen / BinomialGen (int32) on a scalar engine's pre-drawn words (one
// chain); carry: CompressMask's carried lanes [0..3] and their count [8].
// GammaGen's rejection trials (rk 0 GS, 1 tan; f32 / f64) on a scalar
// engine's pre-drawn words: M trials' candidate lanes, rejected lanes NaN.
cudaError_t launch_sx_cand(int rk, int dtype, const uint64_t* w, int64_t M, const DistParams& d, void* cand,
                           cudaStream_t s);
// GammaGen with integral alpha < 20 (U = alpha uniform packets per output
// packet) and StudentTGen (U = 2) on a scalar engine's pre-drawn words.
// BetaGen / FisherFGen on a scalar engine (gr_samplers.cu, k_sx_beta): one
// warp over a chunk of W pre-drawn words; carry: 3 x (2 P) carried lanes and
// cnt: 3 counts (GammaGen(a), GammaGen(b), the beta's own), device, updated;
// res: packets completed, draws they used.
struct SxBetaArgs {
  DistParams beta;  // the BetaGen's parameters (ic: a < 1 and b < 1; post: FisherF map)
  DistParams g[2];  // GammaGen(a), GammaGen(b) in the scalar type (general branch)
  void* out;
  int64_t npk;
  uint64_t* carry;
  int32_t* cnt;
  int64_t* res;
};
cudaError_t launch_sx_beta(const uint64_t* w, int64_t W, const SxBetaArgs& a, int dtype, cudaStream_t s);
cudaError_t launch_sx_staged(const uint64_t* w, void* out, int64_t npk, const DistParams& d, int U,
                             cudaStream_t s);
cudaError_t launch_int_words(const uint64_t* w, int64_t nwords, const DistParams& d, int32_t* out, int64_t npk,
                             int64_t* res, uint32_t* carry, cudaStream_t s);

// Batched vectorize-over-params sets (gr_vop.cu).
struct VopArgs {
  int64_t nsets;
  const int32_t* perm;
  uint64_t seed;
  const float* a;
  const float* b;
  const int32_t* trials;
  const int32_t* counts;
  const int64_t* offsets;
  void* out;
  int32_t* status;
};
cudaError_t launch_vop(int kind, int threads, const VopArgs& va, cudaStream_t s);

// Outputs per granule: the smallest output count a call (or a stream slice)
// may have for the kind.  Packets per unit: 2 for the Box-Muller kinds.
// The scalar operator() tail of a size that is not a whole number of packets
// (gr_kernels.cu): kinds whose scalar form is exact bit arithmetic on one
// draw, and the kernel that applies it to n < P draws w (engine packets'
// first 64-bit lanes, or a scalar engine's draws).
bool kind_has_exact_tail(int kind, int dtype);
// Kinds the 2-lane Vmt19937_64 profile serves: the raw stream and the
// transforms of one 32-bit word (float) or one 64-bit lane (double) per
// output, whose values do not depend on the packet width.
bool kind_two_lane(int kind, int dtype);
cudaError_t launch_tail(const uint64_t* w, void* out, int n, const DistParams& d, bool packet_engine, cudaStream_t s);
int kind_granule(int kind, int dtype);
int kind_packets_per_unit(int kind, int dtype);
bool kind_is_direct(int kind, int dtype, const DistParams& d);

// Host-side helpers shared by the C ABI translation units (gr_api.cu).
EngState* engine_state_ptr(gr_engine* e);
// GR_ERR_UNSUPPORTED (with the error text set) unless e is a 4-lane engine:
// the entry points other than the raw stream and the per-word kinds serve the
// AVX2 profile only.
gr_status need_four_lanes(const gr_engine* e, const char* what);
gr_status set_last_error(gr_status s, const std::string& msg);
// Scalar draws on the packet engine (each takes a whole packet and keeps lane
// 0): stream k of the engine owns samples [s0_k, s0_k + n_k) of `samples`,
// split as any call splits them, and makes per_sample * n_k draws in stream
// order into out[s0_k * per_sample ...].
gr_status draw_first_words(gr_engine* e, uint64_t* out, int64_t per_sample, int64_t samples, cudaStream_t s);

}  // namespace gr
