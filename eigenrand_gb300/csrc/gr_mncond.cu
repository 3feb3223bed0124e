// MultinomialGen's conditional-binomial path (EigenRand/MvDists/Multinomial.h:
// 62-87), taken when trials >= max(30 (dim - 1), 100).
//
// The reference draws row 0 of the (dim x samples) result as
// BinomialVGen<float> over all samples (each lane: its remaining trials, one
// p for the row), subtracts, and repeats for rows 1 .. dim-2 with
// p = probs[i] / rest_p; the last row is what remains.  Within a row the
// packets of 8 samples are evaluated in order, each running
// BinomialVGen<float>::packetOp (Discrete.h:1241-1320): a multiplicative
// Poisson loop for lanes with mean < 1, then a tan-proposal rejection that
// iterates until every lane has a value.  A packet's consumption depends on
// its lanes, so each engine's chain is sequential: one warp per engine, lanes
// 0-7 are the packet lanes and decide the loops by ballot; the warp twists
// its own engine blocks into full packets of 8 words.  The remaining trials
// live in the result's last row until the end.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_math.cuh"
#include "gr_mt.cuh"
#include "gr_mv.cuh"

namespace gr {
namespace {

constexpr int kMcWarps = 1;  // engines per CTA
// per warp: two lane windows (the newest block and the one before) ...
constexpr size_t kMcWarpBytes = (size_t)2 * kLanes * kN * 8;
// ... and, buffered, the newest block's packets tempered into 8 words each
constexpr size_t kMcWarpBytesBuf = kMcWarpBytes + (size_t)kN * 32;

__device__ __forceinline__ float ur_word(uint32_t x) { return u2f((x & 0x7fffffu) | (127u << 23)) - 1.0f; }

// BUF: temper each new block once into a packet buffer (10 KB more shared
// memory, a shorter chain per draw); otherwise temper the words as read.
template <bool BUF>
__global__ void __launch_bounds__(32 * kMcWarps) k_mn_cond(Plan p, McArgs a) {
  extern __shared__ __align__(16) uint64_t mc_dyn[];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kMcWarps + wi;
  if (k >= p.K) return;  // the whole warp
  uint8_t* base = reinterpret_cast<uint8_t*>(mc_dyn) + (size_t)wi * (BUF ? kMcWarpBytesBuf : kMcWarpBytes);
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(base);
  uint32_t(*pw)[8] = reinterpret_cast<uint32_t(*)[8]>(base + kMcWarpBytes);
  EngState* st = p.eng + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t s0 = g0 * p.gran, n = ng * p.gran;  // samples of this engine
  if (n == 0) return;
  const int dim = a.dim;
  int32_t* out = a.out;
  const float fpi = (float)3.1415926535897932;

  for (int i = lane; i < kLanes * kN; i += 32) raw[0][i / kN][i % kN] = st->win[i / kN][i % kN];
  __syncwarp();

  bool abort = false;
  int h = kN, cur = 0;
  int64_t nb = 0;
  // word `lane` of the engine's next full packet (Packet8i: lane j is the low
  // (j even) or high (j odd) half of 64-bit lane j / 2)
  auto next = [&]() -> uint32_t {
    if (h == kN) {
      if (nb >= a.max_blocks) {
        abort = true;
        return 0u;
      }
      __syncwarp();
      uint64_t(*old)[kN] = raw[cur];
      uint64_t(*nw)[kN] = raw[cur ^ 1];
#pragma unroll 1
      for (int ph = 0; ph < 2; ++ph) {
        for (int ii = lane; ii < kM; ii += 32) {
          const int i = ph * kM + ii;
#pragma unroll
          for (int l = 0; l < kLanes; ++l) {
            const uint64_t b = (i + 1 < kN) ? old[l][i + 1] : nw[l][0];
            const uint64_t c = (ph == 0) ? old[l][i + kM] : nw[l][i - kM];
            nw[l][i] = mt_twist(old[l][i], b, c);
            if (BUF) {
              const uint64_t t = mt_temper(nw[l][i]);
              pw[i][2 * l] = (uint32_t)t;
              pw[i][2 * l + 1] = (uint32_t)(t >> 32);
            }
          }
        }
        __syncwarp();
      }
      cur ^= 1;
      ++nb;
      h = 0;
    }
    if (BUF) {
      const uint32_t v = lane < 8 ? pw[h][lane] : 0u;
      ++h;
      return v;
    }
    // tempered as read: word j of packet h is the low (j even) or high half
    // of lane j / 2
    const uint64_t t = mt_temper(raw[cur][(lane & 7) >> 1][h]);
    ++h;
    return lane < 8 ? ((lane & 1) ? (uint32_t)(t >> 32) : (uint32_t)t) : 0u;
  };
  auto mask8 = [&](bool pr) -> unsigned { return __ballot_sync(0xffffffffu, pr && lane < 8) & 0xffu; };

  for (int row = 0; row < a.rows && !abort; ++row) {
    const float pv = __ldg(a.p + row);
    for (int64_t pk = 0; pk < n / 8 && !abort; ++pk) {
      const int64_t s = s0 + pk * 8 + (lane < 8 ? lane : 0);
      const int32_t tr = lane < 8 ? (row == 0 ? a.trials : out[s * dim + dim - 1]) : 0;
      // BinomialVGen<float>::packetOp
      const float small_p = pv < 1.0f - pv ? pv : 1.0f - pv;
      const float ptrials = (float)tr;
      const float mean = ptrials * small_p;
      const float g1 = lgamma_approxf_(ptrials + 1.0f);
      const float sqrt_v = sqrtf((2.0f * mean) * (1.0f - small_p));
      const float lsp = logf_(small_p), lsq = logf_(1.0f - small_p);
      bool valid = mean < 1.0f;
      float vres = 0.0f;
      if (mask8(valid)) {
        const float ne = expf_(-mean);
        float val = 1.0f, res = 0.0f;
        for (;;) {
          val = val * ur_word(next());
          if (abort) break;
          const bool c = (ne < val) && valid;
          if (mask8(c) == 0) break;
          res += c ? 1.0f : 0.0f;
        }
        vres = res;
      }
      if (mask8(valid) != 0xffu) {
        for (;;) {
          float sn, cs;
          sincosf_(fpi * ur_word(next()), sn, cs);
          const float ys = sn / cs;
          const float fres = truncf(sqrt_v * ys + mean);
          const float p1 = ((float)1.2 * sqrt_v) * (1.0f + ys * ys);
          float t = (g1 - lgamma_approxf_(fres + 1.0f)) - lgamma_approxf_((ptrials + 1.0f) - fres);
          t = t + fres * lsp;
          t = t + (ptrials - fres) * lsq;
          const float p2 = expf_(t);
          const float u2 = ur_word(next());
          if (abort) break;
          const bool fv = (0.0f <= fres) && (fres <= ptrials) && (u2 <= p1 * p2);
          if (fv && !valid) vres = fres;
          valid = valid || fv;
          if (mask8(valid) == 0xffu) break;
        }
      }
      if (abort) break;
      const int32_t cnt = (pv == small_p) ? cvtt_f32(vres) : tr - cvtt_f32(vres);
      if (lane < 8) {
        if (row < dim - 1) out[s * dim + row] = cnt;
        out[s * dim + dim - 1] = tr - cnt;
      }
      __syncwarp();
    }
  }

  // ---- state after the call
  if (abort) {
    if (lane == 0) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    return;
  }
  if (nb > 0) {
    const int rr = h;  // packets used of the newest block
    uint64_t(*lastb)[kN] = raw[cur];
    uint64_t(*prevb)[kN] = raw[cur ^ 1];
    for (int t = lane; t < kLanes * kN; t += 32) {
      const int l = t / kN, i = t % kN;
      st->win[l][i] = (i < kN - rr) ? prevb[l][rr + i] : lastb[l][i - (kN - rr)];
    }
    if (lane == 0) st->consumed += (uint64_t)((nb - 1) * kN + rr);
  }
}

}  // namespace

cudaError_t launch_mn_cond(const Plan& p, const McArgs& a, cudaStream_t s) {
  static bool attr[64] = {};
  static int sms[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_mn_cond<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kMcWarpBytesBuf * kMcWarps));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mn_cond<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(kMcWarpBytes * kMcWarps));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  const unsigned grid = (unsigned)((p.K + kMcWarps - 1) / kMcWarps);
  // buffered while every stream's CTA is resident at 30 KB (7 per SM); with
  // more streams the 20 KB form fits 11 per SM
  if ((int64_t)grid <= 7LL * sms[dev])
    k_mn_cond<true><<<grid, 32 * kMcWarps, kMcWarpBytesBuf * kMcWarps, s>>>(p, a);
  else
    k_mn_cond<false><<<grid, 32 * kMcWarps, kMcWarpBytes * kMcWarps, s>>>(p, a);
  return cudaGetLastError();
}

}  // namespace gr
