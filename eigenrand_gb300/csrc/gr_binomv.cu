// Per-element binomial draws: binomial(urng, ArrayXi trials, ArrayXf p)
// (EigenRand/Dists/Discrete.h:1805-1831), BinomialVGen<int32_t>::packetOp
// (:1124-1192) with every lane's own (trials, p).
//
// Each packet of 4 outputs runs a multiplicative Poisson loop for the lanes
// with mean < 1, then a tan-proposal rejection until every lane has a value,
// on float uniforms drawn as half packets (rng.half(), the engine's cached
// upper half first).  A packet's consumption depends on its lanes, so each
// engine's chain is sequential: one warp per engine, lanes 0-3 the packet
// lanes deciding the loops by ballot; the warp twists its own blocks into
// 624 half-packet draws each.  The engine window, its half cache and the
// consumed count are written back at the end, as every engine call does.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_math.cuh"
#include "gr_mt.cuh"

namespace gr {
namespace {

constexpr int kBvWarps = 4;  // engines per CTA
// per warp: two lane windows, then the newest block's 624 half packets
constexpr size_t kBvWarpBytes = (size_t)2 * kLanes * kN * 8 + (size_t)2 * kN * 16;

__device__ __forceinline__ float bv_ur(uint32_t x) { return u2f((x & 0x7fffffu) | (127u << 23)) - 1.0f; }

__global__ void __launch_bounds__(32 * kBvWarps) k_binom_v(Plan p, BinomVArgs a) {
  extern __shared__ __align__(16) uint64_t bv_dyn[];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kBvWarps + wi;
  if (k >= p.K) return;  // the whole warp
  uint8_t* base = reinterpret_cast<uint8_t*>(bv_dyn) + (size_t)wi * kBvWarpBytes;
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(base);
  uint32_t(*hw)[4] = reinterpret_cast<uint32_t(*)[4]>(base + (size_t)2 * kLanes * kN * 8);
  EngState* st = p.eng + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  int32_t* out = static_cast<int32_t*>(p.out);
  const float fpi = (float)3.1415926535897932;

  for (int i = lane; i < kLanes * kN; i += 32) raw[0][i / kN][i % kN] = st->win[i / kN][i % kN];
  __syncwarp();

  // draws: the engine's cached half first, then the halves of new blocks
  bool pending = st->half_valid != 0, abort = false;
  int h = 2 * kN, cur = 0;
  int64_t nb = 0;
  auto next = [&]() -> uint32_t {
    if (pending) {
      pending = false;
      return lane < 4 ? st->half_cache[lane] : 0u;
    }
    if (h == 2 * kN) {
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
          uint64_t pk[kLanes];
#pragma unroll
          for (int l = 0; l < kLanes; ++l) {
            const uint64_t b = (i + 1 < kN) ? old[l][i + 1] : nw[l][0];
            const uint64_t c = (ph == 0) ? old[l][i + kM] : nw[l][i - kM];
            const uint64_t v = mt_twist(old[l][i], b, c);
            nw[l][i] = v;
            pk[l] = mt_temper(v);
          }
          hw[2 * i][0] = (uint32_t)pk[0];
          hw[2 * i][1] = (uint32_t)(pk[0] >> 32);
          hw[2 * i][2] = (uint32_t)pk[1];
          hw[2 * i][3] = (uint32_t)(pk[1] >> 32);
          hw[2 * i + 1][0] = (uint32_t)pk[2];
          hw[2 * i + 1][1] = (uint32_t)(pk[2] >> 32);
          hw[2 * i + 1][2] = (uint32_t)pk[3];
          hw[2 * i + 1][3] = (uint32_t)(pk[3] >> 32);
        }
        __syncwarp();
      }
      cur ^= 1;
      ++nb;
      h = 0;
    }
    const uint32_t v = lane < 4 ? hw[h][lane] : 0u;
    ++h;
    return v;
  };
  auto mask4 = [&](bool pr) -> unsigned { return __ballot_sync(0xffffffffu, pr && lane < 4) & 0xfu; };

  for (int64_t e = 0; e < n / 4 && !abort; ++e) {
    const int64_t i = off + e * 4 + (lane < 4 ? lane : 0);
    const int32_t tr = lane < 4 ? (a.trials ? __ldg(a.trials + i) : a.trials0) : 0;
    const float pv = lane < 4 ? (a.p ? __ldg(a.p + i) : a.p0) : 0.0f;
    const float small_p = pv < 1.0f - pv ? pv : 1.0f - pv;  // pmin(p, 1 - p)
    const float ptrials = (float)tr;
    const float mean = ptrials * small_p;
    const float g1 = lgamma_approxf_(ptrials + 1.0f);
    const float sqrt_v = sqrtf((2.0f * mean) * (1.0f - small_p));
    const float lsp = logf_(small_p), lsq = logf_(1.0f - small_p);
    bool valid = mean < 1.0f;
    float vres = 0.0f;
    if (mask4(valid)) {
      const float ne = expf_(-mean);
      float val = 1.0f;
      int32_t res = 0;
      for (;;) {
        val = val * bv_ur(next());
        if (abort) break;
        const bool c = (ne < val) && valid;
        if (mask4(c) == 0) break;
        res += c ? 1 : 0;
      }
      vres = (float)res;
    }
    if (mask4(valid) != 0xfu) {
      for (;;) {
        float sn, cs;
        sincosf_(fpi * bv_ur(next()), sn, cs);
        const float ys = sn / cs;
        const float fres = truncf(sqrt_v * ys + mean);
        const float p1 = ((float)1.2 * sqrt_v) * (1.0f + ys * ys);
        float t = (g1 - lgamma_approxf_(fres + 1.0f)) - lgamma_approxf_((ptrials + 1.0f) - fres);
        t = t + fres * lsp;
        t = t + (ptrials - fres) * lsq;
        const float p2 = expf_(t);
        const float u2 = bv_ur(next());
        if (abort) break;
        const bool fv = (0.0f <= fres) && (fres <= ptrials) && (u2 <= p1 * p2);
        if (fv && !valid) vres = fres;
        valid = valid || fv;
        if (mask4(valid) == 0xfu) break;
      }
    }
    if (abort) break;
    if (lane < 4) out[i] = (pv == small_p) ? cvtt_f32(vres) : tr - cvtt_f32(vres);
  }

  // ---- state after the call (as k_negbin: the last draw's block, the
  // cached upper half when a packet was split)
  if (abort) {
    if (lane == 0) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    return;
  }
  if (nb > 0) {
    const int last = h - 1;       // last half packet drawn from the newest block
    const int rr = last / 2 + 1;  // packets used of it
    uint64_t(*lastb)[kN] = raw[cur];
    uint64_t(*prevb)[kN] = raw[cur ^ 1];
    for (int t = lane; t < kLanes * kN; t += 32) {
      const int l = t / kN, i = t % kN;
      st->win[l][i] = (i < kN - rr) ? prevb[l][rr + i] : lastb[l][i - (kN - rr)];
    }
    if (lane < 4) st->half_cache[lane] = (last & 1) == 0 ? hw[last + 1][lane] : 0u;
    if (lane == 0) {
      st->half_valid = (last & 1) == 0 ? 1 : 0;
      st->consumed += (uint64_t)((nb - 1) * kN + rr);
    }
  } else if (lane == 0 && st->half_valid && n > 0) {
    st->half_valid = 0;  // only the cached half was drawn
  }
}

}  // namespace

cudaError_t launch_binom_v(const Plan& p, const BinomVArgs& a, cudaStream_t s) {
  constexpr size_t smem = kBvWarpBytes * kBvWarps;
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_binom_v, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  k_binom_v<<<(p.K + kBvWarps - 1) / kBvWarps, 32 * kBvWarps, smem, s>>>(p, a);
  return cudaGetLastError();
}

}  // namespace gr
