// Per-element binomial draws: binomial(urng, ArrayXi trials, ArrayXf p)
// (EigenRand/Dists/Discrete.h:1805-1831), BinomialVGen<int32_t>::packetOp
// (:1124-1192) with every lane's own (trials, p).
//
// Each packet of 4 outputs runs a multiplicative Poisson loop for the lanes
// with mean < 1, then a tan-proposal rejection until every lane has a value,
// on float uniforms drawn as half packets (rng.half(), the engine's cached
// upper half first).  A packet's consumption depends on its lanes, so each
// engine's chain is sequential: one warp per engine, every group of 4 lanes
// holding the packet's 4 lanes and the loops decided by ballot; the warp
// twists its own blocks into 624 half-packet draws each.  The warp's 8 lane
// groups shorten the chain: they compute the parameter-only constants of 8
// packets at once, and evaluate 8 rounds of the tan rejection at once on the
// next 16 resident half packets (a lane keeps its first accepted round, the
// packet ends with the round its last lane first accepts: the same draws and
// values as round by round).  The engine window, its half cache and the
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

constexpr int kBvWarps = 1;  // engines per CTA
// per warp: two lane windows (the newest block and the one before)
constexpr size_t kBvWarpBytes = (size_t)2 * kLanes * kN * 8;
// with the newest block's 624 half packets stored tempered beside them
constexpr size_t kBvWarpBytesBuf = kBvWarpBytes + (size_t)2 * kN * 16;

__device__ __forceinline__ float bv_ur(uint32_t x) { return u2f((x & 0x7fffffu) | (127u << 23)) - 1.0f; }

// a lane's constants of BinomialVGen<int32_t>::packetOp
struct BvLane {
  float ptrials, mean, g1, sqrt_v, lsp, lsq;
};

// one round of the tan rejection on draws (u, u2): the proposal fres and
// whether this lane accepts it
__device__ __forceinline__ bool bv_trial(const BvLane& L, uint32_t w1, uint32_t w2, float& fres) {
  float sn, cs;
  sincosf_((float)3.1415926535897932 * bv_ur(w1), sn, cs);
  const float ys = sn / cs;
  fres = truncf(L.sqrt_v * ys + L.mean);
  const float p1 = ((float)1.2 * L.sqrt_v) * (1.0f + ys * ys);
  float t = (L.g1 - lgamma_approxf_(fres + 1.0f)) - lgamma_approxf_((L.ptrials + 1.0f) - fres);
  t = t + fres * L.lsp;
  t = t + (L.ptrials - fres) * L.lsq;
  const float p2 = expf_(t);
  const float u2 = bv_ur(w2);
  return (0.0f <= fres) && (fres <= L.ptrials) && (u2 <= p1 * p2);
}

// The draws of a Vmt19937_64 stream as half packets: the engine's cached
// upper half first, then the 624 half packets of each block the warp twists
// (two lane windows in shared memory).  BUF: the newest block's half packets
// are tempered once into a buffer (10 KB more shared memory, a shorter chain
// per draw); otherwise each draw tempers its word as it is read.
template <bool BUF>
struct BvEngineSrc {
  uint64_t (*raw)[kLanes][kN];
  uint32_t (*hw)[4];
  EngState* st;
  int64_t max_blocks;
  int lane;
  bool pending, abort = false;
  int h = 2 * kN, cur = 0;
  int64_t nb = 0;

  __device__ __forceinline__ uint32_t next() {
    if (pending) {
      pending = false;
      return st->half_cache[lane & 3];
    }
    if (h == 2 * kN) {
      if (nb >= max_blocks) {
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
          }
          if (BUF) {
            uint64_t pk[kLanes];
#pragma unroll
            for (int l = 0; l < kLanes; ++l) pk[l] = mt_temper(nw[l][i]);
            hw[2 * i][0] = (uint32_t)pk[0];
            hw[2 * i][1] = (uint32_t)(pk[0] >> 32);
            hw[2 * i][2] = (uint32_t)pk[1];
            hw[2 * i][3] = (uint32_t)(pk[1] >> 32);
            hw[2 * i + 1][0] = (uint32_t)pk[2];
            hw[2 * i + 1][1] = (uint32_t)(pk[2] >> 32);
            hw[2 * i + 1][2] = (uint32_t)pk[3];
            hw[2 * i + 1][3] = (uint32_t)(pk[3] >> 32);
          }
        }
        __syncwarp();
      }
      cur ^= 1;
      ++nb;
      h = 0;
    }
    return half(h++);
  }
  // word (lane & 3) of half packet hh of the newest block: packet hh / 2,
  // its lanes 0-1 (hh even) or 2-3 (hh odd), low or high half of the lane
  __device__ __forceinline__ uint32_t half(int hh) const {
    if (BUF) return hw[hh][lane & 3];
    const uint64_t t = mt_temper(raw[cur][2 * (hh & 1) + ((lane & 3) >> 1)][hh >> 1]);
    return (lane & 1) ? (uint32_t)(t >> 32) : (uint32_t)t;
  }
  // the next 16 half packets are resident (no cached half, no new block)
  __device__ bool peek_ok() const { return !pending && h + 16 <= 2 * kN; }
  __device__ uint32_t peek(int k) const { return half(h + k); }
  __device__ void skip(int m) { h += m; }
  __device__ void mark() {}
};

// The draws of a scalar engine (std::mt19937_64, P8_mt19937_64) as SSE
// uniform packets: RawbitsMaker<Packet4i, Rng, uint64_t, scalar_fullbit>::
// rawbits_34 (arch/SSE/RandUtils.h:36-55) takes two 64-bit draws, the first
// in int32 lanes 0-1 (GCC evaluates _mm_set_epi64x's arguments right to left).
struct BvWordsSrc {
  const uint64_t* w;
  int64_t nh;  // half packets available
  int lane;
  bool abort = false;
  int64_t q = 0, q0 = 0;

  __device__ uint32_t at(int64_t hh) const {
    const uint64_t x = w[2 * hh + ((lane & 3) >> 1)];
    return (lane & 1) ? (uint32_t)(x >> 32) : (uint32_t)x;
  }
  __device__ __forceinline__ uint32_t next() {
    if (q >= nh) {
      abort = true;
      return 0u;
    }
    return at(q++);
  }
  __device__ bool peek_ok() const { return q + 16 <= nh; }
  __device__ uint32_t peek(int k) const { return at(q + k); }
  __device__ void skip(int m) { q += m; }
  __device__ void mark() { q0 = q; }
};

// npk packets of BinomialVGen<int32_t>::packetOp from src, outputs and
// parameters at element off + 4e + lane.  Returns the packets completed
// (fewer than npk when src ran out).
template <class Src>
__device__ __forceinline__ int64_t bv_chain(Src& src, const BinomVArgs& a, int64_t off, int64_t npk, int32_t* out, int lane) {
  auto mask4 = [&](bool pr) -> unsigned { return __ballot_sync(0xffffffffu, pr && lane < 4) & 0xfu; };
  const int jl = lane & 3;  // every group of 4 lanes holds the packet's 4 lanes
  for (int64_t e0 = 0; e0 < npk; e0 += 8) {
    // the parameter-only constants of packets e0 .. e0 + 7, group g = lane / 4
    // computing those of packet e0 + g
    int32_t trg = 0;
    float pvg = 0.0f;
    if (e0 + (lane >> 2) < npk) {
      const int64_t i = off + (e0 + (lane >> 2)) * 4 + jl;
      trg = a.trials ? __ldg(a.trials + i) : a.trials0;
      pvg = a.p ? __ldg(a.p + i) : a.p0;
    }
    const float spg = pvg < 1.0f - pvg ? pvg : 1.0f - pvg;  // pmin(p, 1 - p)
    const float meang = (float)trg * spg;
    const float g1g = lgamma_approxf_((float)trg + 1.0f);
    const float svg = sqrtf((2.0f * meang) * (1.0f - spg));
    const float lspg = logf_(spg), lsqg = logf_(1.0f - spg);
    const float neg = expf_(-meang);
    const int kend = npk - e0 < 8 ? (int)(npk - e0) : 8;
    for (int kk = 0; kk < kend; ++kk) {
      src.mark();
      const int srcl = (kk << 2) | jl;
      const int32_t tr = __shfl_sync(0xffffffffu, trg, srcl);
      const float pv = __shfl_sync(0xffffffffu, pvg, srcl);
      const float small_p = __shfl_sync(0xffffffffu, spg, srcl);
      const float ptrials = (float)tr;
      const float mean = __shfl_sync(0xffffffffu, meang, srcl);
      const float g1 = __shfl_sync(0xffffffffu, g1g, srcl);
      const float sqrt_v = __shfl_sync(0xffffffffu, svg, srcl);
      const float lsp = __shfl_sync(0xffffffffu, lspg, srcl), lsq = __shfl_sync(0xffffffffu, lsqg, srcl);
      const float ne = __shfl_sync(0xffffffffu, neg, srcl);
      bool valid = mean < 1.0f;
      float vres = 0.0f;
      if (mask4(valid)) {
        float val = 1.0f;
        int32_t res = 0;
        for (;;) {
          val = val * bv_ur(src.next());
          if (src.abort) break;
          const bool c = (ne < val) && valid;
          if (mask4(c) == 0) break;
          res += c ? 1 : 0;
        }
        vres = (float)res;
      }
      if (!src.abort && mask4(valid) != 0xfu) {
        const BvLane L{ptrials, mean, g1, sqrt_v, lsp, lsq};
        for (;;) {
          if (src.peek_ok()) {
            // rounds r .. r + 7 at once, group g = lane / 4 evaluating round
            // r + g on half packets 2g, 2g + 1 ahead; a lane keeps its first
            // accepted proposal and the packet ends with the round in which
            // its last lane first accepts, as round by round
            const int g = lane >> 2;
            float fres;
            const bool acc = bv_trial(L, src.peek(2 * g), src.peek(2 * g + 1), fres) && !valid;
            const unsigned bal = __ballot_sync(0xffffffffu, acc);
            unsigned mj = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) mj |= ((bal >> (4 * q + jl)) & 1u) << q;
            const int first = mj ? __ffs(mj) - 1 : 8;
            const float ffirst = __shfl_sync(0xffffffffu, fres, ((first & 7) << 2) | jl);
            int end = valid ? -1 : first;
            end = max(end, __shfl_xor_sync(0xffffffffu, end, 1));
            end = max(end, __shfl_xor_sync(0xffffffffu, end, 2));
            if (!valid && first < 8) {
              vres = ffirst;
              valid = true;
            }
            if (end < 8) {
              src.skip(2 * (end + 1));
              break;
            }
            src.skip(16);
            continue;
          }
          float fres;
          const uint32_t w1 = src.next();
          const uint32_t w2 = src.next();
          if (src.abort) break;
          const bool fv = bv_trial(L, w1, w2, fres);
          if (fv && !valid) vres = fres;
          valid = valid || fv;
          if (mask4(valid) == 0xfu) break;
        }
      }
      if (src.abort) return e0 + kk;
      if (lane < 4) out[off + (e0 + kk) * 4 + jl] = (pv == small_p) ? cvtt_f32(vres) : tr - cvtt_f32(vres);
    }
  }
  return npk;
}

template <bool BUF>
__global__ void __launch_bounds__(32 * kBvWarps, 1) k_binom_v(Plan p, BinomVArgs a) {
  extern __shared__ __align__(16) uint64_t bv_dyn[];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kBvWarps + wi;
  if (k >= p.K) return;  // the whole warp
  uint8_t* base = reinterpret_cast<uint8_t*>(bv_dyn) + (size_t)wi * (BUF ? kBvWarpBytesBuf : kBvWarpBytes);
  EngState* st = p.eng + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  BvEngineSrc<BUF> src{reinterpret_cast<uint64_t(*)[kLanes][kN]>(base),
                       reinterpret_cast<uint32_t(*)[4]>(base + kBvWarpBytes), st, a.max_blocks, lane,
                       st->half_valid != 0};
  for (int i = lane; i < kLanes * kN; i += 32) src.raw[0][i / kN][i % kN] = st->win[i / kN][i % kN];
  __syncwarp();
  bv_chain(src, a, off, n / 4, static_cast<int32_t*>(p.out), lane);

  // ---- state after the call (as k_negbin: the last draw's block, the
  // cached upper half when a packet was split)
  if (src.abort) {
    if (lane == 0) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    return;
  }
  const int h = src.h;
  if (src.nb > 0) {
    const int last = h - 1;       // last half packet drawn from the newest block
    const int rr = last / 2 + 1;  // packets used of it
    uint64_t(*lastb)[kN] = src.raw[src.cur];
    uint64_t(*prevb)[kN] = src.raw[src.cur ^ 1];
    for (int t = lane; t < kLanes * kN; t += 32) {
      const int l = t / kN, i = t % kN;
      st->win[l][i] = (i < kN - rr) ? prevb[l][rr + i] : lastb[l][i - (kN - rr)];
    }
    if (lane < 4) st->half_cache[lane] = (last & 1) == 0 ? src.half(last + 1) : 0u;
    if (lane == 0) {
      st->half_valid = (last & 1) == 0 ? 1 : 0;
      st->consumed += (uint64_t)((src.nb - 1) * kN + rr);
    }
  } else if (lane == 0 && st->half_valid) {
    st->half_valid = 0;  // only the cached half was drawn
  }
}

// One scalar-engine chain over pre-drawn words: res[0] = packets completed,
// res[1] = 64-bit words they consumed.
__global__ void __launch_bounds__(32) k_binom_v_words(const uint64_t* w, int64_t nwords, BinomVArgs a, int32_t* out,
                                                     int64_t npk, int64_t* res) {
  const int lane = threadIdx.x & 31;
  BvWordsSrc src{w, nwords / 2, lane};
  const int64_t done = bv_chain(src, a, 0, npk, out, lane);
  if (lane == 0) {
    res[0] = done;
    res[1] = 2 * (done < npk ? src.q0 : src.q);
  }
}

// PoissonGen<int32_t>, BinomialGen<int32_t>, UniformIntGen<int32_t> and
// NegativeBinomialGen<int32_t> (Discrete.h:855-905, 990-1048, 287-333,
// GammaPoisson.h:55-110) on a scalar engine's pre-drawn
// words, one chain: packets of 4 on SSE packets of two draws each.  Modes: BinomialGen with trials < 25
// (one uniform packet per trial), the multiplicative Poisson loop (PoissonGen
// mean < 12, BinomialGen mean < 1 through its PoissonGen member), and the tan
// rejection through CompressMask (carried lanes in carry[0..3], their count in
// carry[8], kept across chunks of one call).  res[0] = packets completed,
// res[1] = words they consumed.
__global__ void __launch_bounds__(32) k_int_words(const uint64_t* w, int64_t nwords, DistParams d, int32_t* out,
                                                 int64_t npk, int64_t* res, uint32_t* carry) {
  __shared__ uint32_t cb[8];
  const int lane = threadIdx.x & 31;
  BvWordsSrc src{w, nwords / 2, lane};
  auto mask4 = [&](bool pr) -> unsigned { return __ballot_sync(0xffffffffu, pr && lane < 4) & 0xfu; };
  const bool binom = d.kind == GR_BINOMIAL;
  const int mode = d.kind == GR_NEGATIVE_BINOMIAL ? 4
                   : d.kind == GR_UNIFORM_INT     ? 3
                                                  : ((binom && d.ia < 25) ? 0 : (d.ic ? 1 : 2));
  int fc = (int)carry[8];
  if (lane < fc) cb[lane] = carry[lane];
  __syncwarp();
  // CompressMask::compress_append over lanes 0-3 (arch/AVX/PacketFilter.h:147-184)
  auto compress = [&](uint32_t bits, bool acc, uint32_t& r) -> bool {
    const unsigned m = mask4(acc);
    if (m == 0xfu) {
      r = bits;
      return true;
    }
    if (lane < 4 && ((m >> lane) & 1u)) cb[fc + __popc(m & ((1u << lane) - 1))] = bits;
    fc += __popc(m);
    __syncwarp();
    if (fc < 4) return false;
    r = lane < 4 ? cb[lane] : 0u;
    const uint32_t mv = lane < fc - 4 ? cb[4 + lane] : 0u;
    __syncwarp();
    if (lane < fc - 4) cb[lane] = mv;
    fc -= 4;
    __syncwarp();
    return true;
  };
  const BvLane L{d.fh, d.fb, d.fg, d.fa, d.fc, d.fd};  // BinomialGen's tan constants
  int64_t e = 0;
  for (; e < npk; ++e) {
    src.mark();
    const int fc0 = fc;  // the carried lanes before this packet (at most 3)
    const uint32_t cs = lane < fc ? cb[lane] : 0u;
    int32_t r = 0;
    if (mode == 0) {  // res = trials + sum of (p <= u ? -1 : 0) over trials uniform packets
      r = d.ia;
      for (int t = 0; t < d.ia; ++t) r += (d.fa <= bv_ur(src.next())) ? -1 : 0;
    } else if (mode == 1) {
      float val = 1.0f;
      for (;;) {
        val = val * bv_ur(src.next());
        if (src.abort) break;
        const bool c = d.fe < val;
        if (mask4(c) == 0) break;
        r += c ? 1 : 0;
      }
    } else if (mode == 3) {
      // UniformIntGen (Discrete.h:287-333): d.ia = pmin, d.ib = 0 constant /
      // 1 masked bits / 2 rejection on slices of bitsize (d.ncdf) bits with
      // plen (d.ic) compared as signed int32
      if (d.ib == 0) {
        r = d.ia;
      } else {
        uint32_t rx = src.next();
        if (d.ib == 1) {
          r = (int32_t)((rx & d.bitmask) + (uint32_t)d.ia);
        } else {
          int bitcnt = d.ncdf;
          for (;;) {
            if (src.abort) break;
            const uint32_t cands = rx & d.bitmask;
            uint32_t rb;
            if (compress(cands, (int32_t)cands < d.ic, rb)) {
              r = (int32_t)(rb + (uint32_t)d.ia);
              break;
            }
            if (bitcnt + d.ncdf < 32) {
              rx >>= d.ncdf;
              bitcnt += d.ncdf;
            } else {
              rx = src.next();
              bitcnt = d.ncdf;
            }
          }
        }
      }
    } else if (mode == 4) {
      // NegativeBinomialGen (GammaPoisson.h:55-110): a GammaGen<float>(trials,
      // (1 - p) / p) packet (d.ic: 0 exponential, 1 product of d.ia uniforms,
      // 2 tan rejection), then a Poisson draw per lane with that mean; both
      // rejections append to the gamma's CompressMask cache
      const float fpi = (float)3.1415926535897932, eps8 = 1.1920928955078125e-07f / 8;
      float mean = 0.0f;
      if (d.ic == 0) {
        mean = d.fb * (-(logf_(1.0f - bv_ur(src.next())) / 1.0f));
      } else if (d.ic == 1) {
        float y = bv_ur(src.next()) + eps8;
        for (int c = 1; c < d.ia; ++c) y = y * (bv_ur(src.next()) + eps8);
        mean = -(d.fb * logf_(y));
      } else {
        for (;;) {
          float ys, yc;
          sincosf_(fpi * bv_ur(src.next()), ys, yc);
          const float ux = bv_ur(src.next());
          if (src.abort) break;
          const float yx = ys / yc;
          const float xx = d.fc * yx + d.fd;
          const float ub = (yx * yx + 1.0f) * expf_(d.fd * logf_(xx / d.fd) - yx * d.fc);
          uint32_t rb;
          if (compress(f2u(d.fb * xx), (0.0f < xx) && (ux <= ub), rb)) {
            mean = u2f(rb);
            break;
          }
        }
      }
      if (!src.abort) {
        const float pne = expf_(-mean);
        if (mask4(12.0f < mean) == 0) {
          float val = 1.0f;
          for (;;) {
            val = val * bv_ur(src.next());
            if (src.abort) break;
            const bool c = pne < val;
            if (mask4(c) == 0) break;
            r += c ? 1 : 0;
          }
        } else {
          const float sq = sqrtf(2.0f * mean), lm = logf_(mean), g1 = mean * lm - lgamma_approxf_(mean + 1.0f);
          for (;;) {
            float s2, c2;
            sincosf_(fpi * bv_ur(src.next()), s2, c2);
            const float yx = s2 / c2;
            const float fres = truncf(sq * yx + mean);
            const float p1 = (yx * yx + 1.0f) * 0.9f;
            const float u2 = bv_ur(src.next());
            if (src.abort) break;
            const float p2 = expf_((fres * lm - lgamma_approxf_(fres + 1.0f)) - g1);
            uint32_t rb;
            if (compress(f2u(fres), (0.0f <= fres) && (u2 <= p1 * p2), rb)) {
              r = cvtt_f32(u2f(rb));
              break;
            }
          }
        }
      }
    } else {
      for (;;) {
        const uint32_t w1 = src.next();
        const uint32_t w2 = src.next();
        if (src.abort) break;
        bool acc;
        float fres;
        if (binom) {
          acc = bv_trial(L, w1, w2, fres);
        } else {
          float sn, cs2;
          sincosf_((float)3.1415926535897932 * bv_ur(w1), sn, cs2);
          const float yx = sn / cs2;
          fres = truncf(d.fa * yx + d.fb);  // sqrt(2 mean) * yx + mean
          const float p1 = (yx * yx + 1.0f) * 0.9f;
          const float p2 = expf_((fres * d.fc - lgamma_approxf_(fres + 1.0f)) - d.fd);
          acc = (0.0f <= fres) && (bv_ur(w2) <= p1 * p2);
        }
        uint32_t rb;
        if (compress(f2u(fres), acc, rb)) {
          r = cvtt_f32(u2f(rb));
          break;
        }
      }
    }
    if (src.abort) {
      __syncwarp();
      fc = fc0;
      if (lane < fc0) cb[lane] = cs;
      __syncwarp();
      break;
    }
    if (binom && mode != 0 && d.ib) r = d.ia - r;  // p > 1/2: trials - res (not the trials < 25 branch)
    if (lane < 4) out[e * 4 + lane] = r;
  }
  __syncwarp();
  if (lane < fc) carry[lane] = cb[lane];
  if (lane == 0) {
    carry[8] = (uint32_t)fc;
    res[0] = e;
    res[1] = 2 * (e < npk ? src.q0 : src.q);
  }
}

}  // namespace

cudaError_t launch_int_words(const uint64_t* w, int64_t nwords, const DistParams& d, int32_t* out, int64_t npk,
                             int64_t* res, uint32_t* carry, cudaStream_t s) {
  k_int_words<<<1, 32, 0, s>>>(w, nwords, d, out, npk, res, carry);
  return cudaGetLastError();
}

cudaError_t launch_binom_v(const Plan& p, const BinomVArgs& a, cudaStream_t s) {
  static bool attr[64] = {};
  static int sms[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_binom_v<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kBvWarpBytesBuf * kBvWarps));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_binom_v<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(kBvWarpBytes * kBvWarps));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  const unsigned grid = (unsigned)((p.K + kBvWarps - 1) / kBvWarps);
  // the buffered form while every stream's CTA is resident at 30 KB (7 per
  // SM); with more streams the 20 KB form fits 11 per SM
  if ((int64_t)grid <= 7LL * sms[dev])
    k_binom_v<true><<<grid, 32 * kBvWarps, kBvWarpBytesBuf * kBvWarps, s>>>(p, a);
  else
    k_binom_v<false><<<grid, 32 * kBvWarps, kBvWarpBytes * kBvWarps, s>>>(p, a);
  return cudaGetLastError();
}

cudaError_t launch_binom_v_words(const uint64_t* w, int64_t nwords, const BinomVArgs& a, int32_t* out, int64_t npk,
                                 int64_t* res, cudaStream_t s) {
  k_binom_v_words<<<1, 32, 0, s>>>(w, nwords, a, out, npk, res);
  return cudaGetLastError();
}

}  // namespace gr
