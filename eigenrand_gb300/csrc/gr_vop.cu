// Batched vectorize-over-params sampling: many parameter sets in one launch.
//
// Set i is drawn from its own Vmt19937_64(seed + 4 i), seeded in shared
// memory by the CTA that owns the set, with a fresh generator: the same values
// as seeding an engine and calling the per-call API once per set, so the
// batched and per-call paths agree bit for bit, and sets need no engine
// state in HBM.  A set of c samples draws ceil(c / P) packets with the packet
// algorithm and keeps the first c values.
//  * GammaGen<float>(alpha_i, beta_i) (EigenRand/Dists/NormalExp.h:527-604):
//    the branch (GS rejection, exponential, product of alpha uniforms, tan
//    rejection) is chosen per set; every branch is a run of fixed-size trials
//    resolved with the CompressMask automaton (closed forms accept every lane).
//  * BinomialVGen<int32_t> with (trials_i, p_i) (Discrete.h:1124-1192): the
//    multiplicative Poisson loop when trials*min(p,1-p) < 1, else the tan
//    proposal with a per-lane accepted mask; the packet ends when every lane
//    has a value, so its length depends on the data and a walk resolves it.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_math.cuh"
#include "gr_mt.cuh"

namespace gr {
namespace {

constexpr int kMaxTr = 320;
constexpr int kMaxCd = 2560;  // candidate lanes per block: <= 312 trials x 8 (alpha == 1)

__device__ __forceinline__ void seed_engine(uint64_t (*raw)[kN], uint64_t seed) {
  // MersenneTwister::seed (PacketRandomEngine.h:256-265), lane l = seed + l
  if (threadIdx.x < kLanes) {
    uint64_t prev = seed + threadIdx.x;
    raw[threadIdx.x][0] = prev;
    for (int i = 1; i < kN; ++i) {
      prev = (prev ^ (prev >> 62)) * kSeedF + (uint64_t)i;
      raw[threadIdx.x][i] = prev;
    }
  }
}

template <int kT>
__device__ __forceinline__ uint32_t scanT(uint32_t v, uint32_t* warp_tot) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t x = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += x;
  }
  if (lane == 31) warp_tot[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int i = 0; i < kT / 32; ++i) {
      uint32_t t = warp_tot[i];
      warp_tot[i] = acc;
      acc += t;
    }
  }
  __syncthreads();
  return v + warp_tot[w];
}

}  // namespace



constexpr size_t kVopGammaSmem = (size_t)(4 * kLanes * kN + kMaxCd) * 8;

template <int kT>
__global__ void __launch_bounds__(kT) k_vop_gamma(VopArgs va, int64_t set0) {
  extern __shared__ __align__(16) uint64_t dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(dyn);
  uint64_t(*tp)[kN][kLanes] = reinterpret_cast<uint64_t(*)[kN][kLanes]>(dyn + 2 * kLanes * kN);
  uint32_t* cand = reinterpret_cast<uint32_t*>(dyn + 4 * kLanes * kN);
  __shared__ uint32_t tmask[kMaxTr];
  __shared__ uint32_t tscan[kMaxTr];
  __shared__ uint32_t fifo[2][16];
  __shared__ int64_t emit_q[kMaxTr + 2];
  __shared__ uint32_t wt[kT / 32];
  __shared__ int s_tstar;
  constexpr int P = 8;
  const int64_t idx = set0 + blockIdx.x;
  if (idx >= va.nsets) return;
  const int64_t set = va.perm ? va.perm[idx] : idx;
  const int tid = threadIdx.x;
  const int32_t count = va.counts[set];
  if (count <= 0) return;
  const int64_t off = va.offsets[set];
  const float alpha = va.a[set], beta = va.b[set];
  // GammaGen branch for this set, NormalExp.h:533-604
  int type, U;
  const int cnt = (int)alpha;
  if (alpha < 1) { type = 2; U = 3; }
  else if (alpha == 1) { type = 0; U = 1; }
  else if ((float)cnt == alpha && cnt < 20) { type = 1; U = cnt; }
  else { type = 3; U = 2; }
  const int Wt = 8 * U;
  const float inv_a = 1 / alpha, a1 = alpha - 1;
  const float px = (float)(2.7182818284590452 / (alpha + 2.7182818284590452));
  const float sq = sqrtf(2 * alpha - 1);
  const int64_t Npk = (count + P - 1) / P;

  seed_engine(raw[0], va.seed + 4ull * (uint64_t)set);
  __syncthreads();
  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t w) -> uint32_t {
    const int64_t rel = w >> 3;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  int64_t E = 0, t_next = 0;
  int rcnt = 0, fsl = 0, cur = 0;
  const int64_t max_blocks = ((16 * Npk + 4096) * Wt) / (kN * 8) + 64;
  bool done = false;
  for (int64_t nb = 0; nb < max_blocks && !done; ++nb) {
    const int slot = (int)(nb & 1);
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
    });
    cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    const int64_t t_end = ((nb + 1) * kN * 8) / Wt;
    const int B = (int)min((int64_t)kMaxTr, t_end - t_next);
    if (B <= 0) continue;
    for (int base = 0; base < B * P; base += kT) {
      const int e = base + tid;
      const bool valid = e < B * P;
      const int tl = e / P, j = e % P;
      bool acc = false;
      uint32_t cb = 0;
      if (valid) {
        const int64_t w0 = (t_next + tl) * Wt + j;
        if (type == 0) {
          cb = f2u(beta * (-(logf_(1.0f - ur_f(word(w0))) / 1.0f)));
          acc = true;
        } else if (type == 1) {
          float y = ur_f(word(w0)) + 1.1920928955078125e-07f / 8;
          for (int t = 1; t < U; ++t) y = y * (ur_f(word(w0 + 8 * t)) + 1.1920928955078125e-07f / 8);
          cb = f2u(-(beta * logf_(y)));
          acc = true;
        } else if (type == 2) {
          const float ux = ur_f(word(w0));
          const float vx = ur_f(word(w0 + 8)) + 1.1920928955078125e-07f / 8;
          const float ux2 = ur_f(word(w0 + 16));
          const float lv = logf_(vx);
          float xx, qx;
          if (ux < px) {
            xx = expf_(inv_a * lv);
            qx = expf_(-xx);
          } else {
            xx = 1.0f - lv;
            qx = expf_(logf_(xx) * a1);
          }
          cb = f2u(beta * xx);
          acc = ux2 < qx;
        } else {
          float ys, yc;
          sincosf_((float)3.1415926535897932 * ur_f(word(w0)), ys, yc);
          const float yx = ys / yc;
          const float xx = sq * yx + a1;
          const float ub = (yx * yx + 1.0f) * expf_(a1 * logf_(xx / a1) - yx * sq);
          acc = (0.0f < xx) && (ur_f(word(w0 + 8)) <= ub);
          cb = f2u(beta * xx);
        }
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, acc);
      if (valid) {
        cand[tl * P + j] = cb;
        if (j == 0) tmask[tl] = (bal >> (threadIdx.x & 31 & ~(P - 1))) & 0xffu;
      }
    }
    __syncthreads();
    // each thread sums kMaxTr / kT consecutive trials, then one block scan
    constexpr int PER = kMaxTr / kT;
    uint32_t vv[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int tl = PER * tid + q;
      vv[q] = 0;
      if (tl < B) {
        const int c = __popc(tmask[tl]);
        vv[q] = c == P ? (1u << 16) : (uint32_t)c;
      }
      sum += vv[q];
    }
    uint32_t run = scanT<kT>(sum, wt) - sum;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int tl = PER * tid + q;
      if (tl < B) tscan[tl] = run;
      run += vv[q];
    }
    if (tid == 0) s_tstar = -1;
    __syncthreads();
    for (int tl = tid; tl < B; tl += kT) {
      const int c = __popc(tmask[tl]);
      const int64_t nf = tscan[tl] >> 16, at = (int64_t)rcnt + (tscan[tl] & 0xffffu);
      const bool full = c == P, cross = !full && ((at + c) / P > at / P);
      const int64_t eidx = E + nf + at / P;
      if (cross) emit_q[at / P] = eidx;
      if ((full || cross) && eidx == Npk - 1) s_tstar = tl;
    }
    __syncthreads();
    const int tstar = s_tstar;
    const int Bu = tstar >= 0 ? tstar + 1 : B;
    const int cl = __popc(tmask[Bu - 1]);
    const int64_t nf_end = (tscan[Bu - 1] >> 16) + (cl == P ? 1 : 0);
    const int64_t a_end = (int64_t)rcnt + (tscan[Bu - 1] & 0xffffu) + (cl == P ? 0 : cl);
    const int64_t qe = a_end / P;
    float* out = reinterpret_cast<float*>(va.out) + off;
    for (int e = tid; e < Bu * P; e += kT) {
      const int tl = e / P, j = e % P;
      const uint32_t m = tmask[tl];
      const int c = __popc(m);
      const int64_t nf = tscan[tl] >> 16, at = (int64_t)rcnt + (tscan[tl] & 0xffffu);
      const uint32_t v = cand[tl * P + j];
      if (c == P) {
        const int64_t o = (E + nf + at / P) * P + j;
        if (o < count) out[o] = u2f(v);
      } else if ((m >> j) & 1u) {
        const int64_t f = at + __popc(m & ((1u << j) - 1));
        if (f / P < qe) {
          const int64_t o = emit_q[f / P] * P + f % P;
          if (o < count) out[o] = u2f(v);
        } else {
          fifo[fsl ^ 1][f - qe * P] = v;
        }
      }
    }
    if (tid < rcnt) {
      if (tid / P < qe) {
        const int64_t o = emit_q[tid / P] * P + tid % P;
        if (o < count) out[o] = u2f(fifo[fsl][tid]);
      } else {
        fifo[fsl ^ 1][tid - qe * P] = fifo[fsl][tid];
      }
    }
    __syncthreads();
    E += nf_end + qe;
    rcnt = (int)(a_end - qe * P);
    fsl ^= 1;
    t_next += Bu;
    done = tstar >= 0;
  }
  if (!done && tid == 0) atomicOr(va.status, (int)GR_DEV_REJECT_LIMIT);
}

// ------------------------------------------------------------------ binomial
constexpr int kBRing = 1280;  // start positions (half packets) kept
constexpr int kBRec = 704;
constexpr size_t kVopBinSmem = (size_t)(4 * kLanes * kN) * 8 + (size_t)kBRing * 4 * 4 + (size_t)kBRing * 4 + kBRec * 16;

template <int kT>
__global__ void __launch_bounds__(kT) k_vop_binomial(VopArgs va, int64_t set0) {
  extern __shared__ __align__(16) uint64_t dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(dyn);
  uint64_t(*tp)[kN][kLanes] = reinterpret_cast<uint64_t(*)[kN][kLanes]>(dyn + 2 * kLanes * kN);
  float* fres_r = reinterpret_cast<float*>(dyn + 4 * kLanes * kN);  // [kBRing][4] value at position
  uint32_t* aux = reinterpret_cast<uint32_t*>(fres_r + kBRing * 4);  // Poisson: L; tan: accept mask
  int64_t* rec = reinterpret_cast<int64_t*>(aux + kBRing);  // start position per output packet
  uint64_t* rec_first = reinterpret_cast<uint64_t*>(rec + kBRec);  // tan: 4 x 16-bit lane offsets
  __shared__ int s_nrec, s_stop, s_err;
  __shared__ int64_t s_ebase;
  constexpr int P = 4;
  constexpr int kLookB = 64;
  const int64_t idx = set0 + blockIdx.x;
  if (idx >= va.nsets) return;
  const int64_t set = va.perm ? va.perm[idx] : idx;
  const int tid = threadIdx.x;
  const int32_t count = va.counts[set];
  if (count <= 0) return;
  const int64_t off = va.offsets[set];
  const int32_t n = va.trials[set];
  const float p = va.a[set];
  // packetOp's per-lane constants (uniform over the set)
  const float small_p = p < 1.0f - p ? p : 1.0f - p;
  const float ptrials = (float)n;
  const float mean = ptrials * small_p;
  const float g1 = lgamma_approxf_(ptrials + 1.0f);
  const float sqrt_v = sqrtf((2.0f * mean) * (1.0f - small_p));
  const float lsp = logf_(small_p), lsq = logf_(1.0f - small_p);
  const float ne = expf_(-mean);
  const bool poisson = mean < 1.0f;
  const bool flip = !(p == small_p);
  const int64_t Npk = (count + P - 1) / P;

  seed_engine(raw[0], va.seed + 4ull * (uint64_t)set);
  if (tid == 0) {
    s_stop = 0;
    s_err = 0;
  }
  __syncthreads();
  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t w) -> uint32_t {
    const int64_t rel = w >> 3;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  int64_t s = 0, E = 0, done_pos = 0;
  int cur = 0;
  const int64_t max_blocks = (Npk * 64) / (2 * kN) + 64;
  int64_t nb = 0;
  for (; nb < max_blocks; ++nb) {
    const int slot = (int)(nb & 1);
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
    });
    cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    const int64_t lim = 2 * (nb + 1) * kN - kLookB;  // half packets whose lookahead exists
    if (tid == 0 && lim - s > kBRing) s_err = 1;
    for (int64_t x = done_pos + tid; x < lim; x += kT) {
      const int ri = (int)(x % kBRing);
      if (poisson) {
        float val[4] = {1, 1, 1, 1};
        int kk[4] = {0, 0, 0, 0}, L = 0;
        bool any = true;
        for (int it = 0; it < kLookB && any; ++it) {
          any = false;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            val[j] = val[j] * ur_f(word((x + it) * 4 + j));
            const bool c = ne < val[j];
            kk[j] += c ? 1 : 0;
            any |= c;
          }
          L = it + 1;
        }
        if (any) atomicOr(&s_err, 1);
        aux[ri] = (uint32_t)L;
#pragma unroll
        for (int j = 0; j < 4; ++j) fres_r[ri * 4 + j] = (float)kk[j];
      } else {
        uint32_t m = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float sn, cs;
          sincosf_((float)3.1415926535897932 * ur_f(word(x * 4 + j)), sn, cs);
          const float ys = sn / cs;
          const float fres = truncf(sqrt_v * ys + mean);
          const float p1 = ((float)1.2 * sqrt_v) * (1.0f + ys * ys);
          float t = (g1 - lgamma_approxf_(fres + 1.0f)) - lgamma_approxf_((ptrials + 1.0f) - fres);
          t = t + fres * lsp;
          t = t + (ptrials - fres) * lsq;
          const float p2 = expf_(t);
          const bool acc = (0.0f <= fres) && (fres <= ptrials) && (ur_f(word((x + 1) * 4 + j)) <= p1 * p2);
          fres_r[ri * 4 + j] = fres;
          m |= acc ? (1u << j) : 0u;
        }
        aux[ri] = m;
      }
    }
    done_pos = max(done_pos, lim);
    __syncthreads();
    if (tid == 0) {
      s_ebase = E;
      int nrec = 0;
      while (E < Npk && nrec < kBRec) {
        if (poisson) {
          if (s >= done_pos) break;
          rec[nrec++] = s;  // value: counts at s
          s += aux[s % kBRing];
        } else {
          // lanes take the value of their first accepting iteration (s + 2i)
          int need = 0xf, first[4] = {0, 0, 0, 0};
          int64_t x = s;
          bool ok = true;
          while (need) {
            if (x >= done_pos) {
              ok = false;
              break;
            }
            const uint32_t m = aux[x % kBRing] & (uint32_t)need;
            for (int j = 0; j < 4; ++j)
              if ((m >> j) & 1u) first[j] = (int)(x - s);
            need &= ~(int)m;
            x += 2;
          }
          if (!ok) break;
          // the 4 lanes' accepting positions, as offsets from s (< kBRing)
          rec[nrec] = s;
          rec_first[nrec] = (uint64_t)first[0] | ((uint64_t)first[1] << 16) | ((uint64_t)first[2] << 32) |
                            ((uint64_t)first[3] << 48);
          ++nrec;
          s = x;
        }
        ++E;
      }
      s_nrec = nrec;
      if (E >= Npk) s_stop = 1;
    }
    __syncthreads();
    const int nrec = s_nrec;
    const int64_t e0 = s_ebase;
    int32_t* out = reinterpret_cast<int32_t*>(va.out) + off;
    for (int e = tid; e < nrec * P; e += kT) {
      const int i = e / P, j = e % P;
      const int64_t r = rec[i];
      float v;
      if (poisson) {
        v = fres_r[(int)(r % kBRing) * 4 + j];
      } else {
        const int64_t rel = (int64_t)((rec_first[i] >> (16 * j)) & 0xffffu);
        v = fres_r[(int)((r + rel) % kBRing) * 4 + j];
      }
      const int32_t res = (int32_t)v;
      const int64_t o = (e0 + i) * P + j;
      if (o < count) out[o] = flip ? n - res : res;
    }
    __syncthreads();
    if (s_stop) break;
  }
  if (tid == 0 && (!s_stop || s_err)) atomicOr(va.status, (int)GR_DEV_REJECT_LIMIT);
}

template <int kT>
static cudaError_t run_vop(int kk, const VopArgs& va, cudaStream_t s) {
  static bool attr[64][2] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev][kk]) {
    cudaError_t e = kk == 0 ? cudaFuncSetAttribute(k_vop_gamma<kT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)kVopGammaSmem)
                            : cudaFuncSetAttribute(k_vop_binomial<kT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)kVopBinSmem);
    if (e != cudaSuccess) return e;
    attr[dev][kk] = true;
  }
  for (int64_t s0 = 0; s0 < va.nsets; s0 += ((int64_t)1 << 30)) {
    const int64_t nb = min(va.nsets - s0, (int64_t)1 << 30);
    if (kk == 0) k_vop_gamma<kT><<<(unsigned)nb, kT, kVopGammaSmem, s>>>(va, s0);
    else k_vop_binomial<kT><<<(unsigned)nb, kT, kVopBinSmem, s>>>(va, s0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// threads: 160 or 320 (the twist uses 156 threads; the rest evaluate trials)
cudaError_t launch_vop(int kind, int threads, const VopArgs& va, cudaStream_t s) {
  const int kk = kind == GR_GAMMA ? 0 : 1;
  if (threads == 320) return run_vop<320>(kk, va, s);
  return run_vop<160>(kk, va, s);
}

}  // namespace gr
