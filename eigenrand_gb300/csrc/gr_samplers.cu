// Samplers whose draws per output span several packets.
//
// k_staged: a unit of P outputs consumes a fixed run of U packets (or U half
// packets for the int32 kinds), e.g. GammaGen with integer alpha < 20
// multiplies alpha uniforms per output (EigenRand/Dists/NormalExp.h:577-587),
// BinomialGen with trials < 25 compares `trials` uniforms
// (Discrete.h:1000-1009).  The CTA keeps the tempered packets of the last two
// blocks in shared memory; a unit is evaluated as soon as its last packet
// exists.  Fixed consumption means jump-ahead segments still apply.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "../../include/gpurand.h"
#include "gr_exact.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_math.cuh"
#include "gr_mt.cuh"

namespace gr {

enum StagedDT { SD_F32 = 0, SD_F64 = 1, SD_I32H = 2 };

template <int KIND, int DT>
__global__ void __launch_bounds__(160)
    k_staged(Plan p, DistParams d, const CallSnap* snap, int U, int64_t Us, int delta) {
  __shared__ uint64_t raw[2][kLanes][kN];
  __shared__ uint64_t tp[2][kN][kLanes];
  const int k = blockIdx.x / p.S, s = blockIdx.x % p.S;
  const int tid = threadIdx.x;
  EngState* st = p.eng + k;
  constexpr int P = DT == SD_F32 ? 8 : 4;

  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;

  // half-packet kinds start with the engine's cached half, if any
  int c0w = 0;
  uint32_t cw[4] = {0, 0, 0, 0};
  if (DT == SD_I32H) {
    const int hv = p.S > 1 ? snap[k].half_valid : st->half_valid;
    if (hv) {
      c0w = 4;
#pragma unroll
      for (int q = 0; q < 4; ++q) cw[q] = p.S > 1 ? snap[k].half_cache[q] : st->half_cache[q];
    }
  }
  const int64_t wpu = (DT == SD_I32H) ? 4 * (int64_t)U : 8 * (int64_t)U;  // u32 words per unit
  const int64_t Nu = n / P;
  const int64_t u_beg = (int64_t)s * Us;
  const int64_t u_end = min(u_beg + Us, Nu);
  if (u_beg >= Nu) return;
  const bool last = (u_end == Nu);
  const int64_t seg_p0 = (s == 0) ? 0 : (int64_t)s * p.J - delta;
  // last packet holding a word of unit u_end-1
  const int64_t w_last = u_end * wpu - 1 - c0w;
  const int64_t p_last = w_last < 0 ? -1 : w_last / 8;
  const int64_t np_seg = p_last + 1 - seg_p0;

  // lane windows
  if (s == 0 && p.S > 1) load_window(raw[0], p.prefix + (size_t)k * kLanes * kPrefixLen, kPrefixLen);
  else if (s == 0) load_window(raw[0], &st->win[0][0], kN);
  else load_window(raw[0], p.segwin + ((size_t)k * (p.S - 1) + (s - 1)) * kLanes * kN, kN);
  __syncthreads();

  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t wq) -> uint32_t {  // cache-inclusive u32 word
    if (wq < c0w) return cw[wq];
    const int64_t w = wq - c0w;
    const int64_t pp = w >> 3;
    const int64_t rel = pp - seg_p0;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  auto rword = [&](int64_t r) -> uint64_t {  // u64 lane value r of the packet stream (full kinds)
    const int64_t pp = r >> 2;
    const int64_t rel = pp - seg_p0;
    return ring_packet(tp, rel, ring_new, ring_slot)[r & 3];
  };

  int64_t u_next = u_beg;
  int cur = 0;
  int64_t nb = 0;
  for (int64_t base = 0; base < np_seg || (np_seg <= 0 && base == 0); base += kN, ++nb) {
    if (np_seg > 0) {
      uint64_t(*old)[kN] = raw[cur];
      uint64_t(*nw)[kN] = raw[cur ^ 1];
      const int slot = (int)(nb & 1);
      mt_block(old, nw, [&](int i, const uint64_t* pk) {
#pragma unroll
        for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
      });
      cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    }
    // units whose last packet is now available
    const int64_t avail = seg_p0 + base + kN;  // packets [.., avail) exist
    int64_t u_ready = u_end;
    {
      // largest u with ((u+1)*wpu - 1 - c0w)/8 < avail
      const int64_t lim = avail * 8 + c0w;  // words (cache-inclusive) available
      const int64_t by_words = lim / wpu;
      if (by_words < u_ready) u_ready = by_words;
    }
    const int64_t cnt = (u_ready - u_next) * P;
    for (int64_t e = tid; e < cnt; e += blockDim.x) {
      const int64_t u = u_next + e / P;
      const int j = (int)(e % P);
      const int64_t o = off + u * P + j;
      if (DT == SD_F32) {
        const int64_t w0 = u * wpu + j;  // full kinds: c0w == 0
        if (KIND == GR_GAMMA || KIND == GR_CHI_SQUARED) {
          float y = ur_f(word(w0)) + 1.1920928955078125e-07f / 8;
          for (int t = 1; t < U; ++t) y = y * (ur_f(word(w0 + 8 * t)) + 1.1920928955078125e-07f / 8);
          reinterpret_cast<float*>(p.out)[o] = -(d.fb * logf_(y));
        } else if (KIND == GR_STUDENT_T) {
          const float u1 = 1.0f - ur_f(word(w0));
          const float u2 = ur_f(word(w0 + 8));
          // StudentTVGen (NormalExp.h:327-342): n of the element, -2 / n per lane
          const float nn = (d.flags & kParamVecA) ? __ldg(static_cast<const float*>(d.vparam) + o) : d.fa;
          const float ex = (d.flags & kParamVecA) ? -2.0f / nn : d.fc;
          const float radius = sqrtf(nn * (expf_(logf_(u1) * ex) - 1.0f));
          float sn, cs;
          sincosf_((float)(2 * 3.1415926535897932) * u2, sn, cs);
          reinterpret_cast<float*>(p.out)[o] = radius * sn;
        }
      } else if (DT == SD_F64) {
        const int64_t r0 = u * (int64_t)U * 4 + j;
        if (KIND == GR_GAMMA || KIND == GR_CHI_SQUARED) {
          double y = ur_d(rword(r0)) + 2.220446049250313e-16 / 8;
          for (int t = 1; t < U; ++t) y = y * (ur_d(rword(r0 + 4 * t)) + 2.220446049250313e-16 / 8);
          const double l = log_(y);
          reinterpret_cast<double*>(p.out)[o] = (d.flags & kParamUnitScale) ? -l : -(d.db * l);
        } else if (KIND == GR_STUDENT_T) {
          const double u1 = one_minus_ur_d(rword(r0));
          const double u2 = ur_d(rword(r0 + 4));
          const double nn = (d.flags & kParamVecA) ? __ldg(static_cast<const double*>(d.vparam) + o) : d.da;
          const double ex = (d.flags & kParamVecA) ? -2.0 / nn : d.dc;
          const double radius = sqrt(nn * (exp_(log_(u1) * ex) - 1.0));
          double sn, cs;
          sincos_((2 * 3.1415926535897932) * u2, sn, cs);
          reinterpret_cast<double*>(p.out)[o] = radius * sn;
        }
      } else {  // int32 over half packets
        const int64_t w0 = u * wpu + j;
        if (KIND == GR_BINOMIAL) {
          int32_t res = d.ia;  // trials
          for (int t = 0; t < U; ++t) res += (d.fa <= ur_f(word(w0 + 4 * t))) ? -1 : 0;
          reinterpret_cast<int32_t*>(p.out)[o] = res;
        }
      }
    }
    u_next = u_ready;
    __syncthreads();
    if (u_next >= u_end) break;
  }

  if (last) {
    // the loop stops right after the block holding p_last: ceil(np_seg/312)
    // blocks were generated and raw[cur] is the last of them
    if (np_seg > 0) {
      const int64_t nblk = (np_seg + kN - 1) / kN;
      const int rr2 = (int)(np_seg - (nblk - 1) * kN);  // in [1, 312]
      store_window(st, raw[cur], raw[cur ^ 1], rr2);
    }
    if (tid == 0) {
      if (DT == SD_I32H) {
        // the last unit ends mid-packet: its upper half stays cached
        const bool half_left = (w_last >= 0) && ((w_last & 7) == 3);
        if (half_left) {
          const int64_t rel = p_last - seg_p0;
          const int slot = (int)((rel / kN) & 1);
          st->half_cache[0] = (uint32_t)tp[slot][rel % kN][2];
          st->half_cache[1] = (uint32_t)(tp[slot][rel % kN][2] >> 32);
          st->half_cache[2] = (uint32_t)tp[slot][rel % kN][3];
          st->half_cache[3] = (uint32_t)(tp[slot][rel % kN][3] >> 32);
          st->half_valid = 1;
        } else {
          st->half_valid = 0;
        }
      }
      st->consumed += (uint64_t)(p_last + 1);
    }
  }
}

// The staged kinds drawn with a scalar engine as the Urng: output packet k
// reads U uniform packets from pre-drawn 64-bit words, float packets as
// rawbits_34 of three draws (c.lo, c.hi, b.lo, top bytes, b.hi, a.lo, a.hi,
// top bytes; a the first draw), double packets as four draws in order; the
// same per-lane arithmetic as k_staged.  One thread per output lane.
template <int KIND, int DT>
__global__ void __launch_bounds__(256) k_sx_staged(const uint64_t* w, void* out, int64_t npk, DistParams d, int U) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  const int64_t g = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (g >= npk * P) return;
  const int64_t k = g / P;
  const int j = (int)(g % P);
  if (DT == SD_F32) {
    // lane j of uniform packet t of output packet k
    auto word = [&](int t) -> uint32_t {
      const uint64_t* q = w + 3 * (k * U + t);
      const uint32_t v[6] = {(uint32_t)q[2], (uint32_t)(q[2] >> 32), (uint32_t)q[1], (uint32_t)(q[1] >> 32),
                             (uint32_t)q[0], (uint32_t)(q[0] >> 32)};
      switch (j) {
        case 0: return v[0];
        case 1: return v[1];
        case 2: return v[2];
        case 3: return (v[0] >> 24) | ((v[1] >> 24) << 8) | ((v[2] >> 24) << 16) | ((v[2] >> 24) << 24);
        case 4: return v[3];
        case 5: return v[4];
        case 6: return v[5];
        default: return (v[3] >> 24) | ((v[4] >> 24) << 8) | ((v[5] >> 24) << 16) | ((v[5] >> 24) << 24);
      }
    };
    if (KIND == GR_GAMMA) {
      float y = ur_f(word(0)) + 1.1920928955078125e-07f / 8;
      for (int t = 1; t < U; ++t) y = y * (ur_f(word(t)) + 1.1920928955078125e-07f / 8);
      static_cast<float*>(out)[g] = -(d.fb * logf_(y));
    } else {  // GR_STUDENT_T
      const float u1 = 1.0f - ur_f(word(0));
      const float u2 = ur_f(word(1));
      const float radius = sqrtf(d.fa * (expf_(logf_(u1) * d.fc) - 1.0f));
      float sn, cs;
      sincosf_((float)(2 * 3.1415926535897932) * u2, sn, cs);
      static_cast<float*>(out)[g] = radius * sn;
    }
  } else {
    const uint64_t* q = w + 4 * k * U + j;
    if (KIND == GR_GAMMA) {
      double y = ur_d(q[0]) + 2.220446049250313e-16 / 8;
      for (int t = 1; t < U; ++t) y = y * (ur_d(q[4 * t]) + 2.220446049250313e-16 / 8);
      const double l = log_(y);
      static_cast<double*>(out)[g] = (d.flags & kParamUnitScale) ? -l : -(d.db * l);
    } else {  // GR_STUDENT_T
      const double u1 = one_minus_ur_d(q[0]);
      const double u2 = ur_d(q[4]);
      const double radius = sqrt(d.da * (exp_(log_(u1) * d.dc) - 1.0));
      double sn, cs;
      sincos_((2 * 3.1415926535897932) * u2, sn, cs);
      static_cast<double*>(out)[g] = radius * sn;
    }
  }
}

cudaError_t launch_sx_staged(const uint64_t* w, void* out, int64_t npk, const DistParams& d, int U,
                             cudaStream_t s) {
  const int P = d.dtype == GR_F32 ? 8 : 4;
  const unsigned blocks = (unsigned)((npk * P + 255) / 256);
  const bool gam = d.kind == GR_GAMMA;
  if (d.dtype == GR_F32) {
    if (gam) k_sx_staged<GR_GAMMA, SD_F32><<<blocks, 256, 0, s>>>(w, out, npk, d, U);
    else k_sx_staged<GR_STUDENT_T, SD_F32><<<blocks, 256, 0, s>>>(w, out, npk, d, U);
  } else {
    if (gam) k_sx_staged<GR_GAMMA, SD_F64><<<blocks, 256, 0, s>>>(w, out, npk, d, U);
    else k_sx_staged<GR_STUDENT_T, SD_F64><<<blocks, 256, 0, s>>>(w, out, npk, d, U);
  }
  return cudaGetLastError();
}

template <int KIND, int DT>
static cudaError_t run_staged(const Plan& p, const DistParams& d, const CallSnap* snap, int U, int64_t Us,
                              int delta, cudaStream_t s) {
  k_staged<KIND, DT><<<p.K * p.S, 160, 0, s>>>(p, d, snap, U, Us, delta);
  return cudaGetLastError();
}

cudaError_t launch_staged(const Plan& p, const DistParams& d, const CallSnap* snap, int U, int64_t Us, int delta,
                          cudaStream_t s) {
  if (d.kind == GR_GAMMA || d.kind == GR_CHI_SQUARED) {
    if (d.dtype == GR_F32) return run_staged<GR_GAMMA, SD_F32>(p, d, snap, U, Us, delta, s);
    if (d.dtype == GR_F64) return run_staged<GR_GAMMA, SD_F64>(p, d, snap, U, Us, delta, s);
  }
  if (d.kind == GR_STUDENT_T) {
    if (d.dtype == GR_F32) return run_staged<GR_STUDENT_T, SD_F32>(p, d, snap, U, Us, delta, s);
    if (d.dtype == GR_F64) return run_staged<GR_STUDENT_T, SD_F64>(p, d, snap, U, Us, delta, s);
  }
  if (d.kind == GR_BINOMIAL && d.dtype == GR_I32) return run_staged<GR_BINOMIAL, SD_I32H>(p, d, snap, U, Us, delta, s);
  return cudaErrorNotSupported;
}

}  // namespace gr

namespace gr {

// ===========================================================================
// k_reject: rejection samplers driven by CompressMask::compress_append
// (EigenRand/arch/AVX/PacketFilter.h:147-184).  Each trial consumes a fixed
// run of Wt words and yields P candidates with an accept mask.  The
// reference's packetOp loop is an automaton over trials: a fully accepted
// trial is returned as is; otherwise its accepted lanes are appended, in lane
// order, to a FIFO carried in the generator, and a packet is returned once
// the FIFO holds P lanes.  With  NF_t = fully accepted trials before t  and
// A_t = carried lanes + lanes appended before t,  trial t's emission (if any)
// is packet  E + NF_t + floor(A_t / P),  so a batch of trials is resolved with
// one block-wide prefix sum.  The call stops at the trial that completes its
// last output packet; later trials are not consumed.
// ===========================================================================
namespace {

enum RejKind { RK_GAMMA_GS = 0, RK_GAMMA_TAN = 1, RK_BETA_SMALL = 2, RK_POISSON = 3, RK_BINOMIAL = 4 };

constexpr int kRejThreads = 160;
constexpr int kMaxTrials = 320;  // trials resolved per block of packets (<= 2496 / 8 + 1)
constexpr int kMaxCand = 1280;   // candidate lanes per block: <= 2496 words / Wt * P + P
constexpr size_t kRejDynSmem = (size_t)(4 * kLanes * kN + kMaxCand) * sizeof(uint64_t);

// inclusive block scan of one uint32 per thread (kRejThreads threads)
__device__ __forceinline__ uint32_t block_incl_scan(uint32_t v, uint32_t* warp_tot) {
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
    for (int i = 0; i < kRejThreads / 32; ++i) {
      uint32_t t = warp_tot[i];
      warp_tot[i] = acc;
      acc += t;
    }
  }
  __syncthreads();
  return v + warp_tot[w];
}

}  // namespace

// Accept test of a double GS trial (GammaGen, alpha < 1, NormalExp.h:535-556)
// decided in float arithmetic where the float result lies clearly on one side
// of both comparisons: 1 accept, 0 reject, -1 undecided (evaluate in double).
// Bounds: vx converts with relative error < 2^-19 (vx >= 2^-12 here), ux2
// with absolute error < 2^-24, float log / exp are within 1 ulp and
// |log vx| <= 8.4, so the float qx is within 1e-5 (1 + 1/alpha) of the double
// qx, relatively (qx >= 0.027); the band used is 2^-18 (1 + 40/alpha), over
// 14 times wider.  The branch test ux < px is trusted outside
// |ux - px| <= 2^-21 (float ux is within 2^-24 of ux).
__device__ __forceinline__ int gs_filter_f64(uint64_t bux, uint64_t bvx, uint64_t bux2, float pxf, float inv_a,
                                             float am1, float band) {
  constexpr uint64_t M = 0xfffffffffffffull;
  // top 32 of the 52 fraction bits (absolute error < 2^-32); vx below 2^-12
  // is left to the double test, so vx keeps a relative error below 2^-19
  const float ux = __uint2float_rn((uint32_t)((bux & M) >> 20)) * 0x1p-32f;
  if (fabsf(ux - pxf) <= 0x1p-21f) return -1;
  const uint64_t mv = bvx & M;
  if ((mv >> 40) == 0) return -1;
  const float vx = __uint2float_rn((uint32_t)(mv >> 20)) * 0x1p-32f;
  const float ux2 = __uint2float_rn((uint32_t)((bux2 & M) >> 20)) * 0x1p-32f;
  const float lv = logf_(vx);
  const bool c = ux < pxf;
  const float e1 = expf_(c ? inv_a * lv : logf_(1.0f - lv) * am1);  // one exp for both branches
  const float qx = c ? expf_(-e1) : e1;
  if (ux2 < qx * (1.0f - band)) return 1;
  if (ux2 > qx * (1.0f + band)) return 0;
  return -1;
}

// Candidate of a double GS trial already known to be accepted: xx only
// (no acceptance bound); ux < px is decided on the integer fraction against
// tpx = ceil(px * 2^52).
__device__ __forceinline__ double gs_value_f64(uint64_t bux, uint64_t bvx, uint64_t tpx, double inv_a) {
  const double vx = ur_d(bvx) + 2.220446049250313e-16 / 8;
  const double lv = log_(vx);
  return ((bux & 0xfffffffffffffull) < tpx) ? exp_(inv_a * lv) : 1.0 - lv;
}

// One rejection trial, lane j: candidate bits and accept flag.  Trial t
// reads words [t * Wt, (t + 1) * Wt) of the cache-inclusive word stream
// (word(w)); full-packet double kinds read u64 lane values (rval(r)).
template <int RK, int DT, class WF, class RF>
__device__ __forceinline__ bool rej_trial(const DistParams& d, int64_t t, int j, WF&& word, RF&& rval,
                                          uint64_t& cbits) {
  constexpr int Wt = (RK == RK_GAMMA_GS) ? 3 * 8 : (RK == RK_POISSON || RK == RK_BINOMIAL) ? 8 : 2 * 8;
  bool acc = false;
  cbits = 0;

  const int64_t w0 = t * Wt;
  if (DT == SD_F32) {
    if (RK == RK_GAMMA_GS) {
      const float ux = ur_f(word(w0 + j));
      const float vx = ur_f(word(w0 + 8 + j)) + 1.1920928955078125e-07f / 8;
      const float ux2 = ur_f(word(w0 + 16 + j));
      // the reference evaluates both branches and blends (NormalExp.h:543-553);
      // evaluating only the selected one gives the same bits
      // branch c: xx = exp(lv / alpha), bound exp(-xx); else xx = 1 - lv,
      // bound exp(log(xx) (alpha - 1)).  One exp serves both branches, so a
      // warp with lanes in both runs three transcendentals after lv, not four
      const float lv = logf_(vx);
      const bool c = ux < d.fe;  // px
      const float e1 = expf_(c ? d.fc * lv : logf_(1.0f - lv) * d.fd);  // 1/alpha, alpha - 1
      const float xx = c ? e1 : 1.0f - lv;
      const float qx = c ? expf_(-e1) : e1;
      cbits = f2u(d.fb * xx);
      acc = ux2 < qx;
    } else if (RK == RK_GAMMA_TAN) {
      const float u = ur_f(word(w0 + j));
      const float ux = ur_f(word(w0 + 8 + j));
      float ys, yc;
      sincosf_((float)3.1415926535897932 * u, ys, yc);
      const float yx = ys / yc;
      const float xx = d.ff * yx + d.fd;  // sqrt * yx + (alpha - 1)
      const bool c = 0.0f < xx;
      const float ub = (yx * yx + 1.0f) * expf_(d.fd * logf_(xx / d.fd) - yx * d.ff);
      acc = c && (ux <= ub);
      cbits = f2u(d.fb * xx);
    } else if (RK == RK_BETA_SMALL) {
      const float u1 = ur_f(word(w0 + j));
      const float u2 = ur_f(word(w0 + 8 + j));
      const float p1 = expf_(logf_(u1) * d.fc);  // 1/a
      const float p2 = expf_(logf_(u2) * d.fd);  // 1/b
      const float x = p1 + p2;
      cbits = f2u(p1 / x);
      acc = x <= 1.0f;
    }
  } else if (DT == SD_F64) {
    const int64_t r0 = (t * Wt / 8) * 4 + j;  // u64 lane index of the trial's first packet
    if (RK == RK_GAMMA_GS) {
      // float filter first: rejected lanes need nothing more, accepted ones
      // only the candidate (the exact branch is known)
      const int f = gs_filter_f64(rval(r0), rval(r0 + 4), rval(r0 + 8), d.fe, d.fc, d.fd, d.fh);
      if (f == 0) {
        acc = false;
      } else if (f == 1) {
        cbits = d2u(d.db * gs_value_f64(rval(r0), rval(r0 + 4), d2u(d.dg), d.dc));  // dg holds tpx as bits
        acc = true;
      } else {
        const double ux = ur_d(rval(r0));
        const double vx = ur_d(rval(r0 + 4)) + 2.220446049250313e-16 / 8;
        const double ux2 = ur_d(rval(r0 + 8));
        const double lv = log_(vx);
        const bool c = ux < d.de;
        double xx, qx;
        if (c) {
          xx = exp_(d.dc * lv);
          qx = exp_(-xx);
        } else {
          xx = 1.0 - lv;
          qx = exp_(log_(xx) * d.dd);
        }
        cbits = d2u(d.db * xx);
        acc = ux2 < qx;
      }
    } else if (RK == RK_GAMMA_TAN) {
      const double u = ur_d(rval(r0));
      const double ux = ur_d(rval(r0 + 4));
      double ys, yc;
      sincos_(3.1415926535897932 * u, ys, yc);
      const double yx = ys / yc;
      const double xx = d.df * yx + d.dd;
      const bool c = 0.0 < xx;
      const double ub = (yx * yx + 1.0) * exp_(d.dd * log_(xx / d.dd) - yx * d.df);
      acc = c && (ux <= ub);
      cbits = d2u(d.db * xx);
    } else if (RK == RK_BETA_SMALL) {
      const double u1 = ur_d(rval(r0));
      const double u2 = ur_d(rval(r0 + 4));
      const double p1 = exp_(log_(u1) * d.dc);
      const double p2 = exp_(log_(u2) * d.dd);
      const double x = p1 + p2;
      cbits = d2u(p1 / x);
      acc = x <= 1.0;
    }
  } else {  // int32 kinds with Packet4f internals over half packets
    const float u = ur_f(word(w0 + j));
    const float u2 = ur_f(word(w0 + 4 + j));
    float s, c;
    sincosf_((float)3.1415926535897932 * u, s, c);
    const float yx = s / c;
    if (RK == RK_POISSON) {
      const float fres = truncf(d.fa * yx + d.fb);  // sqrt(2 mean) * yx + mean
      const float p1 = (yx * yx + 1.0f) * 0.9f;
      const float p2 = expf_((fres * d.fc - lgamma_approxf_(fres + 1.0f)) - d.fd);
      acc = (0.0f <= fres) && (u2 <= p1 * p2);
      cbits = f2u(fres);
    } else {  // binomial, BinomialGen::packetOp tan branch (Discrete.h:1014-1046)
      const float fres = truncf(d.fa * yx + d.fb);  // sqrt_v * ys + mean
      const float p1 = ((float)1.2 * d.fa) * (1.0f + yx * yx);
      float tt = (d.fg - lgamma_approxf_(fres + 1.0f)) - lgamma_approxf_((d.fh + 1.0f) - fres);
      tt = tt + fres * d.fc;
      tt = tt + (d.fh - fres) * d.fd;
      const float p2 = expf_(tt);
      acc = (0.0f <= fres) && (fres <= d.fh) && (u2 <= p1 * p2);
      cbits = f2u(fres);
    }
  }
        return acc;
}

// GammaGen's rejection trials drawn with a scalar engine (std::mt19937_64,
// P8_mt19937_64) as the Urng: trial t's candidate lanes from pre-drawn 64-bit
// words, a rejected lane written as NaN (accepted gamma candidates are never
// NaN), for TruncGen's CompressMask filter with an unbounded support.  A float
// uniform packet is RawbitsMaker<Packet8i, Rng, uint64_t, scalar_fullbit>::
// rawbits_34 of three draws (arch/AVX/RandUtils.h:59-144: lanes c.lo, c.hi,
// b.lo, top bytes, b.hi, a.lo, a.hi, top bytes, a the first draw); a double
// packet is rawbits, four draws in order.
template <int RK, int DT>
__global__ void __launch_bounds__(256) k_sx_cand(const uint64_t* w, int64_t M, DistParams d, void* cand) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  const int64_t g = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (g >= M * P) return;
  const int64_t t = g / P;
  const int j = (int)(g % P);
  auto word = [&](int64_t wi) -> uint32_t {
    const uint64_t* q = w + 3 * (wi >> 3);
    const uint32_t v[6] = {(uint32_t)q[2], (uint32_t)(q[2] >> 32), (uint32_t)q[1], (uint32_t)(q[1] >> 32),
                           (uint32_t)q[0], (uint32_t)(q[0] >> 32)};
    switch (wi & 7) {
      case 0: return v[0];
      case 1: return v[1];
      case 2: return v[2];
      case 3: return (v[0] >> 24) | ((v[1] >> 24) << 8) | ((v[2] >> 24) << 16) | ((v[2] >> 24) << 24);
      case 4: return v[3];
      case 5: return v[4];
      case 6: return v[5];
      default: return (v[3] >> 24) | ((v[4] >> 24) << 8) | ((v[5] >> 24) << 16) | ((v[5] >> 24) << 24);
    }
  };
  auto rval = [&](int64_t r) -> uint64_t { return w[r]; };
  uint64_t cb;
  const bool acc = rej_trial<RK, DT>(d, t, j, word, rval, cb);
  if (DT == SD_F32)
    static_cast<uint32_t*>(cand)[g] = acc ? (uint32_t)cb : 0x7fc00000u;
  else
    static_cast<uint64_t*>(cand)[g] = acc ? cb : 0x7ff8000000000000ull;
}

cudaError_t launch_sx_cand(int rk, int dtype, const uint64_t* w, int64_t M, const DistParams& d, void* cand,
                           cudaStream_t s) {
  const int P = dtype == GR_F32 ? 8 : 4;
  const unsigned blocks = (unsigned)((M * P + 255) / 256);
  if (dtype == GR_F32 && rk == RK_GAMMA_GS) k_sx_cand<RK_GAMMA_GS, SD_F32><<<blocks, 256, 0, s>>>(w, M, d, cand);
  else if (dtype == GR_F32 && rk == RK_GAMMA_TAN) k_sx_cand<RK_GAMMA_TAN, SD_F32><<<blocks, 256, 0, s>>>(w, M, d, cand);
  else if (dtype == GR_F64 && rk == RK_GAMMA_GS) k_sx_cand<RK_GAMMA_GS, SD_F64><<<blocks, 256, 0, s>>>(w, M, d, cand);
  else if (dtype == GR_F64 && rk == RK_GAMMA_TAN) k_sx_cand<RK_GAMMA_TAN, SD_F64><<<blocks, 256, 0, s>>>(w, M, d, cand);
  else return cudaErrorNotSupported;
  return cudaGetLastError();
}

// BetaGen / FisherFGen drawn with a scalar engine (std::mt19937_64,
// P8_mt19937_64) as the Urng, a fresh generator (the free functions;
// NormalExp.h:949-976, 1016-1021).  The draws are a chain: in the general
// branch every output packet is GammaGen(a)'s packetOp then GammaGen(b)'s,
// each a CompressMask loop with its own carried lanes when it rejects, so
// one warp walks it over a chunk of pre-drawn 64-bit words, lane j computing
// packet lane j with the same per-lane expressions as the packet engine's
// kernels (rej_trial; the exponential for alpha = 1; the product of alpha
// uniforms for an integral alpha < 20).  The a, b < 1 branch is the beta's
// own CompressMask loop over pairs of uniform packets; its mask is carried
// explicitly (an accepted lane may be 0/0).  A float uniform packet is three
// draws (rawbits_34), a double packet four.  The carried lanes are
// snapshotted at every completed output packet: the launch reports the
// packets it completed and the draws they used, and leaves the carried
// lanes as of that point, so the next chunk continues exactly there.
template <int DT>
__global__ void __launch_bounds__(32) k_sx_beta(const uint64_t* w, int64_t W, SxBetaArgs a) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  constexpr int64_t DPK = DT == SD_F32 ? 3 : 4;  // draws per uniform packet
  constexpr unsigned kFull = (1u << P) - 1u;
  const int lane = threadIdx.x;
  __shared__ uint64_t cache[3][2 * P], snap[3][2 * P];
  __shared__ int s_cnt[3], s_snap[3];
  for (int c = 0; c < 3; ++c) {
    if (lane < 2 * P) cache[c][lane] = snap[c][lane] = a.carry[c * 2 * P + lane];
    if (lane == 0) s_cnt[c] = s_snap[c] = a.cnt[c];
  }
  __syncwarp();
  int64_t pos = 0, used = 0, done = 0;  // draws consumed; by completed packets; packets completed

  // lane wi & 7 of float uniform packet wi >> 3 at draw offset pos (rawbits_34
  // of three draws a, b, c: c.lo, c.hi, b.lo, top bytes, b.hi, a.lo, a.hi, top bytes)
  auto word = [&](int64_t wi) -> uint32_t {
    const uint64_t* q = w + pos + 3 * (wi >> 3);
    const uint32_t v[6] = {(uint32_t)q[2], (uint32_t)(q[2] >> 32), (uint32_t)q[1], (uint32_t)(q[1] >> 32),
                           (uint32_t)q[0], (uint32_t)(q[0] >> 32)};
    switch (wi & 7) {
      case 0: return v[0];
      case 1: return v[1];
      case 2: return v[2];
      case 3: return (v[0] >> 24) | ((v[1] >> 24) << 8) | ((v[2] >> 24) << 16) | ((v[2] >> 24) << 24);
      case 4: return v[3];
      case 5: return v[4];
      case 6: return v[5];
      default: return (v[3] >> 24) | ((v[4] >> 24) << 8) | ((v[5] >> 24) << 16) | ((v[5] >> 24) << 24);
    }
  };
  // lane r & 3 of double uniform packet r >> 2 at draw offset pos (rawbits: four draws in order)
  auto rval = [&](int64_t r) -> uint64_t { return w[pos + r]; };

  // CompressMask::compress_append over lanes 0 .. P-1 into carried set c
  // (arch/AVX/PacketFilter.h:147-184): a full packet is returned as it is;
  // otherwise the accepted lanes join the carried ones and the first P leave
  auto compress = [&](int c, uint64_t bits, bool acc, uint64_t& res) -> bool {
    const unsigned m = __ballot_sync(0xffffffffu, acc && lane < P) & kFull;
    if (m == kFull) {
      res = bits;
      return true;
    }
    int fc = s_cnt[c];
    if (lane < P && ((m >> lane) & 1u)) cache[c][fc + __popc(m & ((1u << lane) - 1u))] = bits;
    fc += __popc(m);
    __syncwarp();
    if (fc < P) {
      if (lane == 0) s_cnt[c] = fc;
      __syncwarp();
      return false;
    }
    res = lane < P ? cache[c][lane] : 0;
    const uint64_t mv = lane < fc - P ? cache[c][P + lane] : 0;
    __syncwarp();
    if (lane < fc - P) cache[c][lane] = mv;
    if (lane == 0) s_cnt[c] = fc - P;
    __syncwarp();
    return true;
  };

  // GammaGen(alpha)'s packetOp for component c (0: a, 1: b); false when the
  // chunk runs out first
  auto gamma_packet = [&](int c, uint64_t& v) -> bool {
    const DistParams& g = a.g[c];
    if (g.ic) {  // alpha < 1: GS rejection, three uniform packets per trial
      for (;;) {
        if (pos + 3 * DPK > W) return false;
        uint64_t cb = 0;
        const bool acc = lane < P && rej_trial<RK_GAMMA_GS, DT>(g, 0, lane, word, rval, cb);
        pos += 3 * DPK;
        if (compress(c, cb, acc, v)) return true;
      }
    }
    if (g.ia) {  // alpha == 1: beta * ExponentialGen
      if (pos + DPK > W) return false;
      if (lane < P) {
        if (DT == SD_F32) {
          v = f2u(g.fb * (-(logf_(1.0f - ur_f(word(lane))) / 1.0f)));
        } else {
          const double l = -(log_(one_minus_ur_d(rval(lane))) / 1.0);
          v = d2u((g.flags & kParamUnitScale) ? l : g.db * l);
        }
      }
      pos += DPK;
      return true;
    }
    if (g.ib >= 2) {  // integral alpha < 20: product of alpha nonzero uniforms
      if (pos + g.ib * DPK > W) return false;
      if (lane < P) {
        if (DT == SD_F32) {
          float y = ur_f(word(lane)) + 1.1920928955078125e-07f / 8;
          for (int t = 1; t < g.ib; ++t) y = y * (ur_f(word(8 * t + lane)) + 1.1920928955078125e-07f / 8);
          v = f2u(-(g.fb * logf_(y)));
        } else {
          double y = ur_d(rval(lane)) + 2.220446049250313e-16 / 8;
          for (int t = 1; t < g.ib; ++t) y = y * (ur_d(rval(4 * t + lane)) + 2.220446049250313e-16 / 8);
          const double l = log_(y);
          v = d2u((g.flags & kParamUnitScale) ? -l : -(g.db * l));
        }
      }
      pos += g.ib * DPK;
      return true;
    }
    for (;;) {  // the tan proposal, two uniform packets per trial
      if (pos + 2 * DPK > W) return false;
      uint64_t cb = 0;
      const bool acc = lane < P && rej_trial<RK_GAMMA_TAN, DT>(g, 0, lane, word, rval, cb);
      pos += 2 * DPK;
      if (compress(c, cb, acc, v)) return true;
    }
  };

  while (done < a.npk) {
    uint64_t v = 0;
    bool ok = true;
    if (a.beta.ic) {  // a < 1 and b < 1: the beta's own rejection loop
      for (;;) {
        if (pos + 2 * DPK > W) {
          ok = false;
          break;
        }
        uint64_t cb = 0;
        const bool acc = lane < P && rej_trial<RK_BETA_SMALL, DT>(a.beta, 0, lane, word, rval, cb);
        pos += 2 * DPK;
        if (compress(2, cb, acc, v)) break;
      }
    } else {
      uint64_t p1 = 0, p2 = 0;
      ok = gamma_packet(0, p1) && gamma_packet(1, p2);
      if (ok) {
        if (DT == SD_F32) v = f2u(u2f((uint32_t)p1) / (u2f((uint32_t)p1) + u2f((uint32_t)p2)));
        else v = d2u(u2d(p1) / (u2d(p1) + u2d(p2)));
      }
    }
    if (!ok) break;
    v = beta_post<DT == SD_F64>(v, a.beta);
    if (lane < P) {
      if (DT == SD_F32) static_cast<uint32_t*>(a.out)[done * P + lane] = (uint32_t)v;
      else static_cast<uint64_t*>(a.out)[done * P + lane] = v;
    }
    ++done;
    used = pos;
    for (int c = 0; c < 3; ++c) {
      if (lane < 2 * P) snap[c][lane] = cache[c][lane];
      if (lane == 0) s_snap[c] = s_cnt[c];
    }
    __syncwarp();
  }
  // the carried lanes as of the last completed packet
  for (int c = 0; c < 3; ++c) {
    if (lane < 2 * P) a.carry[c * 2 * P + lane] = snap[c][lane];
    if (lane == 0) a.cnt[c] = s_snap[c];
  }
  if (lane == 0) {
    a.res[0] = done;
    a.res[1] = used;
  }
}

cudaError_t launch_sx_beta(const uint64_t* w, int64_t W, const SxBetaArgs& a, int dtype, cudaStream_t s) {
  if (dtype == GR_F32) k_sx_beta<SD_F32><<<1, 32, 0, s>>>(w, W, a);
  else k_sx_beta<SD_F64><<<1, 32, 0, s>>>(w, W, a);
  return cudaGetLastError();
}

template <int RK, int DT>  // DT: SD_F32 (P=8), SD_F64 (P=4), SD_I32H (P=4, float internals)
__global__ void __maxnreg__(64) k_reject(Plan p, DistParams d, int64_t max_blocks) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  constexpr bool kWide = DT == SD_F64;  // candidates are 64-bit
  constexpr int Wt = (RK == RK_GAMMA_GS) ? 3 * 8 : (RK == RK_POISSON || RK == RK_BINOMIAL) ? 8 : 2 * 8;
  extern __shared__ __align__(16) uint64_t rej_dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(rej_dyn);
  uint64_t(*tp)[kN][kLanes] = reinterpret_cast<uint64_t(*)[kN][kLanes]>(rej_dyn + 2 * kLanes * kN);
  uint64_t* cand = rej_dyn + 4 * kLanes * kN;  // candidate bits per (trial, lane), kMaxCand
  __shared__ uint32_t tmask[kMaxTrials];
  __shared__ uint32_t tscan[kMaxTrials];      // exclusive: (fulls << 16) | lanes appended
  __shared__ uint64_t fifo[2][16];            // carried lanes (ping-pong)
  __shared__ int64_t emit_of_q[kMaxTrials + 2];
  __shared__ uint32_t warp_tot[kRejThreads / 32];
  __shared__ int s_tstar;
  __shared__ int s_done;

  const int k = blockIdx.x;
  const int tid = threadIdx.x;
  EngState* st = p.eng + k;
  GenSlot* gs = &p.gen[k].s[0];

  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  const int64_t Npk = n / P;  // packets of output to produce

  constexpr bool kHalf = DT == SD_I32H;
  const int c0w = (kHalf && st->half_valid) ? 4 : 0;
  uint32_t cw[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) cw[q] = kHalf ? st->half_cache[q] : 0u;
  int rcnt = gs->rest_cnt;  // carried lanes
  if (tid < 16) fifo[0][tid] = kWide ? ((uint64_t)gs->rest[2 * (tid & 7)] | ((uint64_t)gs->rest[2 * (tid & 7) + 1] << 32))
                                     : (uint64_t)gs->rest[tid];
  load_window(raw[0], &st->win[0][0], kN);
  if (tid == 0) s_done = 0;
  __syncthreads();

  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t wq) -> uint32_t {
    if (wq < c0w) return cw[wq];
    const int64_t w = wq - c0w;
    const int64_t rel = w >> 3;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  // int32 result: BinomialGen returns trials - res when p > 1/2 (Discrete.h:1051)
  auto iout = [&](uint32_t fbits) -> int32_t {
    const int32_t r = (int32_t)u2f(fbits);
    return (RK == RK_BINOMIAL && d.ib) ? (int32_t)d.fh - r : r;
  };
  auto rval = [&](int64_t r) -> uint64_t {  // u64 lane value (full-packet f64 kinds)
    const int64_t rel = r >> 2;
    return ring_packet(tp, rel, ring_new, ring_slot)[r & 3];
  };

  int64_t E = 0;        // output packets emitted so far
  int64_t t_next = 0;   // next trial
  int cur = 0, fsl = 0;
  int64_t nb = 0;
  int64_t end_word = -1;  // words consumed (cache-inclusive), set when done
  for (; nb < max_blocks; ++nb) {
    const int slot = (int)(nb & 1);
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
    });
    cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    const int64_t avail_words = (nb + 1) * kN * 8 + c0w;
    int64_t t_end = avail_words / Wt;  // trials whose words all exist
    int B = (int)min((int64_t)kMaxTrials, t_end - t_next);
    if (B <= 0) continue;
    // ---- candidates and accept masks
    for (int base = 0; base < B * P; base += kRejThreads) {
      const int e = base + tid;
      const bool valid = e < B * P;
      const int tl = e / P, j = e % P;
      const int64_t t = t_next + tl;
      bool acc = false;
      uint64_t cbits = 0;
      if (valid) acc = rej_trial<RK, DT>(d, t, j, word, rval, cbits);
      const uint32_t bal = __ballot_sync(0xffffffffu, acc);
      if (valid) {
        cand[tl * P + j] = cbits;
        if (j == 0) tmask[tl] = (bal >> (threadIdx.x & 31 & ~(P - 1))) & ((1u << P) - 1);
      }
    }
    __syncthreads();
    // ---- prefix sums over trials: (fulls << 16) | appended lanes
    uint32_t v0 = 0, v1 = 0;
    const int ta = 2 * tid, tb = 2 * tid + 1;
    if (ta < B) {
      const int c = __popc(tmask[ta]);
      v0 = (c == P) ? (1u << 16) : (uint32_t)c;
    }
    if (tb < B) {
      const int c = __popc(tmask[tb]);
      v1 = (c == P) ? (1u << 16) : (uint32_t)c;
    }
    const uint32_t incl = block_incl_scan(v0 + v1, warp_tot);
    if (ta < B) tscan[ta] = incl - v0 - v1;
    if (tb < B) tscan[tb] = incl - v1;
    if (tid == 0) s_tstar = -1;
    __syncthreads();
    // ---- emissions of this batch; find the trial completing packet Npk-1
    for (int tl = tid; tl < B; tl += kRejThreads) {
      const uint32_t m = tmask[tl];
      const int c = __popc(m);
      const int64_t nf = tscan[tl] >> 16;
      const int64_t at = (int64_t)rcnt + (tscan[tl] & 0xffffu);
      const bool full = c == P;
      const bool cross = !full && ((at + c) / P > at / P);
      const int64_t eidx = E + nf + at / P;
      if (cross) emit_of_q[at / P] = eidx;
      if ((full || cross) && eidx == Npk - 1) s_tstar = tl;
    }
    __syncthreads();
    const int tstar = s_tstar;
    const int Bu = tstar >= 0 ? tstar + 1 : B;  // trials consumed in this batch
    // FIFO level after the consumed trials
    int64_t a_end;
    int64_t nf_end;
    {
      const int tl = Bu - 1;
      const int c = __popc(tmask[tl]);
      nf_end = (tscan[tl] >> 16) + (c == P ? 1 : 0);
      a_end = (int64_t)rcnt + (tscan[tl] & 0xffffu) + (c == P ? 0 : c);
    }
    const int64_t qe = a_end / P;  // FIFO packets emitted through the consumed trials
    // ---- write outputs
    for (int e = tid; e < Bu * P; e += kRejThreads) {
      const int tl = e / P, j = e % P;
      const uint32_t m = tmask[tl];
      const int c = __popc(m);
      const int64_t nf = tscan[tl] >> 16;
      const int64_t at = (int64_t)rcnt + (tscan[tl] & 0xffffu);
      uint64_t v = cand[tl * P + j];
      if (RK == RK_BETA_SMALL) v = beta_post<kWide>(v, d);
      if (c == P) {
        const int64_t eidx = E + nf + at / P;
        if (eidx < Npk) {
          if (kWide) reinterpret_cast<uint64_t*>(p.out)[off + eidx * P + j] = v;
          else if (DT == SD_I32H) reinterpret_cast<int32_t*>(p.out)[off + eidx * P + j] = iout((uint32_t)v);
          else reinterpret_cast<uint32_t*>(p.out)[off + eidx * P + j] = (uint32_t)v;
        }
      } else if ((m >> j) & 1u) {
        const int64_t f = at + __popc(m & ((1u << j) - 1));
        const int64_t q = f / P;
        if (q < qe) {
          const int64_t eidx = emit_of_q[q];
          if (eidx < Npk) {
            if (kWide) reinterpret_cast<uint64_t*>(p.out)[off + eidx * P + f % P] = v;
            else if (DT == SD_I32H) reinterpret_cast<int32_t*>(p.out)[off + eidx * P + f % P] = iout((uint32_t)v);
            else reinterpret_cast<uint32_t*>(p.out)[off + eidx * P + f % P] = (uint32_t)v;
          }
        } else {
          fifo[fsl ^ 1][f - qe * P] = cand[tl * P + j];  // the FIFO keeps beta draws
        }
      }
    }
    // carried lanes that were emitted in this batch's first FIFO packets
    if (tid < rcnt) {
      const int64_t f = tid;
      if (f / P < qe) {
        const int64_t eidx = emit_of_q[f / P];
        const uint64_t v = RK == RK_BETA_SMALL ? beta_post<kWide>(fifo[fsl][tid], d) : fifo[fsl][tid];
        if (eidx < Npk) {
          if (kWide) reinterpret_cast<uint64_t*>(p.out)[off + eidx * P + f % P] = v;
          else if (DT == SD_I32H) reinterpret_cast<int32_t*>(p.out)[off + eidx * P + f % P] = iout((uint32_t)v);
          else reinterpret_cast<uint32_t*>(p.out)[off + eidx * P + f % P] = (uint32_t)v;
        }
      } else {
        fifo[fsl ^ 1][f - qe * P] = fifo[fsl][tid];
      }
    }
    __syncthreads();
    E += nf_end + qe;
    rcnt = (int)(a_end - qe * P);
    fsl ^= 1;
    t_next += Bu;
    if (tstar >= 0) {
      end_word = t_next * Wt;
      break;
    }
  }

  // ---- engine and generator state after the call
  if (end_word < 0) {  // iteration cap: report, keep a consistent state
    if (tid == 0) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    end_word = t_next * Wt;
  }
  const int64_t w_pk = end_word - c0w;  // packet words consumed
  const int64_t np = (w_pk + 7) / 8;    // packets consumed
  if (np > 0) {
    // the call ends inside the last generated block (block nb): its trials are
    // the first whose words all exist, and every earlier trial was resolved
    // one block earlier
    const int64_t rr = np - nb * kN;
    if (rr >= 1 && rr <= kN) store_window(st, raw[cur], raw[cur ^ 1], (int)rr);
    else if (tid == 0) atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
  }
  if (tid == 0) {
    if (kHalf) {
      if ((w_pk & 7) == 4) {  // ends mid-packet: upper half cached
        const int64_t pl = np - 1;
        const int sl = (int)((pl / kN) & 1);
        const uint64_t a = tp[sl][pl % kN][2], b = tp[sl][pl % kN][3];
        st->half_cache[0] = (uint32_t)a;
        st->half_cache[1] = (uint32_t)(a >> 32);
        st->half_cache[2] = (uint32_t)b;
        st->half_cache[3] = (uint32_t)(b >> 32);
        st->half_valid = 1;
      } else {
        st->half_valid = 0;
      }
    }
    st->consumed += (uint64_t)max(np, (int64_t)0);
    gs->rest_cnt = rcnt;
  }
  if (tid < 16) {
    const uint64_t v = fifo[fsl][tid & 15];
    if (kWide) {
      if (tid < 8) {
        gs->rest[2 * tid] = (uint32_t)fifo[fsl][tid];
        gs->rest[2 * tid + 1] = (uint32_t)(fifo[fsl][tid] >> 32);
      }
    } else {
      gs->rest[tid] = (uint32_t)v;
    }
  }
}

template <int RK, int DT>
static cudaError_t run_reject(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s) {
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_reject<RK, DT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRejDynSmem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  k_reject<RK, DT><<<p.K, kRejThreads, kRejDynSmem, s>>>(p, d, max_blocks);
  return cudaGetLastError();
}

cudaError_t launch_reject(const Plan& p, const DistParams& d, int rk, int64_t max_blocks, cudaStream_t s) {
  const int dt = d.dtype == GR_F32 ? SD_F32 : d.dtype == GR_F64 ? SD_F64 : SD_I32H;
#define GR_RJ(R)                                                              \
  if (rk == R) {                                                               \
    if (dt == SD_F32) return run_reject<R, SD_F32>(p, d, max_blocks, s);       \
    if (dt == SD_F64) return run_reject<R, SD_F64>(p, d, max_blocks, s);       \
  }
  GR_RJ(RK_GAMMA_GS)
  GR_RJ(RK_GAMMA_TAN)
  GR_RJ(RK_BETA_SMALL)
#undef GR_RJ
  if (rk == RK_POISSON && dt == SD_I32H) return run_reject<RK_POISSON, SD_I32H>(p, d, max_blocks, s);
  if (rk == RK_BINOMIAL && dt == SD_I32H) return run_reject<RK_BINOMIAL, SD_I32H>(p, d, max_blocks, s);
  return cudaErrorNotSupported;
}

// ===========================================================================
// Segmented rejection for long calls on few engines.  The trial stream of a
// call is cut into S segments of Ts trials; segment s starts at packet s*J
// (J = Ts * packets per trial; half-packet kinds one packet earlier) from a
// jump-ahead window, so the segments run on separate SMs.
//   k_rs_count   per segment: fully accepted trials F and lanes of partially
//                accepted trials L.
//   k_rs_scan    per engine: prefix of (F, L) after the carried lanes, and
//                the segment s* whose trials complete the last output packet
//                (the last segment when the planned trials fall short: it
//                then runs on past its end, one CTA, until done).
//   k_rs_write   segments s <= s*: the automaton of k_reject from the
//                segment's starting (NF, A).  Full trials go straight to the
//                output; lanes of partial trials go to a lane buffer at their
//                FIFO position; the trial completing FIFO packet q records
//                its output index pos[q].  Segment s* stops at the trial that
//                completes the last packet and stores the engine state there.
//   k_rs_gather  FIFO packets to their output index (carried lanes from the
//                generator), then k_rs_finish carries the leftover lanes.
// The result is identical to k_reject's: the same trials, the same automaton.
// ===========================================================================
namespace {

template <int RK>
struct RejTraits {
  static constexpr int Wt = (RK == RK_GAMMA_GS) ? 3 * 8 : (RK == RK_POISSON || RK == RK_BINOMIAL) ? 8 : 2 * 8;
};

// Common per-CTA set-up of the segmented kernels.
template <int RK, int DT>
struct RsSeg {
  static constexpr int P = DT == SD_F32 ? 8 : 4;
  static constexpr bool kHalf = DT == SD_I32H;
  static constexpr int Wt = RejTraits<RK>::Wt;
  int k, s;
  int64_t off, Npk;
  int64_t seg_p0;  // first packet generated by this CTA
  int c0w;
  uint32_t cw[4];
  __device__ bool init(const Plan& p, const CallSnap* snap) {
    k = blockIdx.x / p.S;
    s = blockIdx.x % p.S;
    const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
    const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
    off = g0 * p.gran;
    Npk = ng * p.gran / P;
    c0w = (kHalf && snap[k].half_valid) ? 4 : 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) cw[q] = kHalf ? snap[k].half_cache[q] : 0u;
    seg_p0 = s == 0 ? 0 : (int64_t)s * p.J - (kHalf ? 1 : 0);
    return Npk > 0;
  }
};

__device__ __forceinline__ void rs_load_window(uint64_t (*raw)[kN], const Plan& p, int k, int s) {
  if (s == 0) load_window(raw, p.prefix + (size_t)k * kLanes * kPrefixLen, kPrefixLen);
  else load_window(raw, p.segwin + ((size_t)k * (p.S - 1) + (s - 1)) * kLanes * kN, kN);
}

}  // namespace

template <int RK, int DT>
__global__ void __launch_bounds__(kRejThreads) k_rs_count(Plan p, DistParams d, const CallSnap* snap, RsArgs a) {
  using G = RsSeg<RK, DT>;
  constexpr int P = G::P, Wt = G::Wt;
  extern __shared__ __align__(16) uint64_t rej_dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(rej_dyn);
  uint64_t(*tp)[kN][kLanes] = reinterpret_cast<uint64_t(*)[kN][kLanes]>(rej_dyn + 2 * kLanes * kN);
  __shared__ uint32_t tmask[kMaxTrials];
  __shared__ unsigned long long red[2];
  G g;
  if (!g.init(p, snap)) return;
  const int tid = threadIdx.x;
  rs_load_window(raw[0], p, g.k, g.s);
  if (tid < 2) red[tid] = 0;
  __syncthreads();
  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t wq) -> uint32_t {
    if (wq < g.c0w) return g.cw[wq];
    const int64_t w = wq - g.c0w;
    const int64_t rel = (w >> 3) - g.seg_p0;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  auto rval = [&](int64_t r) -> uint64_t {
    const int64_t rel = (r >> 2) - g.seg_p0;
    return ring_packet(tp, rel, ring_new, ring_slot)[r & 3];
  };
  const int64_t t_beg = (int64_t)g.s * a.Ts, t_end = t_beg + a.Ts;
  int64_t t_next = t_beg;
  uint64_t nfull = 0, nlanes = 0;
  int cur = 0;
  for (int64_t nb = 0; t_next < t_end; ++nb) {
    const int slot = (int)(nb & 1);
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
    });
    cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    const int64_t t_av = ((g.seg_p0 + (nb + 1) * kN) * 8 + g.c0w) / Wt;
    const int B = (int)(min(t_av, t_end) - t_next);
    if (B <= 0) continue;
    for (int base = 0; base < B * P; base += kRejThreads) {
      const int e = base + tid;
      const bool valid = e < B * P;
      const int tl = e / P, j = e % P;
      uint64_t cbits = 0;
      bool acc = false;
      if (valid) acc = rej_trial<RK, DT>(d, t_next + tl, j, word, rval, cbits);
      const uint32_t bal = __ballot_sync(0xffffffffu, acc);
      if (valid && j == 0) tmask[tl] = (bal >> (threadIdx.x & 31 & ~(P - 1))) & ((1u << P) - 1);
    }
    __syncthreads();
    for (int tl = tid; tl < B; tl += kRejThreads) {
      const int c = __popc(tmask[tl]);
      if (c == P) ++nfull;
      else nlanes += (uint64_t)c;
    }
    t_next += B;
    __syncthreads();
  }
  atomicAdd(&red[0], (unsigned long long)nfull);
  atomicAdd(&red[1], (unsigned long long)nlanes);
  __syncthreads();
  if (tid == 0) {
    a.cnt[((size_t)g.k * p.S + g.s) * 2] = (int64_t)red[0];
    a.cnt[((size_t)g.k * p.S + g.s) * 2 + 1] = (int64_t)red[1];
  }
}

template <int P>
__global__ void k_rs_scan(Plan p, RsArgs a) {
  const int k = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t Npk = ng * p.gran / P;
  int64_t NF = 0, A = p.gen[k].s[0].rest_cnt;
  int sstar = p.S - 1;
  for (int s = 0; s < p.S; ++s) {
    a.start[((size_t)k * p.S + s) * 2] = NF;
    a.start[((size_t)k * p.S + s) * 2 + 1] = A;
    NF += a.cnt[((size_t)k * p.S + s) * 2];
    A += a.cnt[((size_t)k * p.S + s) * 2 + 1];
    if (NF + A / P >= Npk) {
      sstar = s;
      break;
    }
  }
  a.fin[(size_t)k * 4] = Npk > 0 ? sstar : -1;
  a.fin[(size_t)k * 4 + 1] = 0;  // A and NF at the end, written by segment s*
  a.fin[(size_t)k * 4 + 2] = 0;
}

template <int RK, int DT>
__global__ void __launch_bounds__(kRejThreads) k_rs_write(Plan p, DistParams d, const CallSnap* snap, RsArgs a) {
  using G = RsSeg<RK, DT>;
  constexpr int P = G::P, Wt = G::Wt;
  constexpr bool kWide = DT == SD_F64;
  extern __shared__ __align__(16) uint64_t rej_dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(rej_dyn);
  uint64_t(*tp)[kN][kLanes] = reinterpret_cast<uint64_t(*)[kN][kLanes]>(rej_dyn + 2 * kLanes * kN);
  uint64_t* cand = rej_dyn + 4 * kLanes * kN;
  __shared__ uint32_t tmask[kMaxTrials];
  __shared__ uint32_t tscan[kMaxTrials];
  __shared__ uint32_t warp_tot[kRejThreads / 32];
  __shared__ int s_tstar;
  G g;
  if (!g.init(p, snap)) return;
  const int sstar = (int)a.fin[(size_t)g.k * 4];
  if (g.s > sstar) return;
  const int tid = threadIdx.x;
  EngState* st = p.eng + g.k;
  rs_load_window(raw[0], p, g.k, g.s);
  __syncthreads();
  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t wq) -> uint32_t {
    if (wq < g.c0w) return g.cw[wq];
    const int64_t w = wq - g.c0w;
    const int64_t rel = (w >> 3) - g.seg_p0;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  auto rval = [&](int64_t r) -> uint64_t {
    const int64_t rel = (r >> 2) - g.seg_p0;
    return ring_packet(tp, rel, ring_new, ring_slot)[r & 3];
  };
  auto iout = [&](uint32_t fbits) -> int32_t {
    const int32_t r = (int32_t)u2f(fbits);
    return (RK == RK_BINOMIAL && d.ib) ? (int32_t)d.fh - r : r;
  };
  auto put = [&](int64_t idx, uint64_t v) {
    if (RK == RK_BETA_SMALL) v = beta_post<kWide>(v, d);
    if (kWide) reinterpret_cast<uint64_t*>(p.out)[g.off + idx] = v;
    else if (DT == SD_I32H) reinterpret_cast<int32_t*>(p.out)[g.off + idx] = iout((uint32_t)v);
    else reinterpret_cast<uint32_t*>(p.out)[g.off + idx] = (uint32_t)v;
  };
  const bool last = g.s == sstar;
  const bool open = last && g.s == p.S - 1;  // may run past the planned trials
  const int64_t t_beg = (int64_t)g.s * a.Ts;
  const int64_t t_lim = open ? INT64_MAX : t_beg + a.Ts;
  // lane buffer of engine k: 64-bit lanes for double, 32-bit otherwise
  uint64_t* lanes64 = a.lanes + (size_t)g.k * a.lane_cap;
  uint32_t* lanes32 = reinterpret_cast<uint32_t*>(a.lanes) + (size_t)g.k * a.lane_cap;
  int64_t* pos = a.pos + (size_t)g.k * a.pos_cap;
  int64_t NF = a.start[((size_t)g.k * p.S + g.s) * 2];
  int64_t A = a.start[((size_t)g.k * p.S + g.s) * 2 + 1];
  int64_t t_next = t_beg;
  int cur = 0;
  int64_t nb = 0;
  bool stopped = false;
  const int64_t nb_cap = open ? a.max_blocks : INT64_MAX;
  for (; nb < nb_cap && t_next < t_lim; ++nb) {
    const int slot = (int)(nb & 1);
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
    });
    cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    const int64_t t_av = ((g.seg_p0 + (nb + 1) * kN) * 8 + g.c0w) / Wt;
    const int B = (int)(min(t_av, t_lim) - t_next);
    if (B <= 0) continue;
    for (int base = 0; base < B * P; base += kRejThreads) {
      const int e = base + tid;
      const bool valid = e < B * P;
      const int tl = e / P, j = e % P;
      uint64_t cbits = 0;
      bool acc = false;
      if (valid) acc = rej_trial<RK, DT>(d, t_next + tl, j, word, rval, cbits);
      const uint32_t bal = __ballot_sync(0xffffffffu, acc);
      if (valid) {
        cand[tl * P + j] = cbits;
        if (j == 0) tmask[tl] = (bal >> (threadIdx.x & 31 & ~(P - 1))) & ((1u << P) - 1);
      }
    }
    __syncthreads();
    uint32_t v0 = 0, v1 = 0;
    const int ta = 2 * tid, tb = 2 * tid + 1;
    if (ta < B) {
      const int c = __popc(tmask[ta]);
      v0 = (c == P) ? (1u << 16) : (uint32_t)c;
    }
    if (tb < B) {
      const int c = __popc(tmask[tb]);
      v1 = (c == P) ? (1u << 16) : (uint32_t)c;
    }
    const uint32_t incl = block_incl_scan(v0 + v1, warp_tot);
    if (ta < B) tscan[ta] = incl - v0 - v1;
    if (tb < B) tscan[tb] = incl - v1;
    if (tid == 0) s_tstar = -1;
    __syncthreads();
    if (last) {
      for (int tl = tid; tl < B; tl += kRejThreads) {
        const int c = __popc(tmask[tl]);
        const int64_t at = A + (tscan[tl] & 0xffffu);
        const bool full = c == P;
        const bool cross = !full && ((at + c) / P > at / P);
        const int64_t eidx = NF + (tscan[tl] >> 16) + at / P;
        if ((full || cross) && eidx == g.Npk - 1) s_tstar = tl;
      }
      __syncthreads();
    }
    const int tstar = s_tstar;
    const int Bu = tstar >= 0 ? tstar + 1 : B;
    for (int e = tid; e < Bu * P; e += kRejThreads) {
      const int tl = e / P, j = e % P;
      const uint32_t m = tmask[tl];
      const int c = __popc(m);
      const int64_t nf = NF + (tscan[tl] >> 16);
      const int64_t at = A + (tscan[tl] & 0xffffu);
      const uint64_t v = cand[tl * P + j];
      if (c == P) {
        const int64_t eidx = nf + at / P;
        if (eidx < g.Npk) put(eidx * P + j, v);
      } else {
        if ((m >> j) & 1u) {
          const int64_t f = at + __popc(m & ((1u << j) - 1));
          if (f < a.lane_cap) {
            if (kWide) lanes64[f] = v;
            else lanes32[f] = (uint32_t)v;
          }
          else atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
        }
        if (j == 0 && (at + c) / P > at / P) {  // this trial completes FIFO packet at / P
          const int64_t q = at / P;
          if (q < a.pos_cap) pos[q] = nf + q;
          else atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
        }
      }
    }
    {  // advance (NF, A) past the consumed trials
      const int tl = Bu - 1;
      const int c = __popc(tmask[tl]);
      NF += (tscan[tl] >> 16) + (c == P ? 1 : 0);
      A += (tscan[tl] & 0xffffu) + (c == P ? 0 : c);
    }
    t_next += Bu;
    __syncthreads();
    if (tstar >= 0) {
      stopped = true;
      break;
    }
  }
  if (!last) return;
  if (!stopped && tid == 0) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
  // engine state after the call: packets through the end of trial t_next - 1
  const int64_t w_pk = t_next * Wt - g.c0w;  // packet-stream words consumed
  const int64_t np = (w_pk + 7) / 8;
  const int64_t np_rel = np - g.seg_p0;  // generated by this CTA
  if (np_rel > 0) {
    const int64_t rr = np_rel - nb * kN;
    if (rr >= 1 && rr <= kN) store_window(st, raw[cur], raw[cur ^ 1], (int)rr);
    else if (tid == 0) atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
  }
  if (tid == 0) {
    if (G::kHalf) {
      if ((w_pk & 7) == 4) {
        const int64_t rel = np - 1 - g.seg_p0;
        const int sl = (int)((rel / kN) & 1);
        const uint64_t x = tp[sl][rel % kN][2], y = tp[sl][rel % kN][3];
        st->half_cache[0] = (uint32_t)x;
        st->half_cache[1] = (uint32_t)(x >> 32);
        st->half_cache[2] = (uint32_t)y;
        st->half_cache[3] = (uint32_t)(y >> 32);
        st->half_valid = 1;
      } else {
        st->half_valid = 0;
      }
    }
    st->consumed += (uint64_t)max(np, (int64_t)0);
    a.fin[(size_t)g.k * 4 + 1] = A;
    a.fin[(size_t)g.k * 4 + 2] = NF;
  }
}

// u64 value of carried lane f (the generator's rest, float or double lanes)
template <int DT>
__device__ __forceinline__ uint64_t rs_rest(const GenSlot* gs, int64_t f) {
  if (DT == SD_F64) return (uint64_t)gs->rest[2 * f] | ((uint64_t)gs->rest[2 * f + 1] << 32);
  return (uint64_t)gs->rest[f];
}

template <int DT>
__device__ __forceinline__ uint64_t rs_lane(const RsArgs& a, int k, int64_t f) {
  if (DT == SD_F64) return a.lanes[(size_t)k * a.lane_cap + f];
  return reinterpret_cast<const uint32_t*>(a.lanes)[(size_t)k * a.lane_cap + f];
}

template <int RK, int DT>
__global__ void k_rs_gather(Plan p, DistParams d, RsArgs a) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  const int k = blockIdx.y;
  if (a.fin[(size_t)k * 4] < 0) return;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, Npk = ng * p.gran / P;
  const int64_t Qend = min(a.fin[(size_t)k * 4 + 1] / P, min(a.pos_cap, a.lane_cap / P));
  const GenSlot* gs = &p.gen[k].s[0];
  const int64_t rc0 = gs->rest_cnt;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Qend * P; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = i / P, f = i;
    const int64_t eidx = a.pos[(size_t)k * a.pos_cap + q];
    if (eidx < 0 || eidx >= Npk) continue;
    uint64_t v = f < rc0 ? rs_rest<DT>(gs, f) : rs_lane<DT>(a, k, f);
    if (RK == RK_BETA_SMALL) v = beta_post<DT == SD_F64>(v, d);
    const int64_t o = off + eidx * P + (f - q * P);
    if (DT == SD_F64) {
      reinterpret_cast<uint64_t*>(p.out)[o] = v;
    } else if (DT == SD_I32H) {
      const int32_t r = (int32_t)u2f((uint32_t)v);
      reinterpret_cast<int32_t*>(p.out)[o] = (RK == RK_BINOMIAL && d.ib) ? (int32_t)d.fh - r : r;
    } else {
      reinterpret_cast<uint32_t*>(p.out)[o] = (uint32_t)v;
    }
  }
}

template <int DT>
__global__ void k_rs_finish(Plan p, RsArgs a) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  const int k = blockIdx.x;
  if (a.fin[(size_t)k * 4] < 0) return;
  GenSlot* gs = &p.gen[k].s[0];
  const int64_t Aend = min(a.fin[(size_t)k * 4 + 1], a.lane_cap);
  const int64_t q0 = (Aend / P) * P;
  const int64_t rc0 = gs->rest_cnt;
  const int l = threadIdx.x;  // 32 threads
  uint64_t v = 0;
  const int64_t f = q0 + l;
  if (l < P && f < Aend) v = f < rc0 ? rs_rest<DT>(gs, f) : rs_lane<DT>(a, k, f);
  __syncwarp();
  if (l < P && f < Aend) {
    if (DT == SD_F64) {
      gs->rest[2 * l] = (uint32_t)v;
      gs->rest[2 * l + 1] = (uint32_t)(v >> 32);
    } else {
      gs->rest[l] = (uint32_t)v;
    }
  }
  if (l == 0) gs->rest_cnt = (int32_t)(Aend - q0);
}

template <int RK, int DT>
static cudaError_t run_rs(const Plan& p, const DistParams& d, const CallSnap* snap, const RsArgs& a, int64_t gather_n,
                          cudaStream_t s) {
  constexpr int P = DT == SD_F32 ? 8 : 4;
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_rs_count<RK, DT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRejDynSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_rs_write<RK, DT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRejDynSmem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  k_rs_count<RK, DT><<<p.K * p.S, kRejThreads, kRejDynSmem, s>>>(p, d, snap, a);
  k_rs_scan<P><<<p.K, 32, 0, s>>>(p, a);
  k_rs_write<RK, DT><<<p.K * p.S, kRejThreads, kRejDynSmem, s>>>(p, d, snap, a);
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((gather_n + 255) / 256, 4096));
  k_rs_gather<RK, DT><<<dim3((unsigned)blocks, (unsigned)p.K), 256, 0, s>>>(p, d, a);
  k_rs_finish<DT><<<p.K, 32, 0, s>>>(p, a);
  return cudaGetLastError();
}

cudaError_t launch_reject_segmented(const Plan& p, const DistParams& d, int rk, const CallSnap* snap, const RsArgs& a,
                                    int64_t gather_n, cudaStream_t s) {
  const int dt = d.dtype == GR_F32 ? SD_F32 : d.dtype == GR_F64 ? SD_F64 : SD_I32H;
#define GR_RS(R)                                                           \
  if (rk == R) {                                                            \
    if (dt == SD_F32) return run_rs<R, SD_F32>(p, d, snap, a, gather_n, s); \
    if (dt == SD_F64) return run_rs<R, SD_F64>(p, d, snap, a, gather_n, s); \
  }
  GR_RS(RK_GAMMA_GS)
  GR_RS(RK_GAMMA_TAN)
  GR_RS(RK_BETA_SMALL)
#undef GR_RS
  if (rk == RK_POISSON && dt == SD_I32H) return run_rs<RK_POISSON, SD_I32H>(p, d, snap, a, gather_n, s);
  if (rk == RK_BINOMIAL && dt == SD_I32H) return run_rs<RK_BINOMIAL, SD_I32H>(p, d, snap, a, gather_n, s);
  return cudaErrorNotSupported;
}

}  // namespace gr

namespace gr {

// ===========================================================================
// k_poisson: PoissonGen with mean < 12 (Discrete.h:870-882), also BinomialGen
// with trials * min(p, 1-p) < 1 (its PoissonGen member).  One packetOp
// multiplies half packets of uniforms until every lane's product is
// <= exp(-mean) and returns, per lane, how many products stayed above it; the
// step from half packet s consumes L(s) half packets and the next starts at
// s + L(s).  Per block of 312 packets: the uniforms go to a float ring as the
// packets are made; every new start position gets its step (L and the four
// counts, packed in one word) in parallel; thread 0 follows s += L(s); all
// threads write the visited steps' counts.
// ===========================================================================
namespace {
constexpr int kPoisThreads = 160;
constexpr int kPoisLook = 64;    // half packets one step may read; a longer step is reported
constexpr int kPoisRing = 1024;  // start positions kept (>= 2 * 312 + kPoisLook)
constexpr int kPoisRec = 704;    // steps recorded per block (<= 624 + kPoisLook)
constexpr size_t kPoisSmem = (size_t)3 * kLanes * kN * 8 +  // raw x3
                             (size_t)2 * kN * 8 * 4 +       // uniforms of the two newest blocks
                             (size_t)kPoisRing * 4 +        // per position: L << 24 | counts (6 bits each)
                             (size_t)kPoisRec * 2;          // visited positions (ring index)
}  // namespace

__global__ void __launch_bounds__(kPoisThreads) k_poisson(Plan p, DistParams d, int64_t max_blocks) {
  extern __shared__ __align__(16) uint64_t pois_dyn[];
  // raw: three block buffers so the window before the end of the call is
  // still in shared memory when the call ends in the previous block
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(pois_dyn);
  float(*uf)[kN][8] = reinterpret_cast<float(*)[kN][8]>(pois_dyn + 3 * kLanes * kN);
  uint32_t* pos = reinterpret_cast<uint32_t*>(pois_dyn + 3 * kLanes * kN + kN * 8);
  uint16_t* rec = reinterpret_cast<uint16_t*>(pos + kPoisRing);
  __shared__ int s_nrec, s_stop, s_err;
  __shared__ int64_t s_ebase, s_end;
  __shared__ float4 s_cache;  // uniforms of the engine's cached half packet
  const int k = blockIdx.x;
  const int tid = threadIdx.x;
  EngState* st = p.eng + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  const int64_t Npk = n / 4;
  const int c0w = st->half_valid ? 4 : 0;  // the first half packet comes from the engine's cache
  load_window(raw[0], &st->win[0][0], kN);
  if (tid == 0) {
    s_err = 0;
    s_stop = 0;
    s_cache = make_float4(ur_f(st->half_cache[0]), ur_f(st->half_cache[1]), ur_f(st->half_cache[2]),
                          ur_f(st->half_cache[3]));
  }
  __syncthreads();
  int64_t s = 0, E = 0, done_pos = 0;  // walk (thread 0); positions evaluated up to done_pos
  int cur = 0;
  int64_t nb = 0;
  for (; nb < max_blocks; ++nb) {
    const int slot = (int)(nb & 1);
    const int nxt = cur == 2 ? 0 : cur + 1;
    mt_block(raw[cur], raw[nxt], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) {
        uf[slot][i][2 * l] = ur_f((uint32_t)pk[l]);
        uf[slot][i][2 * l + 1] = ur_f((uint32_t)(pk[l] >> 32));
      }
    });
    cur = nxt;
    // positions whose whole step (<= kPoisLook half packets) exists
    const int64_t lim = c0w / 4 + 2 * (nb + 1) * kN - kPoisLook;
    if (tid == 0 && lim - s > kPoisRing) s_err = 1;
    // ---- steps of the new start positions
    for (int64_t x = done_pos + tid; x < lim; x += kPoisThreads) {
      // half packet x starts at packet-stream word 4x - c0w (negative: the
      // engine's cached half packet); w = offset from the newest block's first word
      const bool cached = 4 * x < c0w;
      int w = (int)(4 * x - c0w - 8 * nb * (int64_t)kN);
      float val[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      int kk[4] = {0, 0, 0, 0};
      int L = 0;
      bool any = true;
      for (int it = 0; it < kPoisLook && any; ++it, w += 4) {
        float4 u;
        if (it == 0 && cached) {
          u = s_cache;
        } else {
          int pk = w >> 3, sl = slot;
          if (pk < 0) {
            pk += kN;
            sl ^= 1;
          }
          u = *reinterpret_cast<const float4*>(&uf[sl][pk][w & 7]);
        }
        const float uu[4] = {u.x, u.y, u.z, u.w};
        any = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          val[j] = val[j] * uu[j];
          const bool c = d.fe < val[j];  // exp(-mean) < val
          kk[j] += c ? 1 : 0;
          any |= c;
        }
        L = it + 1;
      }
      if (any) atomicOr(&s_err, 1);
      pos[(int)(x & (kPoisRing - 1))] =
          ((uint32_t)L << 24) | (uint32_t)kk[0] | ((uint32_t)kk[1] << 6) | ((uint32_t)kk[2] << 12) | ((uint32_t)kk[3] << 18);
    }
    done_pos = max(done_pos, lim);
    __syncthreads();
    // ---- walk (thread 0)
    if (tid == 0) {
      s_ebase = E;
      int nrec = 0;
      while (s < done_pos && E < Npk && nrec < kPoisRec) {
        const int ri = (int)(s & (kPoisRing - 1));
        rec[nrec++] = (uint16_t)ri;
        s += pos[ri] >> 24;
        ++E;
      }
      s_nrec = nrec;
      if (E >= Npk) {
        s_stop = 1;
        s_end = s;
      }
    }
    __syncthreads();
    // ---- write the visited steps
    const int nrec = s_nrec;
    const int64_t e_first = s_ebase;
    for (int e = tid; e < nrec * 4; e += kPoisThreads) {
      const int i = e >> 2, j = e & 3;
      int32_t v = (int32_t)((pos[rec[i]] >> (6 * j)) & 63);
      if (d.ic) v = d.ia - v;  // BinomialGen: trials - res when p > 1/2
      reinterpret_cast<int32_t*>(p.out)[off + (e_first + i) * 4 + j] = v;
    }
    __syncthreads();
    if (s_stop || s_err) break;
  }
  // ---- state after the call
  if (tid == 0 && (!s_stop || s_err)) {
    if (!s_stop) s_end = s;
    atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
  }
  __syncthreads();
  const int64_t fresh = s_end - c0w / 4;  // half packets drawn fresh
  const int64_t np = (fresh + 1) / 2;     // packets consumed
  const int prv = cur == 0 ? 2 : cur - 1, prv2 = prv == 0 ? 2 : prv - 1;
  const int64_t nblk = min(nb + 1, max_blocks);  // blocks generated
  if (np > 0) {
    const int64_t lastb = (np - 1) / kN;
    const int64_t rr = np - lastb * kN;  // in [1, 312]
    if (lastb == nblk - 1) store_window(st, raw[cur], raw[prv], (int)rr);
    else if (lastb == nblk - 2) store_window(st, raw[prv], raw[prv2], (int)rr);
    else if (tid == 0) atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
  }
  if (tid == 0) {
    if (fresh & 1) {  // the last packet's upper half stays in the engine's half cache
      const int64_t pl = np - 1;
      const int buf = (pl / kN == nblk - 1) ? cur : prv;
      const uint64_t a = mt_temper(raw[buf][2][pl % kN]), b = mt_temper(raw[buf][3][pl % kN]);
      st->half_cache[0] = (uint32_t)a;
      st->half_cache[1] = (uint32_t)(a >> 32);
      st->half_cache[2] = (uint32_t)b;
      st->half_cache[3] = (uint32_t)(b >> 32);
      st->half_valid = 1;
    } else {
      st->half_valid = 0;
    }
    st->consumed += (uint64_t)max(np, (int64_t)0);
  }
}

static cudaError_t run_poisson(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s) {
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_poisson, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPoisSmem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  k_poisson<<<p.K, kPoisThreads, kPoisSmem, s>>>(p, d, max_blocks);
  return cudaGetLastError();
}

// ===========================================================================
// PoissonGen (mean < 12) and BinomialGen (mean < 1) on few engines over
// jump-ahead segments.  The steps x -> x + L(x) of one engine form a chain
// that a single CTA would have to follow from start to end; here segment s of
// engine k (fresh packets [sJ, (s+1)J)) runs on its own CTA, in three
// launches:
//   scan   follows a speculative chain from the segment's first position,
//          marking its step starts in a bitmap, and the chains from each of
//          the other kPwEntries - 1 positions where the true chain can enter
//          the segment (the previous segment's last step overshoots its end
//          by less than kPoisLook) until they meet the marked chain; records,
//          per entry offset, the steps the chain takes in the segment and the
//          offset at which it leaves it;
//   plan   (one CTA per engine) chains the entry offsets from segment to
//          segment and turns the step counts into output offsets;
//   write  follows its segment's true chain and writes its steps at their
//          offsets; the segment holding the call's last step leaves the
//          engine state, and an engine's last segment runs on past its end
//          when the planned segments hold too few steps.
// A step depends only on its start position, so two chains that meet share
// every later step: the outputs equal the single-CTA walk's, bit for bit.
// ===========================================================================
template <int MODE>  // 0 scan, 1 write
__global__ void __launch_bounds__(kPoisThreads) k_pw(Plan p, DistParams d, PwArgs a) {
  extern __shared__ __align__(16) uint64_t pois_dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(pois_dyn);
  float(*uf)[kN][8] = reinterpret_cast<float(*)[kN][8]>(pois_dyn + 3 * kLanes * kN);
  uint32_t* pos = reinterpret_cast<uint32_t*>(pois_dyn + 3 * kLanes * kN + kN * 8);
  uint16_t* rec = reinterpret_cast<uint16_t*>(pos + kPoisRing);
  __shared__ int s_nrec, s_stop, s_err, s_walkers, s_cnt0;
  __shared__ int64_t s_ebase, s_end, s_x0;
  __shared__ float4 s_cache;
  const int S = p.S;
  const int k = blockIdx.x / S, sg = blockIdx.x % S;
  const int tid = threadIdx.x;
  EngState* st = p.eng + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  const int64_t Npk = n / 4;
  const int c = a.snap[k].half_valid ? 1 : 0;  // position 0 is the engine's cached half packet
  const int c0w = 4 * c;
  const int64_t pk0 = (int64_t)sg * a.J;  // first fresh packet of the segment
  const int64_t seg_lo = sg == 0 ? 0 : 2 * pk0 + c;
  const int64_t seg_hi = 2 * (pk0 + a.J) + c;
  const bool lastseg = sg == S - 1;
  const size_t sidx = (size_t)k * S + sg;
  int64_t start = seg_lo, O = 0, nsteps = INT64_MAX;
  if (MODE == 1) {
    start = seg_lo + a.plan[sidx * 3 + 0];
    O = a.plan[sidx * 3 + 1];
    if (!lastseg) nsteps = a.plan[sidx * 3 + 2];
    if (O >= Npk) return;  // the call ends in an earlier segment
  }
  // lane windows: segment 0 from the call-start copy, the others from the jumps
  if (sg == 0) load_window(raw[0], p.prefix + (size_t)k * kLanes * kPrefixLen, kPrefixLen);
  else load_window(raw[0], p.segwin + ((size_t)k * (S - 1) + (sg - 1)) * kLanes * kN, kN);
  if (tid == 0) {
    s_err = 0;
    s_stop = 0;
    s_walkers = (MODE == 0 && sg > 0) ? kPwEntries - 1 : 0;
    const uint32_t* hc = a.snap[k].half_cache;
    s_cache = make_float4(ur_f(hc[0]), ur_f(hc[1]), ur_f(hc[2]), ur_f(hc[3]));
  }
  __syncthreads();
  uint32_t* bits = a.bits + sidx * (size_t)a.words_per_seg;
  const int64_t max_blocks = lastseg ? a.max_blocks : (2 * a.J + 4 * kPoisLook) / (2 * kN) + 3;
  // chain of thread 0 (the speculative chain, or the true one); scan-mode
  // walkers: thread t in [1, kPwEntries) follows the chain entering at seg_lo + t
  int64_t x0 = start, E = 0;
  int32_t cnt0 = 0;
  int64_t bw = -1;  // bitmap word held by thread 0
  uint32_t bv = 0;
  int64_t xt = seg_lo + tid, mt = 0;
  int32_t nt = 0;
  int wstate = (MODE == 0 && sg > 0 && tid >= 1 && tid < kPwEntries) ? 1 : 0;  // 1 active, 2 met, 3 left
  int64_t done_pos = start;
  int cur = 0;
  int64_t nb = 0;
  for (; nb < max_blocks; ++nb) {
    const int slot = (int)(nb & 1);
    const int nxt = cur == 2 ? 0 : cur + 1;
    mt_block(raw[cur], raw[nxt], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) {
        uf[slot][i][2 * l] = ur_f((uint32_t)pk[l]);
        uf[slot][i][2 * l + 1] = ur_f((uint32_t)(pk[l] >> 32));
      }
    });
    cur = nxt;
    const int64_t lim = c + 2 * pk0 + 2 * (nb + 1) * kN - kPoisLook;
    if (tid == 0 && lim - x0 > kPoisRing) s_err = 1;  // positions still needed would leave the ring
    // ---- steps of the new start positions (as in k_poisson)
    for (int64_t x = done_pos + tid; x < lim; x += kPoisThreads) {
      const bool cached = 4 * x < c0w;
      int w = (int)(4 * (x - c - 2 * pk0) - 8 * nb * (int64_t)kN);
      float val[4] = {1.0f, 1.0f, 1.0f, 1.0f};
      int kk[4] = {0, 0, 0, 0};
      int L = 0;
      bool any = true;
      for (int it = 0; it < kPoisLook && any; ++it, w += 4) {
        float4 u;
        if (it == 0 && cached) {
          u = s_cache;
        } else {
          int pkk = w >> 3, sl = slot;
          if (pkk < 0) {
            pkk += kN;
            sl ^= 1;
          }
          u = *reinterpret_cast<const float4*>(&uf[sl][pkk][w & 7]);
        }
        const float uu[4] = {u.x, u.y, u.z, u.w};
        any = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          val[j] = val[j] * uu[j];
          const bool cc = d.fe < val[j];
          kk[j] += cc ? 1 : 0;
          any |= cc;
        }
        L = it + 1;
      }
      if (any) atomicOr(&s_err, 1);
      pos[(int)(x & (kPoisRing - 1))] =
          ((uint32_t)L << 24) | (uint32_t)kk[0] | ((uint32_t)kk[1] << 6) | ((uint32_t)kk[2] << 12) | ((uint32_t)kk[3] << 18);
    }
    done_pos = max(done_pos, lim);
    __syncthreads();
    if (MODE == 0) {
      // ---- the speculative chain (thread 0), its step starts marked
      if (tid == 0) {
        while (x0 < done_pos && x0 < seg_hi) {
          const int64_t r = x0 - seg_lo;
          if ((r >> 5) != bw) {
            if (bw >= 0) bits[bw] = bv;
            for (int64_t q = bw + 1; q < (r >> 5); ++q) bits[q] = 0u;
            bw = r >> 5;
            bv = 0;
          }
          bv |= 1u << (r & 31);
          ++cnt0;
          x0 += pos[(int)(x0 & (kPoisRing - 1))] >> 24;
        }
        if (bw >= 0) bits[bw] = bv;
        s_x0 = x0;
        if (x0 >= seg_hi && s_walkers == 0) s_stop = 1;
      }
      __syncthreads();
      // ---- walkers: until they meet the marked chain or leave the segment
      if (wstate == 1) {
        const int64_t xs = s_x0;
        while (xt < done_pos) {
          if (xt >= seg_hi) {
            wstate = 3;
            break;
          }
          const int64_t r = xt - seg_lo;
          if (xt == xs || (xt < xs && ((bits[r >> 5] >> (r & 31)) & 1u))) {
            wstate = 2;
            mt = xt;
            break;
          }
          ++nt;
          xt += pos[(int)(xt & (kPoisRing - 1))] >> 24;
        }
        if (wstate != 1) atomicSub(&s_walkers, 1);
      }
      __syncthreads();
      if (tid == 0 && s_x0 >= seg_hi && s_walkers == 0) s_stop = 1;
      __syncthreads();
    } else {
      // ---- the true chain (thread 0), as k_poisson's walk
      if (tid == 0) {
        s_ebase = E;
        int nrec = 0;
        const int64_t want = min(nsteps, Npk - O);
        while (x0 < done_pos && E < want && nrec < kPoisRec) {
          const int ri = (int)(x0 & (kPoisRing - 1));
          rec[nrec++] = (uint16_t)ri;
          x0 += pos[ri] >> 24;
          ++E;
        }
        s_nrec = nrec;
        if (E >= want) {
          s_stop = (O + E >= Npk) ? 1 : 2;  // 1: the call ends here
          s_end = x0;
        }
      }
      __syncthreads();
      const int nrec = s_nrec;
      const int64_t e_first = O + s_ebase;
      for (int e = tid; e < nrec * 4; e += kPoisThreads) {
        const int i = e >> 2, j = e & 3;
        int32_t v = (int32_t)((pos[rec[i]] >> (6 * j)) & 63);
        if (d.ic) v = d.ia - v;  // BinomialGen: trials - res when p > 1/2
        reinterpret_cast<int32_t*>(p.out)[off + (e_first + i) * 4 + j] = v;
      }
      __syncthreads();
    }
    if (s_stop || s_err) break;
  }
  if (MODE == 0) {
    if (tid == 0 && (!s_stop || s_err)) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    const int64_t xs = s_x0;
    if (tid == 0) {
      s_cnt0 = cnt0;  // the chain's steps, for the walkers' counts below
      int32_t* info = a.info + sidx * 4;
      info[0] = (int32_t)(xs - seg_hi);
      info[1] = cnt0;
      info[2] = 1;  // every entry met the chain (cleared below otherwise)
      int32_t* en = a.ent + sidx * kPwEntries * 2;
      en[0] = cnt0;
      en[1] = (int32_t)(xs - seg_hi);
    }
    __syncthreads();
    if (wstate == 2) {
      // steps of the marked chain before the meeting point
      const int64_t r = mt - seg_lo;
      int32_t rank = 0;
      for (int64_t q = 0; q < (r >> 5); ++q) rank += __popc(bits[q]);
      rank += __popc(bits[r >> 5] & ((1u << (r & 31)) - 1u));
      int32_t* en = a.ent + (sidx * kPwEntries + tid) * 2;
      en[0] = nt + s_cnt0 - rank;
      en[1] = (int32_t)(xs - seg_hi);
    } else if (wstate == 3 || wstate == 1) {
      int32_t* en = a.ent + (sidx * kPwEntries + tid) * 2;
      en[0] = nt;
      en[1] = (int32_t)(xt - seg_hi);
      a.info[sidx * 4 + 2] = 0;
    }
    return;
  }
  // ---- write mode: the engine state, from the segment that ends the call
  if (tid == 0 && (s_stop == 0 || s_err)) {
    // an engine's last segment ran out of blocks, or a step was too long
    atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
  }
  __syncthreads();
  if (s_stop != 1) return;
  const int64_t fresh = s_end - c;    // half packets drawn fresh, from the call start
  const int64_t np = (fresh + 1) / 2;  // packets consumed
  const int64_t lp = np - pk0;          // ... of this segment's blocks
  const int prv = cur == 0 ? 2 : cur - 1, prv2 = prv == 0 ? 2 : prv - 1;
  const int64_t nblk = min(nb + 1, max_blocks);
  if (lp > 0) {
    const int64_t lastb = (lp - 1) / kN;
    const int64_t rr = lp - lastb * kN;
    if (lastb == nblk - 1) store_window(st, raw[cur], raw[prv], (int)rr);
    else if (lastb == nblk - 2) store_window(st, raw[prv], raw[prv2], (int)rr);
    else if (tid == 0) atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
  } else if (tid == 0) {
    atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
  }
  if (tid == 0) {
    if (fresh & 1) {  // the last packet's upper half stays in the engine's half cache
      const int64_t pl = lp - 1;
      const int buf = (pl / kN == nblk - 1) ? cur : prv;
      const uint64_t aa = mt_temper(raw[buf][2][pl % kN]), bb = mt_temper(raw[buf][3][pl % kN]);
      st->half_cache[0] = (uint32_t)aa;
      st->half_cache[1] = (uint32_t)(aa >> 32);
      st->half_cache[2] = (uint32_t)bb;
      st->half_cache[3] = (uint32_t)(bb >> 32);
      st->half_valid = 1;
    } else {
      st->half_valid = 0;
    }
    st->consumed += (uint64_t)max(np, (int64_t)0);
  }
}

// One CTA per engine: entry offsets chained from segment to segment, output
// offsets from the step counts.
__global__ void __launch_bounds__(1024) k_pw_plan(Plan p, PwArgs a) {
  __shared__ int32_t s_tot[32];
  __shared__ int64_t s_carry;
  const int S = p.S, k = blockIdx.x, tid = threadIdx.x;
  const size_t base = (size_t)k * S;
  // entry offsets: known where the previous segment's entries all met
  for (int sg = tid; sg < S; sg += blockDim.x) {
    int64_t dv = -1;
    if (sg == 0) dv = 0;
    else if (a.info[(base + sg - 1) * 4 + 2]) dv = a.info[(base + sg - 1) * 4 + 0];
    a.plan[(base + sg) * 3 + 0] = dv;
  }
  __syncthreads();
  if (tid == 0) {
    for (int sg = 1; sg < S; ++sg) {
      if (a.plan[(base + sg) * 3 + 0] >= 0) continue;
      const int64_t dp = a.plan[(base + sg - 1) * 3 + 0];
      a.plan[(base + sg) * 3 + 0] = a.ent[((base + sg - 1) * kPwEntries + dp) * 2 + 1];
    }
    s_carry = 0;
  }
  __syncthreads();
  // steps per segment, then their exclusive prefix sums
  for (int b0 = 0; b0 < S; b0 += blockDim.x) {
    const int sg = b0 + tid;
    int32_t v = 0;
    if (sg < S) {
      int64_t dv = a.plan[(base + sg) * 3 + 0];
      if (dv < 0 || dv >= kPwEntries) dv = 0;  // unreachable: offsets stay below kPoisLook
      v = a.ent[((base + sg) * kPwEntries + dv) * 2 + 0];
    }
    // block-wide inclusive scan of v
    int32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if ((tid & 31) >= o) x += y;
    }
    if ((tid & 31) == 31) s_tot[tid >> 5] = x;
    __syncthreads();
    if (tid < 32) {
      int32_t t = s_tot[tid];
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, t, o);
        if (tid >= o) t += y;
      }
      s_tot[tid] = t;
    }
    __syncthreads();
    const int64_t incl = s_carry + x + ((tid >> 5) ? s_tot[(tid >> 5) - 1] : 0);
    if (sg < S) {
      a.plan[(base + sg) * 3 + 1] = incl - v;
      a.plan[(base + sg) * 3 + 2] = v;
    }
    __syncthreads();
    if (tid == blockDim.x - 1) s_carry = incl;
    __syncthreads();
  }
}

cudaError_t launch_poisson_segmented(const Plan& p, const DistParams& d, const PwArgs& a, cudaStream_t s) {
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_pw<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPoisSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pw<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPoisSmem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  k_pw<0><<<p.K * p.S, kPoisThreads, kPoisSmem, s>>>(p, d, a);
  k_pw_plan<<<p.K, 1024, 0, s>>>(p, a);
  k_pw<1><<<p.K * p.S, kPoisThreads, kPoisSmem, s>>>(p, d, a);
  return cudaGetLastError();
}

// ===========================================================================
// k_beta: BetaGen with a >= 1 or b >= 1 (NormalExp.h:970-975).  Each output
// packet draws one packet from GammaGen(a), then one from GammaGen(b); a
// component is closed form (alpha == 1: 1 packet; integer alpha < 20: alpha
// packets) or a rejection sampler (GS trials of 3 packets, tan trials of 2)
// with its own CompressMask carry.
// The ring of packets is the newest three raw engine blocks in shared
// memory, tempered where read (no tempered copy), so four CTAs fit on an SM
// and all engines run in one wave.  Every start position of a rejection
// component gets its P-lane accept mask ahead of the walk; the walk over
// the masks and the value work run on separate warps (the kernel below).
// ===========================================================================
namespace {

constexpr int kBetaRing = 1024;  // positions whose accept masks are kept (a power of two)

template <int DT>
__host__ __device__ constexpr int beta_lanes() {
  return DT == SD_F64 ? 4 : 8;
}

// Constants of one GammaGen component of a BetaGen, computed on the host
// with the same IEEE expressions the generator uses (so with the same bits),
// and passed as a kernel parameter: in the sampling loops they cost a
// constant-bank load, never a division.
struct BetaComp {
  int type, U;                      // gamma_branch: type << 8 | packets
  float af, f_px, f_inv, f_am1, f_sq;
  float f_band;                     // band of the float pre-test of a double GS trial
  double ad, d_px, d_inv, d_am1, d_sq;
  uint64_t tpx;                     // ceil(px * 2^52): double GS branch on the integer fraction
};
struct BetaConsts {
  BetaComp c[2];
  int post;              // FisherFGen: write (b/a) x / (1 - x)
  float fpost;           // b/a in the scalar type
  double dpost;
};

BetaComp beta_component(int branch, float af, double ad) {
  BetaComp b;
  b.type = branch >> 8;
  b.U = branch & 0xff;
  b.af = af;
  b.f_px = (float)(2.7182818284590452 / ((double)af + 2.7182818284590452));
  b.f_inv = 1 / af;
  b.f_am1 = af - 1;
  b.f_sq = std::sqrt(2 * af - 1);
  b.f_band = (float)(0x1p-18 * (1.0 + 40.0 / ad));
  b.ad = ad;
  b.d_px = 2.7182818284590452 / (ad + 2.7182818284590452);
  b.d_inv = 1 / ad;
  b.d_am1 = ad - 1;
  b.d_sq = std::sqrt(2 * ad - 1);
  b.tpx = (uint64_t)std::ceil(b.d_px * 0x1p52);
  return b;
}

// Value (closed form) or candidate (rejection trial) of one GammaGen
// component of sampler type `type` at one lane: Uf(q) / Ud(q) give the
// lane's uniform in the q-th packet of the draw.  ACC: also decide
// acceptance (the rejection types); without it only the candidate is
// computed, for lanes already known to be accepted (the same expressions,
// so the same bits).
template <int DT, bool ACC, class UFF, class UDF>
__device__ __forceinline__ uint64_t beta_comp_u(const BetaComp g, const int type, UFF&& Uf, UDF&& Ud, bool& acc) {
  acc = true;
  const int U = g.U;
  if (DT == SD_F32) {
    if (type == 0) return f2u(1.0f * (-(logf_(1.0f - Uf(0)) / 1.0f)));
    if (type == 1) {
      float y = Uf(0) + 1.1920928955078125e-07f / 8;
      for (int t = 1; t < U; ++t) y = y * (Uf(t) + 1.1920928955078125e-07f / 8);
      return f2u(-(1.0f * logf_(y)));
    }
    if (type == 2) {
      const float ux = Uf(0), vx = Uf(1) + 1.1920928955078125e-07f / 8;
      const float lv = logf_(vx);
      const bool c = ux < g.f_px;
      if (!ACC) return f2u(1.0f * (c ? expf_(g.f_inv * lv) : 1.0f - lv));
      const float e1 = expf_(c ? g.f_inv * lv : logf_(1.0f - lv) * g.f_am1);  // one exp for both branches
      acc = Uf(2) < (c ? expf_(-e1) : e1);
      return f2u(1.0f * (c ? e1 : 1.0f - lv));
    }
    const float a1 = g.f_am1, sq = g.f_sq;
    float ys, yc;
    sincosf_((float)3.1415926535897932 * Uf(0), ys, yc);
    const float yx = ys / yc;
    const float xx = sq * yx + a1;
    if (ACC) {
      const float ub = (yx * yx + 1.0f) * expf_(a1 * logf_(xx / a1) - yx * sq);
      acc = (0.0f < xx) && (Uf(1) <= ub);
    }
    return f2u(1.0f * xx);
  } else {
    if (type == 0) return d2u(1.0 * (-(log_(1.0 - Ud(0)) / 1.0)));
    if (type == 1) {
      double y = Ud(0) + 2.220446049250313e-16 / 8;
      for (int t = 1; t < U; ++t) y = y * (Ud(t) + 2.220446049250313e-16 / 8);
      return d2u(-(1.0 * log_(y)));
    }
    if (type == 2) {
      const double ux = Ud(0), vx = Ud(1) + 2.220446049250313e-16 / 8;
      const double lv = log_(vx);
      double xx;
      if (ux < g.d_px) {
        xx = exp_(g.d_inv * lv);
        if (ACC) acc = Ud(2) < exp_(-xx);
      } else {
        xx = 1.0 - lv;
        if (ACC) acc = Ud(2) < exp_(log_(xx) * g.d_am1);
      }
      return d2u(1.0 * xx);
    }
    const double a1 = g.d_am1, sq = g.d_sq;
    double ys, yc;
    sincos_(3.1415926535897932 * Ud(0), ys, yc);
    const double yx = ys / yc;
    const double xx = sq * yx + a1;
    if (ACC) {
      const double ub = (yx * yx + 1.0) * exp_(a1 * log_(xx / a1) - yx * sq);
      acc = (0.0 < xx) && (Ud(1) <= ub);
    }
    return d2u(1.0 * xx);
  }
}

}  // namespace

// ===========================================================================
// k_beta: the walk with the reference automaton on a warp of its own, one
// step ahead of the workers.
//   chase  (warp 0) follows the automaton over the accept masks: per trial
//          of a rejection component one mask read, its popcount and two
//          compares.  Per step it records the source of every output packet
//          (closed-form position, full-trial value slot or FIFO offset) and,
//          for every accepted lane of a consumed partial trial, its FIFO slot
//          (position and lane, written by the warp's first P lanes at once),
//          into one of two buffers.
//   work   (warps 1-5) take the previous step's buffer: the full-trial values
//          of the rejection component, the accepted partial lanes and the
//          positional values of the other component as one task list;
//          p1 / (p1 + p2) per output lane; the carried lanes to the front of
//          the lane buffer; then they twist the next engine block and
//          evaluate its accept masks.
// The chase of step t reads only masks; the workers of step t - 1 read the
// raw ring (blocks t - 2 .. t) before they overwrite block t - 2 with block
// t + 1, so the step's packets must start at block t - 2 or later (checked;
// a record longer than two blocks ends the call with the iteration-cap
// status).  Buffers hold more than one block's worth of records, partial
// lanes and FIFO lanes, so a chase that fell behind catches up.
// TY0 / TY1: the components' sampler types when known at compile time (the
// kernel then carries only their code), else -1.
// ===========================================================================
namespace {

constexpr int kBcThreads = 192;       // four CTAs per SM
constexpr int kBcThreadsAlone = 512;  // one CTA per SM (no more engines than SMs): fifteen worker warps
constexpr uint16_t kBcTabNone = 0xffffu;  // visit-table entry not known yet
constexpr int kBcRec = 160;         // output packets per step (a block holds at most 156)
constexpr int kBcFifo = 112;        // FIFO outputs per component per step (at most 104 per block)
constexpr int kBcFull = 112;        // full-trial outputs of the buffered component per step
constexpr int kBcFullTag = 16384;   // record source >= this: full-trial value slot

template <int DT>
__host__ __device__ constexpr int bc_lb() {  // lane buffer per component: carried + one step's FIFO lanes
  return 16 + kBcFifo * beta_lanes<DT>();
}

struct BcStep {
  int64_t base, e0;  // first packet of the step (sources are relative to it), first output packet
  int nrec, nf, fs[2], A[2], f[2];
};

template <int DT, bool TAB>
__host__ __device__ constexpr size_t bc_smem_bytes() {
  return (TAB ? (size_t)kBetaRing * beta_lanes<DT>() * 2 + (size_t)2 * kBcRec * 6 : 0) +  // visit table, record starts
         (size_t)3 * kLanes * kN * 8 +                                                   // raw windows
         ((size_t)2 * bc_lb<DT>() + (size_t)(kBcFull + kBcRec) * beta_lanes<DT>()) *     // lane buffers, full-
             (DT == SD_F64 ? 8 : 4) +                                                    //   trial and positional values
         (size_t)2 * kBcRec * 2 * 2 +                                                    // records
         (size_t)2 * kBcFull * 2 +                                                       // full-trial positions
         (size_t)2 * 2 * bc_lb<DT>() * 2 +                                               // partial-lane tasks
         (size_t)2 * kBetaRing;                                                          // masks per position
}

}  // namespace

// ALONE: one CTA per SM.  For the GS + integral-alpha pairs it also keeps a
// visit table: for every position and carry, where the GS visit starting
// there ends, whether on a full trial, and the lanes its partial trials
// accept.  The chase then reads one entry per record, and the workers
// expand each record's partial trials into FIFO slots themselves.
template <int DT, int TY0, int TY1, bool ALONE>  // DT: SD_F32 or SD_F64
__global__ void __maxnreg__(80) k_beta(Plan p, BetaConsts bk, int64_t max_blocks) {
  constexpr int NT = ALONE ? kBcThreadsAlone : kBcThreads;
  constexpr int kBcWork = NT - 32;
  constexpr bool kFusedPair = (TY0 == 2 && TY1 == 1) || (TY0 == 1 && TY1 == 2);
  constexpr bool TAB = ALONE && kFusedPair;
  constexpr int P = beta_lanes<DT>();
  constexpr int LB = bc_lb<DT>();
  constexpr unsigned FULL = 0xffffffffu;
  using V = typename std::conditional<DT == SD_F64, uint64_t, uint32_t>::type;
  extern __shared__ __align__(16) uint64_t bc_dyn[];
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(bc_dyn);
  V* lanebuf = reinterpret_cast<V*>(bc_dyn + 3 * kLanes * kN);          // [2][LB]
  V* fullval = lanebuf + 2 * LB;                                         // [kBcFull][P]
  V* posval = fullval + kBcFull * P;                                     // [kBcRec][P]
  int16_t* rec = reinterpret_cast<int16_t*>(posval + kBcRec * P);        // [2][kBcRec][2]
  int16_t* fpos = rec + 2 * kBcRec * 2;                                  // [2][kBcFull]
  uint16_t* ptask = reinterpret_cast<uint16_t*>(fpos + 2 * kBcFull);     // [2][2][LB]
  uint8_t* pmask = reinterpret_cast<uint8_t*>(ptask + 2 * 2 * LB);       // [2][kBetaRing]
  uint16_t* vtab = reinterpret_cast<uint16_t*>(pmask + 2 * kBetaRing);    // [kBetaRing][P] (TAB)
  int16_t* rxs = reinterpret_cast<int16_t*>(vtab + (TAB ? kBetaRing * P : 0));  // [2][kBcRec] visit starts (TAB)
  uint16_t* ras = reinterpret_cast<uint16_t*>(rxs + (TAB ? 2 * kBcRec : 0));    // [2][kBcRec] FIFO tail at the start
  uint16_t* rfs = ras + (TAB ? 2 * kBcRec : 0);                                 // [2][kBcRec] carry at the start
  __shared__ BcStep s_step[2];
  __shared__ int s_done, s_err, s_fc[2];
  __shared__ int64_t s_end;
  __shared__ unsigned long long s_inv[2];  // TAB: first position whose table entry is still unknown

  const int k = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  EngState* st = p.eng + k;
  GenState* gs = p.gen + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  const int64_t Npk = n / P;

  const int type0 = TY0 >= 0 ? TY0 : bk.c[0].type, type1 = TY1 >= 0 ? TY1 : bk.c[1].type;
  const int U0 = bk.c[0].U, U1 = bk.c[1].U;
  const bool post = bk.post == 1;
  const int umax = max(max(U0, U1), 3);
  // bc: the rejection component whose full-trial values get a slot; ob: the
  // component whose positional values are computed with them
  const int bc = type0 >= 2 ? 0 : (type1 >= 2 ? 1 : -1);
  const int ob = bc == 0 ? 1 : (bc == 1 ? 0 : 1);
  load_window(raw[2], &st->win[0][0], kN);  // block -1; block b lives in window b mod 3
  // carried lanes of the two GammaGens (generator slots 1 and 2)
  if (tid < 2 * 8) {
    const int c = tid / 8, j = tid % 8;
    const GenSlot& g = gs->s[1 + c];
    if (j < g.rest_cnt)
      lanebuf[c * LB + j] = (V)(DT == SD_F64 ? ((uint64_t)g.rest[2 * j] | ((uint64_t)g.rest[2 * j + 1] << 32))
                                             : (uint64_t)g.rest[j]);
  }
  if (tid == 0) {
    s_err = 0;
    s_done = 0;
  }
  __syncthreads();
  // The newest three raw blocks are the ring of packets; words are tempered
  // where they are read.  Each thread keeps its own view of the newest block.
  int64_t ring_new = 0;
  int wb0 = 0, wb1 = 2, wb2 = 1;
  auto set_ring = [&](int64_t B) {
    ring_new = B * kN;
    wb0 = (int)(B % 3);
    wb1 = (int)((B + 2) % 3);
    wb2 = (int)((B + 1) % 3);
  };
  auto tword = [&](int64_t rel, int l) -> uint64_t {
    int dd = (int)(rel - ring_new);
    int w = wb0;
    if (dd < 0) {
      dd += kN;
      w = wb1;
      if (dd < 0) {
        dd += kN;
        w = wb2;
      }
    }
    if ((unsigned)dd >= (unsigned)kN) dd = 0;  // outside the ring: never read past the buffers
    return mt_temper(raw[w][l][dd]);
  };
  auto word = [&](int64_t w) -> uint32_t {
    const uint64_t v = tword(w >> 3, (int)((w & 7) >> 1));
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  auto rval = [&](int64_t r) -> uint64_t { return tword(r >> 2, (int)(r & 3)); };
  // value of an accepted trial lane or a closed-form draw; double GS lanes
  // use the branch threshold in integer form
  auto value = [&](int c, int64_t x, int j) -> uint64_t {
    bool acc;
    auto uf = [&](int q) { return ur_f(word((x + q) * 8 + j)); };
    auto ud = [&](int q) { return ur_d(rval((x + q) * 4 + j)); };
    if (c == 0) {
      if (DT == SD_F64 && type0 == 2)
        return d2u(1.0 * gs_value_f64(rval(x * 4 + j), rval((x + 1) * 4 + j), bk.c[0].tpx, bk.c[0].d_inv));
      return beta_comp_u<DT, false>(bk.c[0], type0, uf, ud, acc);
    }
    if (DT == SD_F64 && type1 == 2)
      return d2u(1.0 * gs_value_f64(rval(x * 4 + j), rval((x + 1) * 4 + j), bk.c[1].tpx, bk.c[1].d_inv));
    return beta_comp_u<DT, false>(bk.c[1], type1, uf, ud, acc);
  };
  // The GS + integral-alpha pairs: the value of either component is one log
  // (of the GS trial's vx, or of the product of the integral draw's
  // uniforms), then an exp for GS lanes below the branch threshold; every
  // lane of a warp shares the log whichever component it computes.
  constexpr bool kFused = (TY0 == 2 && TY1 == 1) || (TY0 == 1 && TY1 == 2);
  constexpr int gc = TY0 == 2 ? 0 : 1;  // the GS component of a fused pair
  auto value_task = [&](int c, int64_t x, int j) -> uint64_t {
    if (!kFused) return value(c, x, j);
    const BetaComp& g = c == 0 ? bk.c[0] : bk.c[1];
    const bool gsv = c == gc;
    if (DT == SD_F64) {
      constexpr double e = 2.220446049250313e-16 / 8;
      const uint64_t b0 = rval(x * 4 + j), b1 = rval((x + 1) * 4 + j);
      double arg = ur_d(b1) + e;
      if (!gsv) {
        double y = ur_d(b0) + e;
        y = y * arg;
        for (int q = 2; q < g.U; ++q) y = y * (ur_d(rval((x + q) * 4 + j)) + e);
        arg = y;
      }
      const double l = log_(arg);
      if (!gsv) return d2u(-(1.0 * l));
      return d2u(1.0 * (((b0 & 0xfffffffffffffull) < g.tpx) ? exp_(g.d_inv * l) : 1.0 - l));
    } else {
      constexpr float e = 1.1920928955078125e-07f / 8;
      const float u0 = ur_f(word(x * 8 + j)), u1 = ur_f(word((x + 1) * 8 + j));
      float arg = u1 + e;
      if (!gsv) {
        float y = u0 + e;
        y = y * arg;
        for (int q = 2; q < g.U; ++q) y = y * (ur_f(word((x + q) * 8 + j)) + e);
        arg = y;
      }
      const float l = logf_(arg);
      if (!gsv) return f2u(-(1.0f * l));
      return f2u(1.0f * ((u0 < g.f_px) ? expf_(g.f_inv * l) : 1.0f - l));
    }
  };
  const int nrej = (type0 >= 2 ? 1 : 0) + (type1 >= 2 ? 1 : 0);
  const int rej0 = type0 >= 2 ? 0 : 1;
  // accept masks of the rejection components at positions [from, to), by
  // threads t = 0 .. T-1 of whole warps.  Each group of P threads (one per
  // lane) walks a run of consecutive positions and slides a window of the
  // lane's three tempered words along it (one word fetched per position);
  // a ballot per step gives the masks of the warp's 32 / P runs.
  auto masks = [&](int64_t from, int64_t to, int t, int T) {
    if (nrej == 0 || to <= from) return;
    constexpr int G = 32 / P;
    const int runs = (T >> 5) * G;
    const int L = ((int)(to - from) + runs - 1) / runs;
    const int r = (t >> 5) * G + (t & 31) / P, j = t & (P - 1);
    const int lw = DT == SD_F64 ? j : (j >> 1);  // the lane's 64-bit word
    const int64_t x0 = from + (int64_t)r * L;
    for (int ci = 0; ci < nrej; ++ci) {
      const int c = nrej == 2 ? ci : rej0;
      const int ty = c == 0 ? type0 : type1;
      uint64_t w0 = 0, w1 = tword(x0, lw), w2 = tword(x0 + 1, lw);
      for (int i = 0; i < L; ++i) {
        const int64_t x = x0 + i;
        const bool valid = x < to;
        w0 = w1;
        w1 = w2;
        w2 = tword(x + 2, lw);
        bool acc = false;
        if (valid) {
          int f = -1;
          if (DT == SD_F64 && ty == 2)  // float pre-test of a double GS trial
            f = c == 0 ? gs_filter_f64(w0, w1, w2, bk.c[0].f_px, bk.c[0].f_inv, bk.c[0].f_am1, bk.c[0].f_band)
                       : gs_filter_f64(w0, w1, w2, bk.c[1].f_px, bk.c[1].f_inv, bk.c[1].f_am1, bk.c[1].f_band);
          if (f >= 0) {
            acc = f == 1;
          } else {
            auto uf = [&](int q) {
              const uint64_t v = q == 0 ? w0 : (q == 1 ? w1 : w2);
              return ur_f((j & 1) ? (uint32_t)(v >> 32) : (uint32_t)v);
            };
            auto ud = [&](int q) { return ur_d(q == 0 ? w0 : (q == 1 ? w1 : w2)); };
            if (c == 0) beta_comp_u<DT, true>(bk.c[0], type0, uf, ud, acc);
            else beta_comp_u<DT, true>(bk.c[1], type1, uf, ud, acc);
          }
        }
        const uint32_t bal = __ballot_sync(FULL, acc);
        if (valid && j == 0)
          pmask[c * kBetaRing + (int)(x & (kBetaRing - 1))] =
              (uint8_t)((bal >> (threadIdx.x & 31 & ~(P - 1))) & ((1u << P) - 1));
      }
    }
  };
  // TAB: visit-table entries of positions [from, to) (masks known below
  // `to`), by threads t = 0 .. T-1; an entry whose visit runs past `to` stays
  // unknown and its position is noted in *inv
  constexpr int gcomp = TY0 == 2 ? 0 : 1;  // the GS component of a fused pair
  auto build_table = [&](int64_t from, int64_t to, int t, int T, unsigned long long* inv) {
    if (!TAB || to <= from) return;
    const int U = gcomp == 0 ? U0 : U1;
    const int cnt = (int)(to - from) * P;
    for (int u = t; u < cnt; u += T) {
      const int64_t x = from + u / P;
      const int f = u % P;
      uint16_t e = kBcTabNone;
      int acc = 0;
      for (int d = 0; d < 1024 - U; d += U) {
        const int64_t xr = x + d;
        if (xr >= to) break;
        const uint32_t m = pmask[gcomp * kBetaRing + (int)(xr & (kBetaRing - 1))];
        const int cn = __popc(m);
        if (cn == P) {
          e = (uint16_t)(d | (1 << 10) | (acc << 11));
          break;
        }
        acc += cn;
        if (f + acc >= P) {
          e = (uint16_t)(d | (acc << 11));
          break;
        }
      }
      vtab[(int)(x & (kBetaRing - 1)) * P + f] = e;
      if (e == kBcTabNone) atomicMin(inv, (unsigned long long)x);
    }
  };
  // block 0 and its masks (all threads)
  mt_block(raw[2], raw[0], [&](int, const uint64_t*) {});
  set_ring(0);
  masks(0, kN - umax + 1, tid, NT);
  if (TAB) {
    if (tid == 0) s_inv[0] = (unsigned long long)(kN - umax + 1);
    __syncthreads();
    build_table(0, kN - umax + 1, tid, NT, &s_inv[0]);
  }
  __syncthreads();

  // chase state (warp 0, the same in every lane)
  int64_t cx = 0, cE = 0;
  int cf[2] = {0, 0};
  if (warp == 0) {
    cf[0] = gs->s[1].rest_cnt;
    cf[1] = gs->s[2].rest_cnt;
  }
  int64_t B = 0;  // newest block generated
  bool done = false;
  for (int64_t t = 0;; ++t) {
    const bool gen = !done && t + 1 < max_blocks;
    const int64_t M = (t + 1) * kN - umax + 1;  // positions with masks
    if (warp == 0) {
      if (!done) {
        // ---- chase step t into buffer t mod 2
        const int q = (int)(t & 1);
        const int64_t pk_lim = (t + 1) * kN;  // packets generated
        int16_t* rq = rec + q * kBcRec * 2;
        int16_t* fq = fpos + q * kBcFull;
        uint16_t* tq = ptask + q * 2 * LB;
        int16_t* xq = rxs + q * kBcRec;
        uint16_t* aq = ras + q * kBcRec;
        uint16_t* fsq = rfs + q * kBcRec;
        const int64_t base = cx, e0 = cE;
        const int fs0 = cf[0], fs1 = cf[1];
        int nrec = 0, nf = 0, A[2] = {cf[0], cf[1]};
        const bool lag = cx < (t - 1) * kN;
        const int Mr = (int)(M - base), bm = (int)(base & (kBetaRing - 1));
        if (!lag) {
          while (cE < Npk && nrec < kBcRec) {
            const int64_t xs = cx;
            const int cf0 = cf[0], cf1 = cf[1], A0 = A[0], A1 = A[1], nfs = nf;
            // one component of record nrec: 0 done, 1 a buffer is full,
            // 2 positions not evaluated or packets not generated yet
            auto visit = [&](auto cc) -> int {
              constexpr int c = decltype(cc)::value;
              const int ty = c == 0 ? type0 : type1, U = c == 0 ? U0 : U1;
              if (ty <= 1) {
                if (cx + U > pk_lim) return 2;
                if (lane == 0) rq[nrec * 2 + c] = (int16_t)(cx - base);
                cx += U;
                return 0;
              }
              const int fsc = c == 0 ? fs0 : fs1;
              int acc = 0;
              int xr = (int)(cx - base);  // trial position relative to the step
              if (TAB) {
                // one table entry: the visit's end, its kind and the lanes its
                // partial trials accept; the workers place those lanes
                if (xr >= Mr) return 2;
                const uint32_t e = vtab[((bm + xr) & (kBetaRing - 1)) * P + cf[c]];
                if (e == kBcTabNone) return 2;
                acc = (int)(e >> 11);
                if (A[c] + acc > LB) return 1;
                const int xe = xr + (int)(e & 1023u);
                if (lane == 0) {
                  xq[nrec] = (int16_t)xr;
                  aq[nrec] = (uint16_t)A[c];
                  fsq[nrec] = (uint16_t)cf[c];
                }
                if (e & (1u << 10)) {
                  if (c == bc) {
                    if (nf >= kBcFull) return 1;
                    if (lane == 0) {
                      fq[nf] = (int16_t)xe;
                      rq[nrec * 2 + c] = (int16_t)(kBcFullTag + nf);
                    }
                    ++nf;
                  } else if (lane == 0) {
                    rq[nrec * 2 + c] = (int16_t)xe;
                  }
                  cf[c] += acc;
                } else {
                  if (lane == 0) rq[nrec * 2 + c] = (int16_t)(-(1 + (A[c] - cf[c])));
                  cf[c] += acc - P;
                }
                A[c] += acc;
                cx = base + xe + U;
                return 0;
              }
              for (;;) {
                if (xr >= Mr) return 2;
                const uint32_t m = pmask[c * kBetaRing + ((bm + xr) & (kBetaRing - 1))];
                const int cn = __popc(m);
                if (cn == P) {  // a full trial ends the visit; the partial lanes stay carried
                  if (c == bc) {
                    if (nf >= kBcFull) return 1;
                    if (lane == 0) {
                      fq[nf] = (int16_t)xr;
                      rq[nrec * 2 + c] = (int16_t)(kBcFullTag + nf);
                    }
                    ++nf;
                  } else if (lane == 0) {
                    rq[nrec * 2 + c] = (int16_t)xr;
                  }
                  cf[c] += acc;
                  break;
                }
                if (A[c] + acc + cn > LB) return 1;
                // FIFO slots of the trial's accepted lanes
                if (lane < P && ((m >> lane) & 1u))
                  tq[c * LB + A[c] + acc - fsc + __popc(m & ((1u << lane) - 1u))] = (uint16_t)((xr << 3) | lane);
                acc += cn;
                if (cf[c] + acc >= P) {  // the carry fills: its oldest P lanes are the output
                  if (lane == 0) rq[nrec * 2 + c] = (int16_t)(-(1 + (A[c] - cf[c])));
                  cf[c] += acc - P;
                  break;
                }
                xr += U;
              }
              A[c] += acc;
              cx = base + xr + U;
              return 0;
            };
            int r = visit(std::integral_constant<int, 0>{});
            if (!r) r = visit(std::integral_constant<int, 1>{});
            if (r) {
              cx = xs;
              cf[0] = cf0;
              cf[1] = cf1;
              A[0] = A0;
              A[1] = A1;
              nf = nfs;
              break;
            }
            ++nrec;
            ++cE;
          }
        }
        if (lane == 0) {
          BcStep& S = s_step[q];
          S.base = base;
          S.e0 = e0;
          S.nrec = nrec;
          S.nf = nf;
          S.fs[0] = fs0;
          S.fs[1] = fs1;
          S.A[0] = A[0];
          S.A[1] = A[1];
          S.f[0] = cf[0];
          S.f[1] = cf[1];
          if (lag) s_err = 1;
          if (cE >= Npk) {
            s_done = 1;
            s_end = cx;
          }
        }
      }
    } else {
      const int tt = tid - 32;
      if (t >= 1 && s_step[(t - 1) & 1].nrec > 0) {
        // ---- step t - 1: values and outputs
        const int q = (int)((t - 1) & 1);
        const BcStep& S = s_step[q];
        const int nrec = S.nrec, nf = S.nf;
        const int fs0 = S.fs[0], fs1 = S.fs[1];
        const int64_t base = S.base;
        const int16_t* rq = rec + q * kBcRec * 2;
        uint16_t* tq = ptask + q * 2 * LB;
        set_ring(t);
        if (TAB) {
          // the accepted lanes of each record's partial trials at their FIFO
          // slots (the visit walked again from its start)
          const int U = gcomp == 0 ? U0 : U1;
          const int bmq = (int)(base & (kBetaRing - 1));
          const int fsg = gcomp == 0 ? fs0 : fs1;
          for (int i = tt; i < nrec; i += kBcWork) {
            int xr = rxs[q * kBcRec + i], run = 0;
            const int a0 = ras[q * kBcRec + i] - fsg, f0 = rfs[q * kBcRec + i];
            for (int d = 0; d < 1024; d += U, xr += U) {
              const uint32_t m = pmask[gcomp * kBetaRing + ((bmq + xr) & (kBetaRing - 1))];
              const int cn = __popc(m);
              if (cn == P) break;
              for (uint32_t mm = m; mm; mm &= mm - 1) {
                const int j = __ffs(mm) - 1;
                tq[gcomp * LB + a0 + run + __popc(m & ((1u << j) - 1u))] = (uint16_t)((xr << 3) | j);
              }
              run += cn;
              if (f0 + run >= P) break;
            }
          }
          asm volatile("bar.sync 1, %0;" ::"r"(kBcWork) : "memory");
        }
        // one task list, one lane per thread: full trials of the buffered
        // component, the accepted partial-trial lanes, positional values of
        // the other component
        const int t0 = nf * P, tp0 = S.A[0] - fs0, tp1 = S.A[1] - fs1;
        const int t1 = t0 + tp0 + tp1;
        for (int u = tt; u < t1 + nrec * P; u += kBcWork) {
          int c, j, rel;
          V* dst;
          if (u < t0) {
            const int i = u / P;
            j = u % P;
            c = bc;
            rel = fpos[q * kBcFull + i];
            dst = fullval + i * P + j;
          } else if (u < t1) {
            c = u < t0 + tp0 ? 0 : 1;
            const int qq = c == 0 ? u - t0 : u - t0 - tp0;
            const int tk = tq[c * LB + qq];
            j = tk & 7;
            rel = tk >> 3;
            dst = lanebuf + c * LB + (c == 0 ? fs0 : fs1) + qq;
          } else {
            const int i = (u - t1) / P;
            j = (u - t1) % P;
            c = ob;
            rel = rq[i * 2 + ob];
            dst = (rel >= 0 && rel < kBcFullTag) ? posval + i * P + j : nullptr;
          }
          if (dst) *dst = (V)value_task(c, base + rel, j);
        }
        asm volatile("bar.sync 1, %0;" ::"r"(kBcWork) : "memory");
        // output packets
        const int64_t e0 = S.e0;
        for (int u = tt; u < nrec * P; u += kBcWork) {
          const int i = u / P, j = u % P;
          uint64_t v[2];
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            const int src = rq[i * 2 + c];
            if (src < 0) v[c] = (uint64_t)lanebuf[c * LB + (-src - 1) + j];
            else if (src >= kBcFullTag) v[c] = (uint64_t)fullval[(src - kBcFullTag) * P + j];
            else if (c == ob) v[c] = (uint64_t)posval[i * P + j];
            else v[c] = value(c, base + src, j);  // both components closed form
          }
          if (DT == SD_F32) {
            const float p1 = u2f((uint32_t)v[0]), p2 = u2f((uint32_t)v[1]);
            const float x = p1 / (p1 + p2);
            reinterpret_cast<float*>(p.out)[off + (e0 + i) * P + j] = post ? (bk.fpost * x) / (1.0f - x) : x;
          } else {
            const double p1 = u2d(v[0]), p2 = u2d(v[1]);
            const double x = p1 / (p1 + p2);
            reinterpret_cast<double*>(p.out)[off + (e0 + i) * P + j] = post ? (bk.dpost * x) / (1.0 - x) : x;
          }
        }
        // lanes still carried move to the front of each lane buffer
        V carry = 0;
        const int cc = tt / 8, cj = tt % 8;
        const bool mover = tt < 16 && cj < S.f[cc];
        if (mover) carry = lanebuf[cc * LB + S.A[cc] - S.f[cc] + cj];
        asm volatile("bar.sync 1, %0;" ::"r"(kBcWork) : "memory");
        if (mover) lanebuf[cc * LB + cj] = carry;
      }
      if (gen) {
        // ---- block t + 1 and its masks.  Word i < 156 of the new block needs
        // only the old block; word 156 + i needs new word i, which the same
        // thread made (word 311 needs new word 0: recomputed), so the twist
        // needs no barrier of its own
        uint64_t(*old)[kN] = raw[t % 3];
        uint64_t(*nw)[kN] = raw[(t + 1) % 3];
        for (int i = tt; i < kM; i += kBcWork) {
#pragma unroll
          for (int l = 0; l < kLanes; ++l) {
            const uint64_t lo = mt_twist(old[l][i], old[l][i + 1], old[l][i + kM]);
            const uint64_t n0 = i == kM - 1 ? mt_twist(old[l][0], old[l][1], old[l][kM]) : 0;
            const uint64_t hi = mt_twist(old[l][i + kM], i == kM - 1 ? n0 : old[l][i + kM + 1], lo);
            nw[l][i] = lo;
            nw[l][i + kM] = hi;
          }
        }
        asm volatile("bar.sync 1, %0;" ::"r"(kBcWork) : "memory");
        set_ring(t + 1);
        masks(M, M + kN, tt, kBcWork);
        if (TAB) {
          // entries still unknown from the last build and the new positions;
          // positions below (t - 1) * kN are behind any chase that has not
          // failed, so their entries are never read again
          const int q1 = (int)((t + 1) & 1);
          if (tt == 0) s_inv[q1] = (unsigned long long)(M + kN);
          asm volatile("bar.sync 1, %0;" ::"r"(kBcWork) : "memory");
          int64_t from = (int64_t)min(s_inv[t & 1], (unsigned long long)M);
          from = max(from, (t - 1) * (int64_t)kN);
          build_table(from, M + kN, tt, kBcWork, &s_inv[q1]);
        }
      }
    }
    __syncthreads();
    if (done || s_err) break;
    done = s_done != 0;
    if (gen) B = t + 1;
    if (!done && !gen) break;  // no block left for the chase: the iteration cap
  }

  // ---- state after the call
  if (tid == 0) {
    if (!s_done) s_end = cx;
    if (!s_done || s_err) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    s_fc[0] = cf[0];
    s_fc[1] = cf[1];
  }
  __syncthreads();
  const int64_t np = s_end;  // packets consumed
  if (np > 0) {
    const int64_t lastb = (np - 1) / kN;
    const int rr = (int)(np - lastb * kN);  // in [1, 312]
    if (lastb == B) {
      store_window(st, raw[B % 3], raw[(B + 2) % 3], rr);
    } else if (lastb == B - 1) {
      store_window(st, raw[(B + 2) % 3], raw[(B + 1) % 3], rr);
    } else if (lastb == B - 2 && B >= 2) {
      // block B - 3 was overwritten by block B: recover it from block B - 2
      // into block B's window (MT19937-64's twist inverts)
      if (tid < kLanes) {
        uint64_t* nwl = raw[(B + 1) % 3][tid];
        uint64_t* odl = raw[B % 3][tid];
        mt_untwist_block([&](int i) -> uint64_t& { return nwl[i]; }, [&](int i) -> uint64_t& { return odl[i]; });
      }
      __syncthreads();
      store_window(st, raw[(B + 1) % 3], raw[B % 3], rr);
    } else if (tid == 0) {
      atomicOr(&st->status, (int)GR_DEV_BAD_INPUT);
    }
  }
  if (tid < 2 * 8) {
    const int c = tid / 8, j = tid % 8;
    GenSlot& g = gs->s[1 + c];
    const uint64_t v = j < s_fc[c] ? (uint64_t)lanebuf[c * LB + j] : 0;
    if (DT == SD_F64) {
      g.rest[2 * j] = (uint32_t)v;
      g.rest[2 * j + 1] = (uint32_t)(v >> 32);
    } else {
      g.rest[j] = (uint32_t)v;
    }
  }
  __syncthreads();
  if (tid == 0) {
    gs->s[1].rest_cnt = s_fc[0];
    gs->s[2].rest_cnt = s_fc[1];
    st->consumed += (uint64_t)max(np, (int64_t)0);
  }
}

template <int DT>
static cudaError_t run_beta(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s) {
  BetaConsts bk;
  bk.c[0] = beta_component(d.ia, d.fa, d.da);
  bk.c[1] = beta_component(d.ib, d.fb, d.db);
  bk.post = d.post;
  bk.fpost = d.fh;
  bk.dpost = d.dh;
  static bool attr[64] = {};
  static int sms[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  constexpr size_t smem = bc_smem_bytes<DT, false>(), smem_t = bc_smem_bytes<DT, true>();
  if (!attr[dev]) {
    cudaError_t e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_beta<DT, -1, -1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_beta<DT, 2, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_beta<DT, 1, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_beta<DT, 2, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_beta<DT, 1, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  // the GS + integral-alpha pairs (beta(a < 1, integer b) and the mirror)
  // have kernels of their own; with no more engines than SMs each engine's
  // CTA has an SM to itself and runs the visit-table form
  const int t0 = bk.c[0].type, t1 = bk.c[1].type;
  const bool alone = p.K <= sms[dev];
  if (t0 == 2 && t1 == 1) {
    if (alone) k_beta<DT, 2, 1, true><<<p.K, kBcThreadsAlone, smem_t, s>>>(p, bk, max_blocks);
    else k_beta<DT, 2, 1, false><<<p.K, kBcThreads, smem, s>>>(p, bk, max_blocks);
  } else if (t0 == 1 && t1 == 2) {
    if (alone) k_beta<DT, 1, 2, true><<<p.K, kBcThreadsAlone, smem_t, s>>>(p, bk, max_blocks);
    else k_beta<DT, 1, 2, false><<<p.K, kBcThreads, smem, s>>>(p, bk, max_blocks);
  } else {
    k_beta<DT, -1, -1, false><<<p.K, kBcThreads, smem, s>>>(p, bk, max_blocks);
  }
  return cudaGetLastError();
}


// ===========================================================================
// k_uniform_int: UniformIntGen<int32_t>(min, max) whose range is not a power
// of two (Discrete.h:296-331).  Each output packet starts a fresh
// rx = rng.half(), tries its bit slices (the low `bits` bits, then rx >> bits
// while bitcnt + bits < 32) through CompressMask, and draws again until a
// packet is full; a packet with all four lanes accepted is returned as is and
// leaves the carried lanes alone.  One CTA per engine: all threads twist and
// temper a block into its 624 half-packet draws, then thread 0 runs the
// automaton over them (a few integer operations per slice).  A range of one
// value draws nothing and writes the constant.
// ===========================================================================
namespace {
constexpr int kUiThreads = 160;
}

__global__ void __launch_bounds__(kUiThreads) k_uniform_int(Plan p, DistParams d, int64_t max_blocks) {
  __shared__ uint64_t raw[2][kLanes][kN];
  __shared__ uint32_t hw[2 * kN][4];  // draw 2i: low half of packet i, 2i + 1: high half
  __shared__ int s_done;
  __shared__ int s_last;              // last draw consumed in the newest block, or -1
  const int k = blockIdx.x;
  const int tid = threadIdx.x;
  EngState* st = p.eng + k;
  GenSlot* gsl = &p.gen[k].s[0];
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  int32_t* out = reinterpret_cast<int32_t*>(p.out) + off;
  const int32_t pmin = d.ia;
  if (d.ib == 0) {  // pdiff == 0: pset1(pmin), no draws
    for (int64_t i = tid; i < n; i += kUiThreads) out[i] = pmin;
    return;
  }
  const uint32_t mask = d.bitmask;
  const int32_t plen = d.ic;
  const int bits = d.ncdf;
  const int64_t Npk = n / 4;

  // thread-0 automaton state: carried lanes and packets written
  uint32_t cache[8];
  int fc = 0;
  int64_t e = 0;
  auto put = [&](int64_t pk, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3) {
    int32_t* o = out + pk * 4;
    o[0] = (int32_t)(a0 + (uint32_t)pmin);
    o[1] = (int32_t)(a1 + (uint32_t)pmin);
    o[2] = (int32_t)(a2 + (uint32_t)pmin);
    o[3] = (int32_t)(a3 + (uint32_t)pmin);
  };
  // one rng.half() draw; true when it completed an output packet
  auto draw = [&](const uint32_t* w) -> bool {
    uint32_t rx[4] = {w[0], w[1], w[2], w[3]};
    int bitcnt = bits;
    for (;;) {
      uint32_t c[4];
      unsigned m = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        c[j] = rx[j] & mask;
        if ((int32_t)c[j] < plen) m |= 1u << j;
      }
      if (m == 15u) {
        put(e++, c[0], c[1], c[2], c[3]);
        return true;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if ((m >> j) & 1u) cache[fc++] = c[j];
      if (fc >= 4) {
        put(e++, cache[0], cache[1], cache[2], cache[3]);
#pragma unroll
        for (int j = 0; j < 3; ++j) cache[j] = cache[j + 4];
        fc -= 4;
        return true;
      }
      if (bitcnt + bits < 32) {
#pragma unroll
        for (int j = 0; j < 4; ++j) rx[j] >>= bits;
        bitcnt += bits;
      } else {
        return false;
      }
    }
  };

  load_window(raw[0], &st->win[0][0], kN);
  const int hv = st->half_valid;
  if (tid == 0) {
    fc = min(max(gsl->rest_cnt, 0), 3);  // at most P - 1 lanes are ever carried
    for (int j = 0; j < fc; ++j) cache[j] = gsl->rest[j];
    s_done = 0;
    s_last = -1;
    if (hv) {  // the engine's cached half is the first draw
      uint32_t w[4];
      for (int j = 0; j < 4; ++j) w[j] = st->half_cache[j];
      draw(w);
      if (e >= Npk) s_done = 1;
    }
  }
  __syncthreads();
  int cur = 0;
  int64_t nb = 0;
  for (; nb < max_blocks && !s_done; ++nb) {
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
      hw[2 * i][0] = (uint32_t)pk[0];
      hw[2 * i][1] = (uint32_t)(pk[0] >> 32);
      hw[2 * i][2] = (uint32_t)pk[1];
      hw[2 * i][3] = (uint32_t)(pk[1] >> 32);
      hw[2 * i + 1][0] = (uint32_t)pk[2];
      hw[2 * i + 1][1] = (uint32_t)(pk[2] >> 32);
      hw[2 * i + 1][2] = (uint32_t)pk[3];
      hw[2 * i + 1][3] = (uint32_t)(pk[3] >> 32);
    });
    cur ^= 1;
    if (tid == 0) {
      for (int h = 0; h < 2 * kN; ++h) {
        draw(hw[h]);
        if (e >= Npk) {
          s_last = h;
          s_done = 1;
          break;
        }
      }
    }
    __syncthreads();
  }

  // ---- state after the call
  const int last = s_last;
  if (last >= 0) {  // draws of the newest block were consumed: packets up to last / 2
    const int rr = last / 2 + 1;
    store_window(st, raw[cur], raw[cur ^ 1], rr);
  }
  if (tid == 0) {
    if (!s_done) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    if (last >= 0) {
      const int64_t np = (nb - 1) * kN + last / 2 + 1;
      st->consumed += (uint64_t)np;
      if ((last & 1) == 0) {  // the high half of the last packet stays in the half() cache
        for (int j = 0; j < 4; ++j) st->half_cache[j] = hw[last + 1][j];
        st->half_valid = 1;
      } else {
        st->half_valid = 0;
      }
    } else if (hv) {
      st->half_valid = 0;  // only the cached half was drawn
    }
    gsl->rest_cnt = fc;
    for (int j = 0; j < fc; ++j) gsl->rest[j] = cache[j];
  }
}

static cudaError_t run_uniform_int(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s) {
  k_uniform_int<<<p.K, kUiThreads, 0, s>>>(p, d, max_blocks);
  return cudaGetLastError();
}

// ===========================================================================
// k_negbin: NegativeBinomialGen<int32_t>(trials, p) (GammaPoisson.h:42-98).
// Per output packet: a Packet4f GammaGen((float)trials, (float)((1-p)/p))
// draw over rng.half() words (NormalExp.h:568-604), then a Poisson draw with
// those per-lane means: the multiplicative loop while no lane's mean exceeds
// 12, else tan rejection whose CompressMask carry is the GammaGen's.  One
// warp per engine: the warp twists its own engine blocks into 624
// half-packet draws, and lanes 0-3 run the packet code in lock step (one
// lane per packet lane, decisions by ballot).
// ===========================================================================
namespace {
constexpr int kNbWarps = 1;  // engines per CTA (30 KB of shared memory each: 7 CTAs per SM)
constexpr size_t kNbWarpBytes = (size_t)2 * kLanes * kN * 8 + (size_t)2 * kN * 16 + 64;  // windows, draws, carry
}

__global__ void __launch_bounds__(32 * kNbWarps) k_negbin(Plan p, DistParams d, int64_t max_blocks) {
  extern __shared__ __align__(16) uint64_t nb_dyn[];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kNbWarps + wi;
  if (k >= p.K) return;  // the whole warp
  uint8_t* base = reinterpret_cast<uint8_t*>(nb_dyn) + (size_t)wi * kNbWarpBytes;
  uint64_t(*raw)[kLanes][kN] = reinterpret_cast<uint64_t(*)[kLanes][kN]>(base);
  uint32_t(*hw)[4] = reinterpret_cast<uint32_t(*)[4]>(base + (size_t)2 * kLanes * kN * 8);
  uint32_t* carry = reinterpret_cast<uint32_t*>(base + (size_t)2 * kLanes * kN * 8 + (size_t)2 * kN * 16);
  EngState* st = p.eng + k;
  GenSlot* gsl = &p.gen[k].s[0];
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);
  const int64_t off = g0 * p.gran, n = ng * p.gran;
  if (n == 0) return;
  int32_t* out = reinterpret_cast<int32_t*>(p.out) + off;
  const int64_t Npk = n / 4;
  const float alpha = d.fa, beta = d.fb, gsq = d.fc, a1 = d.fd;
  const int count = d.ia, mode = d.ic;  // mode 0: alpha == 1, 1: product of count uniforms, 2: tan rejection
  const float eps8 = 1.1920928955078125e-07f / 8;
  const float fpi = (float)3.1415926535897932;
  (void)alpha;

  for (int i = lane; i < kLanes * kN; i += 32) raw[0][i / kN][i % kN] = st->win[i / kN][i % kN];
  int fc = min(max(gsl->rest_cnt, 0), 3);
  if (lane < fc) carry[lane] = gsl->rest[lane];
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
  // CompressMask::compress_append over lanes 0-3 (arch/AVX/PacketFilter.h:147-184)
  auto compress = [&](uint32_t bits, bool acc, uint32_t& res) -> bool {
    const unsigned m = mask4(acc);
    if (m == 0xfu) {
      res = bits;
      return true;
    }
    if (lane < 4 && ((m >> lane) & 1u)) carry[fc + __popc(m & ((1u << lane) - 1))] = bits;
    fc += __popc(m);
    __syncwarp();
    if (fc < 4) return false;
    res = lane < 4 ? carry[lane] : 0u;
    const uint32_t mv = lane < fc - 4 ? carry[4 + lane] : 0u;
    __syncwarp();
    if (lane < fc - 4) carry[lane] = mv;
    fc -= 4;
    __syncwarp();
    return true;
  };

  int64_t e = 0;
  for (; e < Npk && !abort; ++e) {
    float mean = 0.0f;
    if (mode == 0) {
      mean = beta * (-(logf_(1.0f - ur_f(next())) / 1.0f));
    } else if (mode == 1) {
      float y = ur_f(next()) + eps8;
      for (int c = 1; c < count; ++c) y = y * (ur_f(next()) + eps8);
      mean = -(beta * logf_(y));
    } else {
      for (;;) {
        float ys, yc;
        sincosf_(fpi * ur_f(next()), ys, yc);
        const float ux = ur_f(next());
        if (abort) break;
        const float yx = ys / yc;
        const float xx = gsq * yx + a1;
        const float ub = (yx * yx + 1.0f) * expf_(a1 * logf_(xx / a1) - yx * gsq);
        uint32_t r;
        if (compress(f2u(beta * xx), (0.0f < xx) && (ux <= ub), r)) {
          mean = u2f(r);
          break;
        }
      }
    }
    if (abort) break;
    const float pne = expf_(-mean);
    if (mask4(12.0f < mean) == 0) {
      float val = 1.0f;
      int32_t res = 0;
      for (;;) {
        val = val * ur_f(next());
        if (abort) break;
        const bool c = pne < val;
        if (mask4(c) == 0) break;
        res += c ? 1 : 0;
      }
      if (abort) break;
      if (lane < 4) out[e * 4 + lane] = res;
    } else {
      const float sq = sqrtf(2.0f * mean), lm = logf_(mean), g1 = mean * lm - lgamma_approxf_(mean + 1.0f);
      for (;;) {
        float s, c;
        sincosf_(fpi * ur_f(next()), s, c);
        const float yx = s / c;
        const float fres = truncf(sq * yx + mean);
        const float p1 = (yx * yx + 1.0f) * 0.9f;
        const float u2 = ur_f(next());
        if (abort) break;
        const float p2 = expf_((fres * lm - lgamma_approxf_(fres + 1.0f)) - g1);
        uint32_t r;
        if (compress(f2u(fres), (0.0f <= fres) && (u2 <= p1 * p2), r)) {
          if (lane < 4) out[e * 4 + lane] = cvtt_f32(u2f(r));
          break;
        }
      }
    }
  }

  // ---- state after the call
  if (abort) {
    if (lane == 0) atomicOr(&st->status, (int)GR_DEV_REJECT_LIMIT);
    return;
  }
  const bool used_block = nb > 0;  // the last draw came from the newest block (h >= 1)
  if (used_block) {
    const int last = h - 1;          // last draw consumed in the newest block
    const int rr = last / 2 + 1;     // packets used of it
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
  } else if (lane == 0 && st->half_valid && Npk > 0) {
    st->half_valid = 0;  // only the cached half was drawn
  }
  if (lane < fc) gsl->rest[lane] = carry[lane];
  if (lane == 0) gsl->rest_cnt = fc;
}

static cudaError_t run_negbin(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s) {
  constexpr size_t smem = kNbWarpBytes * kNbWarps;
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_negbin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  k_negbin<<<(p.K + kNbWarps - 1) / kNbWarps, 32 * kNbWarps, smem, s>>>(p, d, max_blocks);
  return cudaGetLastError();
}

cudaError_t launch_walk(const Plan& p, const DistParams& d, int64_t max_blocks, cudaStream_t s) {
  if (d.kind == GR_NEGATIVE_BINOMIAL) return run_negbin(p, d, max_blocks, s);
  if (d.kind == GR_UNIFORM_INT) return run_uniform_int(p, d, max_blocks, s);
  if (d.dtype == GR_I32) return run_poisson(p, d, max_blocks, s);
  if (d.dtype == GR_F32) return run_beta<SD_F32>(p, d, max_blocks, s);
  if (d.dtype == GR_F64) return run_beta<SD_F64>(p, d, max_blocks, s);
  return cudaErrorNotSupported;
}

}  // namespace gr
