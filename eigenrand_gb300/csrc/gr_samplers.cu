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

#include <cstdint>

#include "../../include/gpurand.h"
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

  auto word = [&](int64_t wq) -> uint32_t {  // cache-inclusive u32 word
    if (wq < c0w) return cw[wq];
    const int64_t w = wq - c0w;
    const int64_t pp = w >> 3;
    const int64_t rel = pp - seg_p0;
    const uint64_t v = tp[(rel / kN) & 1][rel % kN][(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  auto rword = [&](int64_t r) -> uint64_t {  // u64 lane value r of the packet stream (full kinds)
    const int64_t pp = r >> 2;
    const int64_t rel = pp - seg_p0;
    return tp[(rel / kN) & 1][rel % kN][r & 3];
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
      cur ^= 1;
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
          const float radius = sqrtf(d.fa * (expf_(logf_(u1) * d.fc) - 1.0f));
          float sn, cs;
          sincosf_((float)(2 * 3.1415926535897932) * u2, sn, cs);
          reinterpret_cast<float*>(p.out)[o] = radius * sn;
        }
      } else if (DT == SD_F64) {
        const int64_t r0 = u * (int64_t)U * 4 + j;
        if (KIND == GR_GAMMA || KIND == GR_CHI_SQUARED) {
          double y = ur_d(rword(r0)) + 2.220446049250313e-16 / 8;
          for (int t = 1; t < U; ++t) y = y * (ur_d(rword(r0 + 4 * t)) + 2.220446049250313e-16 / 8);
          reinterpret_cast<double*>(p.out)[o] = -(d.db * log_(y));
        } else if (KIND == GR_STUDENT_T) {
          const double u1 = 1.0 - ur_d(rword(r0));
          const double u2 = ur_d(rword(r0 + 4));
          const double radius = sqrt(d.da * (exp_(log_(u1) * d.dc) - 1.0));
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
      const int rr2 = (int)(np_seg - (nblk - 1) * kN);
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
