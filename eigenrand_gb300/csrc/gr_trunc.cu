// TruncGen's rejection (EigenRand/Dists/Truncated.h:247-262) over a chunk of
// base packets already drawn into HBM.
//
// TruncGen<Base>::packetOp draws base packets and passes each through
// CompressMask::compress_append with the mask lower <= x <= upper.  As an
// automaton over the base packets (carried lanes r0 at the start):
//   * a packet with every lane accepted ("full") is emitted as it is and the
//     carried lanes stay;
//   * otherwise its accepted lanes join a FIFO after the carried ones, and a
//     packet of P lanes is emitted whenever the FIFO holds P.
// With F_k full packets and A_k accepted lanes of partial packets before
// packet k, packet k emits output index F_k + floor((r0 + A_k) / P) when it
// is full or when it completes FIFO group floor((r0 + A_k) / P); groups are
// the FIFO lanes [P g, P g + P).  So the whole chunk resolves with one prefix
// sum of (full, partial accepted) pairs:
//   k_tr_count   per-CTA sums of the pairs (256 packets per CTA)
//   k_tr_scan    exclusive scan of the CTA sums; carried lanes into the FIFO
//   k_tr_place   per packet: full packets to their output slot, partial lanes
//                to their FIFO slot, output slot of each completed group, and
//                the packet that emits the last wanted output
//   k_tr_gather  FIFO groups to their output slots
//   k_tr_finish  the lanes carried after the stop packet (or the chunk)
// The host draws the base packets, runs this filter, and repeats with more
// packets until the call has its outputs; see gr_api.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "gr_internal.h"
#include "gr_kernels.cuh"

namespace gr {
namespace {

constexpr int kTrThreads = 256;

template <class T>
__device__ __forceinline__ bool in_support(T bits, double lo, double hi);
template <>
__device__ __forceinline__ bool in_support<uint32_t>(uint32_t bits, double lo, double hi) {
  const float v = __uint_as_float(bits);
  return (float)lo <= v && v <= (float)hi;
}
template <>
__device__ __forceinline__ bool in_support<uint64_t>(uint64_t bits, double lo, double hi) {
  const double v = __longlong_as_double((long long)bits);
  return lo <= v && v <= hi;
}

// Accept mask of packet k (bit j = lane j).
template <class T, int P>
__device__ __forceinline__ uint32_t packet_mask(const T* cand, int64_t k, double lo, double hi, T* v) {
  uint32_t m = 0;
#pragma unroll
  for (int j = 0; j < P; ++j) {
    v[j] = cand[k * P + j];
    m |= in_support<T>(v[j], lo, hi) ? (1u << j) : 0u;
  }
  return m;
}

// Exclusive scan of one packed value per thread over a 256-thread CTA.
template <class V>
__device__ __forceinline__ V block_exclusive(V x, V* sh, V& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  V inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const V y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) sh[w] = inc;
  __syncthreads();
  if (w == 0) {
    V t = lane < kTrThreads / 32 ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const V y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kTrThreads / 32) sh[lane] = t;
  }
  __syncthreads();
  total = sh[kTrThreads / 32 - 1];
  const V before = w ? sh[w - 1] : 0;
  __syncthreads();
  return before + inc - x;
}

// (full << 16) | partial accepted lanes of one packet: 256 packets of at most
// 7 lanes stay below 2^16 in the low half.
template <class T, int P>
__global__ void __launch_bounds__(kTrThreads) k_tr_count(TruncFilterArgs a) {
  __shared__ uint32_t sh[kTrThreads / 32];
  const int64_t k = (int64_t)blockIdx.x * kTrThreads + threadIdx.x;
  uint32_t code = 0;
  if (k < a.M) {
    T v[P];
    const uint32_t m = packet_mask<T, P>(static_cast<const T*>(a.cand), k, a.lower, a.upper, v);
    const int c = __popc(m);
    code = c == P ? (1u << 16) : (uint32_t)c;
  }
  uint32_t total;
  block_exclusive<uint32_t>(code, sh, total);
  if (threadIdx.x == 0) {
    a.blk[2 * blockIdx.x] = total >> 16;
    a.blk[2 * blockIdx.x + 1] = total & 0xffffu;
  }
}

// One CTA: exclusive scan of the per-CTA pairs (full count << 32 | lanes;
// a chunk holds < 2^23 packets), totals, and the carried lanes into the FIFO.
template <class T, int P>
__global__ void __launch_bounds__(kTrThreads) k_tr_scan(TruncFilterArgs a, int64_t nb) {
  __shared__ unsigned long long sh[kTrThreads / 32];
  unsigned long long run = 0;
  for (int64_t b0 = 0; b0 < nb; b0 += kTrThreads) {
    const int64_t b = b0 + threadIdx.x;
    const unsigned long long x =
        b < nb ? ((unsigned long long)a.blk[2 * b] << 32) | (unsigned long long)a.blk[2 * b + 1] : 0ull;
    unsigned long long tot;
    const unsigned long long ex = block_exclusive<unsigned long long>(x, sh, tot) + run;
    if (b < nb) {
      a.blk[2 * b] = (int64_t)(ex >> 32);
      a.blk[2 * b + 1] = (int64_t)(ex & 0xffffffffull);
    }
    run += tot;
  }
  const int r0 = a.carry->rest_cnt;
  if (threadIdx.x == 0) {
    const int64_t F = (int64_t)(run >> 32), A = (int64_t)(run & 0xffffffffull);
    const int64_t have = F + (r0 + A) / P;
    a.res[0] = have < a.cap ? have : a.cap;
    a.res[1] = -1;
    a.res[2] = F;
    a.res[3] = A;
    a.res[4] = r0 + A;
    a.res[5] = r0;
  }
  const T* rest = reinterpret_cast<const T*>(a.carry->rest);
  T* q = static_cast<T*>(a.queue);
  if (threadIdx.x < r0) q[threadIdx.x] = rest[threadIdx.x];
}

template <class T, int P>
__global__ void __launch_bounds__(kTrThreads) k_tr_place(TruncFilterArgs a) {
  __shared__ uint32_t sh[kTrThreads / 32];
  const int64_t k = (int64_t)blockIdx.x * kTrThreads + threadIdx.x;
  T v[P];
  uint32_t m = 0, code = 0;
  if (k < a.M) {
    m = packet_mask<T, P>(static_cast<const T*>(a.cand), k, a.lower, a.upper, v);
    const int c = __popc(m);
    code = c == P ? (1u << 16) : (uint32_t)c;
  }
  uint32_t total;
  const uint32_t ex = block_exclusive<uint32_t>(code, sh, total);
  if (k >= a.M) return;
  const int64_t Fk = a.blk[2 * blockIdx.x] + (ex >> 16);
  const int64_t X0 = (int64_t)a.carry->rest_cnt + a.blk[2 * blockIdx.x + 1] + (ex & 0xffffu);
  const int64_t g = X0 / P;
  T* out = static_cast<T*>(a.out);
  if (code >> 16) {
    const int64_t idx = Fk + g;
    if (idx < a.cap) {
#pragma unroll
      for (int j = 0; j < P; ++j) out[idx * P + j] = v[j];
    }
    if (idx == a.cap - 1) {
      a.res[1] = k;
      a.res[4] = X0;
    }
    return;
  }
  T* q = static_cast<T*>(a.queue);
  int r = 0;
#pragma unroll
  for (int j = 0; j < P; ++j) {
    if (m >> j & 1u) q[X0 + r++] = v[j];
  }
  const int64_t X1 = X0 + r;
  if (X1 / P > g) {
    const int64_t idx = Fk + g;
    a.grp[g] = idx < a.cap ? idx : -1;
    if (idx == a.cap - 1) {
      a.res[1] = k;
      a.res[4] = X1;
    }
  }
}

template <class T, int P>
__global__ void k_tr_gather(TruncFilterArgs a) {
  const int64_t G = a.res[4] / P;  // complete groups up to the stop (or the chunk end)
  const T* q = static_cast<const T*>(a.queue);
  T* out = static_cast<T*>(a.out);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < G * P; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t / P;
    const int64_t idx = a.grp[g];
    if (idx >= 0 && idx < a.cap) out[idx * P + (t - g * P)] = q[t];
  }
}

template <class T, int P>
__global__ void k_tr_finish(TruncFilterArgs a) {
  const int64_t X = a.res[4];
  const int64_t base = (X / P) * P;
  const int cnt = (int)(X - base);
  const T* q = static_cast<const T*>(a.queue);
  T* rest = reinterpret_cast<T*>(a.carry->rest);
  if ((int)threadIdx.x < cnt) rest[threadIdx.x] = q[base + threadIdx.x];
  if (threadIdx.x == 0) a.carry->rest_cnt = cnt;
}

template <class T, int P>
cudaError_t run_filter(const TruncFilterArgs& a, cudaStream_t s) {
  const int64_t nb = (a.M + kTrThreads - 1) / kTrThreads;
  k_tr_count<T, P><<<(unsigned)nb, kTrThreads, 0, s>>>(a);
  k_tr_scan<T, P><<<1, kTrThreads, 0, s>>>(a, nb);
  k_tr_place<T, P><<<(unsigned)nb, kTrThreads, 0, s>>>(a);
  const int64_t lanes = (a.M + 1) * P;
  const int64_t gb = (lanes + 255) / 256;
  k_tr_gather<T, P><<<(unsigned)(gb < 4096 ? gb : 4096), 256, 0, s>>>(a);
  k_tr_finish<T, P><<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trunc_filter(int dtype, const TruncFilterArgs& a, cudaStream_t s) {
  if (a.M <= 0 || a.M >= kTruncChunkMax) return cudaErrorInvalidValue;
  return dtype == GR_F64 ? run_filter<uint64_t, 4>(a, s) : run_filter<uint32_t, 8>(a, s);
}

}  // namespace gr
