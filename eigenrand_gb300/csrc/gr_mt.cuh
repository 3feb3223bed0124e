// MT19937-64 device building blocks shared by the sampling kernels.
//
// The recurrence, tempering and constants are those of MT19937-64
// (EigenRand/PacketRandomEngine.h:340-404 twist, :295-310 temper, :421-426
// constants); a Vmt19937_64 runs four such lanes in lock step.
#pragma once
#include <cstdint>

#include "gr_internal.h"
#include "gr_math.cuh"

namespace gr {

__device__ __forceinline__ uint64_t mt_twist(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t t = (a & kUpper) | (b & kLower);
  return (t >> 1) ^ ((0ull - (t & 1ull)) & kMatA) ^ c;
}

__device__ __forceinline__ uint64_t mt_temper(uint64_t r) {
  r ^= (r >> 29) & 0x5555555555555555ull;
  r ^= (r << 17) & 0x71d67fffeda60000ull;
  r ^= (r << 37) & 0xfff7eee000000000ull;
  r ^= r >> 43;
  return r;
}

__device__ __forceinline__ float ur_f(uint32_t x) { return u2f((x & 0x7fffffu) | (127u << 23)) - 1.0f; }
__device__ __forceinline__ double ur_d(uint64_t x) {
  return u2d((x & 0xfffffffffffffull) | (1023ull << 52)) - 1.0;
}

// One block (312 packets) of a 4-lane engine, computed by a CTA of >= 156
// threads: thread t makes new words t and t + 156.  Word t + 156 needs new
// word t (kept in a register) and, for word 311, new word 0 (recomputed from
// the old block), so the halves need no barrier between them.
// per_packet(i, pk) runs on the thread that produced packet i of the block
// (pk = the 4 tempered lane words).  Ends with a CTA barrier.
template <class F>
__device__ __forceinline__ void mt_block(uint64_t (*old)[kN], uint64_t (*nw)[kN], F&& per_packet) {
  const int tid = threadIdx.x;
  if (tid < kM) {
    uint64_t lo[kLanes];
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
      const int i = ph * kM + tid;
      uint64_t pk[kLanes];
#pragma unroll
      for (int l = 0; l < kLanes; ++l) {
        const uint64_t b = (i + 1 < kN) ? old[l][i + 1] : mt_twist(old[l][0], old[l][1], old[l][kM]);
        const uint64_t c = (ph == 0) ? old[l][i + kM] : lo[l];
        const uint64_t v = mt_twist(old[l][i], b, c);
        nw[l][i] = v;
        if (ph == 0) lo[l] = v;
        pk[l] = mt_temper(v);
      }
      per_packet(i, pk);
    }
  }
  __syncthreads();
}

// Packet `rel` of the two-block ring tp (blocks go to slots 0, 1, 0, ... in
// order): ring_new is the number of the newest block's first packet and
// ring_slot its slot.  Valid for ring_new - kN <= rel < ring_new + kN; a
// compare replaces the 64-bit division by 312.
template <class TP>
__device__ __forceinline__ const uint64_t* ring_packet(TP tp, int64_t rel, int64_t ring_new, int ring_slot) {
  int d = (int)(rel - ring_new);
  int sl = ring_slot;
  if (d < 0) {
    d += kN;
    sl ^= 1;
  }
  if ((unsigned)d >= (unsigned)kN) d = 0;  // outside the ring: never read past the buffers
  return tp[sl][d];
}

// Load the 4 lane windows of engine/segment into raw[0].
__device__ __forceinline__ void load_window(uint64_t (*raw)[kN], const uint64_t* src, size_t lane_stride) {
  for (int i = threadIdx.x; i < kLanes * kN; i += blockDim.x)
    raw[i / kN][i % kN] = src[(size_t)(i / kN) * lane_stride + i % kN];
}

// After generating packets up to (exclusive) packet index `end` where the last
// generated block covers [last_base, last_base + 312): write the 312 raw words
// preceding `end` as the engine's new window.
__device__ __forceinline__ void store_window(EngState* st, uint64_t (*lastb)[kN], uint64_t (*prevb)[kN], int rr) {
  for (int t = threadIdx.x; t < kLanes * kN; t += blockDim.x) {
    const int l = t / kN, i = t % kN;
    st->win[l][i] = (i < kN - rr) ? prevb[l][rr + i] : lastb[l][i - (kN - rr)];
  }
}

}  // namespace gr
