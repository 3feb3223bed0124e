// X = L Z + mean for MvNormalGen<float> on the 5th-generation tensor cores
// (tcgen05.mma, operands and accumulators in tensor memory).
//
// The product is computed sample-major, X^T = Z^T L^T: a tile of 128 samples
// is the M dimension (Z holds sample j's dim normals contiguously,
// EigenRand/MvDists/MvNormal.h:103-108), the output dimension is N and the
// input dimension K, in chunks of 32.  3xTF32: both operands are split into
// tf32 high and low parts (cvt.rna.tf32) and every K step issues lo x hi,
// hi x lo and hi x hi with FP32 accumulation.
//
// One persistent CTA per SM, warp-specialised, every hand-off an mbarrier:
//   warp 12  TMA: the tile's Z chunk (32 columns x 128 samples, 128-byte
//            swizzle) into a ring of raw slots;
//   warp 14  the factor: once per CTA when the whole prepared factor fits in
//            shared memory, else one slice per item into a ring of slots;
//   warps 4..11  two groups of four taking alternate items: read a raw slot
//            (row = sample, conflict-free thanks to the swizzle), split, and
//            tcgen05.st the high and low parts into an A stage in tensor memory;
//   warp 13  tcgen05.mma, A from tensor memory, B (the factor) from shared
//            memory, into an accumulator in tensor memory; tcgen05.commit
//            frees the stages and publishes finished accumulators;
//   warps 0..3 and 15..18  epilogue, two groups of four taking alternate
//            passes: tcgen05.ld (warp w owns lanes 32 (w % 4) ..), + mean,
//            through a swizzled staging tile into coalesced 16-byte stores.
// The single-lane work (TMA, bulk copies, MMAs, commits) is issued from
// warp-wide loops by one elected lane, and the per-item quantities (chunk,
// slice offsets, N, instruction descriptor, accumulator column) come from a
// table in the kernel parameters: the issuing loops do almost no arithmetic,
// which is what keeps the tensor pipe fed with M = 128, N <= 128 products.
//
// Tensor memory (512 columns): up to eight accumulator buffers in columns
// 0..255 (the pass width rounded up to 32, as many as fit), and four A
// stages of 64 columns (32 high + 32 low) in columns 256..511.
//
// Output dimensions are covered in passes of 128 (one pass up to D = 128, two
// up to 256).  A lower-triangular factor skips every zero block: chunk c only
// reaches outputs >= 32 c, so its products start at accumulator column
// max(32 c, pass start) with N shrunk to match.
//
// Every wait is bounded (a timer): on expiry the kernel sets a status bit,
// raises a CTA-wide abort flag that every other wait also watches, lets its
// copies and products in flight land, frees the tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "gr_internal.h"
#include "gr_mv.cuh"

namespace gr {

namespace {

constexpr int kUmmaM = 128;      // samples per tile (tensor-memory lanes)
constexpr int kUmmaKC = 32;      // K per chunk (one 128-byte swizzle row of float)
constexpr int kUmmaPassN = 128;  // output columns per pass
constexpr int kMaxItems = 16;    // items per tile: 2 passes x 8 chunks at most
constexpr int kRawSlotsMax = 12;
constexpr int kRawSlotsMin = 4;
constexpr int kAStages = 4;
constexpr int kBSlotsMax = 4;
constexpr int kAccMax = 8;
constexpr int kThreads = 608;  // 19 warps
constexpr int kEpiWarps = 4, kCvtWarp0 = 4, kCvtGroupWarps = 4, kTmaWarp = 12, kMmaWarp = 13, kBWarp = 14,
              kEpi2Warp0 = 15;
constexpr uint32_t kRawBytes = kUmmaM * kUmmaKC * 4;           // 16 KiB
constexpr uint32_t kBSlotBytes = kUmmaPassN * kUmmaKC * 4 * 2;  // 32 KiB (high + low)
constexpr uint32_t kStageOutBytes = 32 * 128;                   // 32 rows x 32 floats
constexpr uint32_t kOutBytes = 2 * kEpiWarps * kStageOutBytes;  // 32 KiB
constexpr uint32_t kMeanBytes = 2048;  // the mean (<= 256 floats + padding); keeps the factor 1024-byte aligned
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kACol0 = 256;  // A stage s at kACol0 + 64 s
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
constexpr uint32_t kItemFirst = 1, kItemLast = 2;       // first / last item of a pass

// Shared-memory matrix descriptor (tcgen05), no swizzle, K-major: leading
// byte offset 128 (the K-adjacent core matrix), stride byte offset 1024 (the
// next 8-row group), version 1; the start address (>> 4) is added in.
constexpr uint64_t kDescConst = ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46);
// the same with another stride byte offset (8-row group pitch)
__host__ __device__ constexpr uint64_t kDescConstW(uint32_t sbo) {
  return ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Instruction descriptor: FP32 accumulator, tf32 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
  return (1u << 4)                      // D format: F32
         | (2u << 7)                    // A format: TF32
         | (2u << 10)                   // B format: TF32
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

// ---- single-lane operations issued by the elected lane of a converged warp
__device__ __forceinline__ void mma_el(uint32_t dtmem, uint32_t atmem, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred e, p;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "@e tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "r"(atmem), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit_el(uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}\n" ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void expect_tx_el(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .pred e;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "@e mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n\t}\n" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ void bulk_g2s_el(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "@e cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n\t}\n" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_2d_el(uint32_t dst, const void* tmap, int x, int y, uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "@e cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];\n\t}\n" ::"r"(dst),
      "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// ---- mbarriers
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for the phase with this parity.  Gives up (false) when the CTA's abort
// flag is raised or after kWaitNs; a timeout raises the flag and the status.
__device__ __noinline__ bool mbar_wait_slow(uint64_t* bar, uint32_t parity, volatile int* abort, int32_t* status) {
  const unsigned long long t0 = gtimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 63) == 0) {
      if (*abort) return false;
      if (gtimer() - t0 > kWaitNs) {
        *abort = 1;
        atomicOr(status, (int)GR_DEV_MMA_TIMEOUT);
        return false;
      }
    }
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort, int32_t* status) {
  if (mbar_try(bar, parity)) return true;
  return mbar_wait_slow(bar, parity, abort, status);
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Warp-wide wait.  Every lane tests the phase (one broadcast read); if it is
// not complete yet, lane 0 waits and the other lanes follow it through
// __syncwarp (which orders their later accesses after lane 0's acquire).
__device__ __noinline__ bool warp_wait_slow(uint64_t* bar, uint32_t parity, volatile int* abort, int32_t* status) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait(bar, parity, abort, status) ? 1 : 0;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, volatile int* abort, int32_t* status) {
  if (__all_sync(0xffffffffu, mbar_test(bar, parity))) return true;
  return warp_wait_slow(bar, parity, abort, status);
}

// one arrival per warp, after every lane's earlier accesses
__device__ __forceinline__ void warp_arrive(uint64_t* bar) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
}

__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  const float r = x - __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  hi = __uint_as_float(h);
  lo = __uint_as_float(l);
}

// byte offset of (row, k) in a K-major no-swizzle tile of KC = 32 columns
__host__ __device__ constexpr uint32_t kmaj_off(int row, int k) {
  return (uint32_t)((row >> 3) * 1024 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// first factor row a chunk holds (zero rows above the diagonal are left out)
__host__ __device__ inline int chunk_row0(int c, int tri) { return tri ? kUmmaKC * c : 0; }

// byte offset of chunk c in the prepared factor: chunk c' holds 2 parts of
// (D - row0(c')) rows x 128 bytes
__host__ __device__ inline uint32_t chunk_off(int c, int D, int tri) {
  const uint32_t rows = tri ? (uint32_t)(c * D - 16 * c * (c - 1)) : (uint32_t)(c * D);
  return rows * 256u;
}

}  // namespace

// The factor as the B operand.  Chunk c (input columns 32c .. 32c + 31) holds
// rows row0(c) .. D - 1 of L (row0 = 32 c for a lower-triangular factor, else
// 0) as two parts, tf32 high then low, each in the K-major no-swizzle
// canonical layout: element (row, k) at kmaj_off(row - row0, k).
// B[row][k] = L[row][32 c + k] (L column-major FP64), zero outside dim x dim.
__global__ void k_prep_lt_umma(const double* L, float* out, int d, int D, int nchunks, int tri) {
  const int64_t total = (int64_t)nchunks * D * kUmmaKC;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / ((int64_t)D * kUmmaKC));
    const int rem = (int)(t % ((int64_t)D * kUmmaKC));
    const int row = rem / kUmmaKC, k = rem % kUmmaKC;
    const int r0 = chunk_row0(c, tri);
    if (row < r0) continue;
    const int kk = c * kUmmaKC + k;
    const float x = (row < d && kk < d) ? (float)L[(size_t)kk * d + row] : 0.0f;
    float hi, lo;
    split_tf32(x, hi, lo);
    float* base = out + chunk_off(c, D, tri) / 4;
    const uint32_t part = (uint32_t)(D - r0) * kUmmaKC;  // floats per part
    base[kmaj_off(row - r0, k) / 4] = hi;
    base[part + kmaj_off(row - r0, k) / 4] = lo;
  }
}

// One unit of work of a tile: chunk c of the input dimensions for the pass
// over outputs [n0, n1); it contributes to outputs [rs, n1).
struct UmmaItem {
  uint32_t x0;     // TMA column of the Z chunk (32 c)
  uint32_t boff;   // byte offset of the slice's high part in the prepared factor
  uint32_t part;   // bytes from a chunk's high part to its low part (prepared layout)
  uint32_t sl;     // bytes of one part of the slice ((n1 - rs) rows x 128)
  uint32_t idesc;  // instruction descriptor (M = 128, N = n1 - rs)
  uint32_t dcol;   // accumulator column of output rs (rs - n0)
  uint32_t n0, n1;
  uint32_t flags;  // kItemFirst / kItemLast of its pass
  uint32_t nks;    // K steps of 8 that hold input columns < dim (1 .. 4)
};

struct MvnUmmaArgs {
  const float* Lp;
  const float* mean;
  float* X;
  int64_t n;
  int32_t* status;
  int d;
  int resident;    // the whole prepared factor sits in shared memory
  int nb;          // slice slots when it does not
  int nr;          // raw Z slots
  int nacc;        // accumulator buffers (2 .. 8)
  int acc_stride;  // tensor-memory columns per accumulator buffer (a multiple of 32)
  uint32_t btotal;
  int nitems;
  UmmaItem items[kMaxItems];
};

__global__ void __launch_bounds__(kThreads, 1) k_mvn_umma(const __grid_constant__ CUtensorMap zmap,
                                                         const __grid_constant__ MvnUmmaArgs a) {
  extern __shared__ __align__(1024) unsigned char um_dyn[];
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)um_dyn + 1023) & ~(uintptr_t)1023);
  unsigned char* raw = base;                                   // nr x 16 KiB
  unsigned char* outst = raw + (uint32_t)a.nr * kRawBytes;     // 4 warps x 4 KiB
  float* smean = reinterpret_cast<float*>(outst + kOutBytes);  // D floats (+ padding)
  unsigned char* bsm = outst + kOutBytes + kMeanBytes;         // factor (resident) or slices

  __shared__ __align__(8) uint64_t raw_full[kRawSlotsMax], raw_empty[kRawSlotsMax];
  __shared__ __align__(8) uint64_t a_full[kAStages], a_empty[kAStages];
  __shared__ __align__(8) uint64_t b_full[kBSlotsMax], b_empty[kBSlotsMax];
  __shared__ __align__(8) uint64_t acc_full[kAccMax], acc_empty[kAccMax], fin_bar;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  __shared__ UmmaItem s_items[kMaxItems];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (a.n + kUmmaM - 1) / kUmmaM;
  const int nitems = a.nitems;
  int32_t* status = a.status;

  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kRawSlotsMax; ++i) {
      mbar_init(&raw_full[i], 1);
      mbar_init(&raw_empty[i], kCvtGroupWarps);
    }
    for (int i = 0; i < kAStages; ++i) {
      mbar_init(&a_full[i], kCvtGroupWarps);
      mbar_init(&a_empty[i], 1);
    }
    for (int i = 0; i < kBSlotsMax; ++i) {
      mbar_init(&b_full[i], 1);
      mbar_init(&b_empty[i], 1);
    }
    for (int i = 0; i < kAccMax; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], kEpiWarps);
    }
    mbar_init(&fin_bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  for (int i = tid; i < (int)(kMeanBytes / 4); i += kThreads) smean[i] = i < a.d ? a.mean[i] : 0.0f;
  if (tid < kMaxItems) s_items[tid] = a.items[tid];
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = __shfl_sync(0xffffffffu, s_tmem, 0);
  const uint32_t nacc = (uint32_t)a.nacc, astride = (uint32_t)a.acc_stride;

  if (warp == kTmaWarp) {
    // ------------------------------------------------------------ Z producer
    if (lane == 0) asm volatile("prefetch.tensormap [%0];" ::"l"(&zmap) : "memory");
    const uint32_t nr = (uint32_t)a.nr;
    uint32_t seq = 0, rsl = 0, ruse = 0;  // rsl = seq % nr, ruse = seq / nr
    bool run = true;
    for (int64_t tile = blockIdx.x; run && tile < ntiles; tile += gridDim.x) {
      const int y0 = (int)(tile * kUmmaM);
      for (int k = 0; k < nitems; ++k) {
        if (ruse > 0 && !warp_wait(&raw_empty[rsl], (ruse - 1) & 1u, &s_abort, status)) {
          run = false;
          break;
        }
        expect_tx_el(&raw_full[rsl], kRawBytes);
        tma_2d_el(smem_u32(raw + rsl * kRawBytes), &zmap, (int)s_items[k].x0, y0, &raw_full[rsl]);
        ++seq;
        if (++rsl == nr) {
          rsl = 0;
          ++ruse;
        }
      }
    }
    // let every copy in flight land before the CTA can leave
    for (uint32_t s = 0; s < nr && s < seq; ++s) {
      const uint32_t last = seq - 1 - ((seq - 1 - s) % nr);  // last item that used slot s
      warp_wait(&raw_full[s], (last / nr) & 1u, &s_abort, status);
    }
  } else if (warp == kBWarp) {
    // ------------------------------------------------------------ factor producer
    if (a.resident) {
      // the whole prepared factor, once (pieces of at most 64 KiB)
      expect_tx_el(&b_full[0], a.btotal);
      for (uint32_t off = 0; off < a.btotal; off += 65536u)
        bulk_g2s_el(smem_u32(bsm + off), reinterpret_cast<const unsigned char*>(a.Lp) + off,
                    min(65536u, a.btotal - off), &b_full[0]);
      warp_wait(&b_full[0], 0, &s_abort, status);
    } else {
      const uint32_t nb = (uint32_t)a.nb;
      uint32_t seq = 0, bs = 0, use = 0;
      bool run = true;
      for (int64_t tile = blockIdx.x; run && tile < ntiles; tile += gridDim.x) {
        for (int k = 0; k < nitems; ++k) {
          if (use > 0 && !warp_wait(&b_empty[bs], (use - 1) & 1u, &s_abort, status)) {
            run = false;
            break;
          }
          const UmmaItem& e = s_items[k];
          const unsigned char* src = reinterpret_cast<const unsigned char*>(a.Lp) + e.boff;
          const uint32_t dst = smem_u32(bsm + bs * kBSlotBytes);
          expect_tx_el(&b_full[bs], 2 * e.sl);
          bulk_g2s_el(dst, src, e.sl, &b_full[bs]);
          bulk_g2s_el(dst + e.sl, src + e.part, e.sl, &b_full[bs]);
          ++seq;
          if (++bs == nb) {
            bs = 0;
            ++use;
          }
        }
      }
      for (uint32_t s = 0; s < nb && s < seq; ++s) {
        const uint32_t last = seq - 1 - ((seq - 1 - s) % nb);
        warp_wait(&b_full[s], (last / nb) & 1u, &s_abort, status);
      }
    }
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA issuer
    const bool resident = a.resident != 0;
    const uint32_t nb = resident ? 1u : (uint32_t)a.nb;
    bool run = !resident || warp_wait(&b_full[0], 0, &s_abort, status);
    const uint64_t bres = kDescConst | (uint64_t)(smem_u32(bsm) >> 4);  // resident factor descriptor base
    uint32_t as = 0, ause = 0, bs = 0, buse = 0, abuf = 0, accuse = 0;
    for (int64_t tile = blockIdx.x; run && tile < ntiles; tile += gridDim.x) {
      // unrolled: the item's fields are kernel-parameter reads at constant
      // offsets, i.e. warp-uniform operands for the tensor instructions
#pragma unroll
      for (int k = 0; k < kMaxItems; ++k) {
        if (k >= nitems) break;
        const UmmaItem& e = a.items[k];
        const uint32_t flags = e.flags;
        if ((flags & kItemFirst) && accuse > 0 &&
            !warp_wait(&acc_empty[abuf], (accuse - 1) & 1u, &s_abort, status)) {
          run = false;
          break;
        }
        if (!warp_wait(&a_full[as], ause & 1u, &s_abort, status)) {
          run = false;
          break;
        }
        uint64_t dbh, dbl;
        if (resident) {
          dbh = bres + (e.boff >> 4);
          dbl = dbh + (e.part >> 4);
        } else {
          if (!warp_wait(&b_full[bs], buse & 1u, &s_abort, status)) {
            run = false;
            break;
          }
          dbh = kDescConst | (uint64_t)(smem_u32(bsm + bs * kBSlotBytes) >> 4);
          dbl = dbh + (e.sl >> 4);
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dcol = tmem + abuf * astride + e.dcol;
        const uint32_t ahi = tmem + kACol0 + as * 64u, alo = ahi + 32u;
        const uint32_t idesc = e.idesc;
        const uint32_t first = (flags & kItemFirst) ? 0u : 1u;
        // K step ks: 8 tf32 columns = 8 tensor-memory columns of A and two
        // 128-byte core matrices (+16 in descriptor units) of B
        // (K steps past the last input column multiply zeros: left out)
        const uint32_t nks = e.nks;
        mma_el(dcol, alo, dbh, idesc, first);
        mma_el(dcol, ahi, dbl, idesc, 1u);
        mma_el(dcol, ahi, dbh, idesc, 1u);
#pragma unroll
        for (uint32_t ks = 1; ks < kUmmaKC / 8; ++ks) {
          if (ks < nks) {
            mma_el(dcol, alo + 8u * ks, dbh + 16u * ks, idesc, 1u);
            mma_el(dcol, ahi + 8u * ks, dbl + 16u * ks, idesc, 1u);
            mma_el(dcol, ahi + 8u * ks, dbh + 16u * ks, idesc, 1u);
          }
        }
        commit_el(&a_empty[as]);
        if (++as == kAStages) {
          as = 0;
          ++ause;
        }
        if (!resident) {
          commit_el(&b_empty[bs]);
          if (++bs == nb) {
            bs = 0;
            ++buse;
          }
        }
        if (flags & kItemLast) {
          commit_el(&acc_full[abuf]);
          if (++abuf == nacc) {
            abuf = 0;
            ++accuse;
          }
        }
      }
    }
    // every product issued has finished before the tensor memory is freed
    commit_el(&fin_bar);
    warp_wait(&fin_bar, 0, &s_abort, status);
  } else if (warp >= kCvtWarp0 && warp < kCvtWarp0 + 2 * kCvtGroupWarps) {
    // ------------------------------------------------------------ converters
    // group g (warps 4..7 or 8..11) takes the items with seq % 2 == g; warp w
    // of a group owns samples 32 (w % 4) .. + 31 (its tensor-memory lanes)
    const int quad = warp & 3, grp = (warp - kCvtWarp0) >> 2;
    const int row = 32 * quad + lane;
    const uint32_t lane_addr = (uint32_t)(32 * quad) << 16;
    const uint32_t nr = (uint32_t)a.nr;
    uint32_t seq = 0;
    bool run = true;
    for (int64_t tile = blockIdx.x; run && tile < ntiles; tile += gridDim.x) {
      for (int k = 0; k < nitems; ++k, ++seq) {
        if ((int)(seq & 1u) != grp) continue;
        const uint32_t rsl = seq % nr, as = seq % kAStages, ause = seq / kAStages;
        if (!warp_wait(&raw_full[rsl], (seq / nr) & 1u, &s_abort, status) ||
            (ause > 0 && !warp_wait(&a_empty[as], (ause - 1) & 1u, &s_abort, status))) {
          run = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        // this sample's 32 columns, 16 at a time: 16-byte chunk j of row r is
        // stored at chunk position j ^ (r % 8) (128-byte swizzle)
        const unsigned char* rrow = raw + rsl * kRawBytes + (uint32_t)row * 128u;
        const uint32_t ta = tmem + lane_addr + kACol0 + as * 64u;
        float v[2][16];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 f = *reinterpret_cast<const float4*>(rrow + ((j ^ (row & 7)) << 4));
          v[j >> 2][4 * (j & 3)] = f.x;
          v[j >> 2][4 * (j & 3) + 1] = f.y;
          v[j >> 2][4 * (j & 3) + 2] = f.z;
          v[j >> 2][4 * (j & 3) + 3] = f.w;
        }
        warp_arrive(&raw_empty[rsl]);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          uint32_t h[16], l[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float hf, lf;
            split_tf32(v[hh][j], hf, lf);
            h[j] = __float_as_uint(hf);
            l[j] = __float_as_uint(lf);
          }
          asm volatile(
              "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
                  ta + 16u * hh),
              "r"(h[0]), "r"(h[1]), "r"(h[2]), "r"(h[3]), "r"(h[4]), "r"(h[5]), "r"(h[6]), "r"(h[7]), "r"(h[8]),
              "r"(h[9]), "r"(h[10]), "r"(h[11]), "r"(h[12]), "r"(h[13]), "r"(h[14]), "r"(h[15]));
          asm volatile(
              "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
                  ta + 32u + 16u * hh),
              "r"(l[0]), "r"(l[1]), "r"(l[2]), "r"(l[3]), "r"(l[4]), "r"(l[5]), "r"(l[6]), "r"(l[7]), "r"(l[8]),
              "r"(l[9]), "r"(l[10]), "r"(l[11]), "r"(l[12]), "r"(l[13]), "r"(l[14]), "r"(l[15]));
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        warp_arrive(&a_full[as]);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // group g (warps 0..3 or 15..18) takes the passes with q % 2 == g (the
    // accumulator buffer count is even, so buffer b always has the same
    // group); warp w owns samples 32 (w % 4) .. + 31 of the tile (its
    // tensor-memory lanes).  Per 32-column block: tcgen05.ld (thread =
    // sample), + mean, into a swizzled 32 x 32 staging tile, read back 4 rows
    // x 128 bytes per store instruction (coalesced 16-byte stores).
    const int quad = warp & 3, egrp = warp >= kEpi2Warp0 ? 1 : 0;
    const uint32_t lane_addr = (uint32_t)(32 * quad) << 16;
    unsigned char* stg = outst + (uint32_t)(4 * egrp + quad) * kStageOutBytes;
    const float4* mean4 = reinterpret_cast<const float4*>(smean);
    const int cc = lane & 7;           // 16-byte chunk of a staging row (store phase)
    const int rsub = lane >> 3;        // row within a group of 4 (store phase)
    uint32_t abuf = 0, accuse = 0, q = 0;
    bool run = true;
    for (int64_t tile = blockIdx.x; run && tile < ntiles; tile += gridDim.x) {
      const int64_t y0 = tile * kUmmaM + 32 * quad;
      for (int k = 0; k < nitems; ++k) {
        const UmmaItem& e = s_items[k];
        if (!(e.flags & kItemLast)) continue;
        const uint32_t mybuf = abuf, myuse = accuse;
        const bool mine = (int)(q & 1u) == egrp;
        ++q;
        if (++abuf == nacc) {
          abuf = 0;
          ++accuse;
        }
        if (!mine) continue;
        const int n0 = (int)e.n0, n1 = (int)e.n1;
        if (!warp_wait(&acc_full[mybuf], myuse & 1u, &s_abort, status)) {
          run = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        bool released = false;
        // a warp whose 32 samples all lie past the end has nothing to store
        for (int cb = n0; cb < n1 && y0 < a.n; cb += 32) {
          uint32_t r[32];
          const uint32_t ta = tmem + lane_addr + mybuf * astride + (uint32_t)(cb - n0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
              : "r"(ta));
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
                "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                "=r"(r[30]), "=r"(r[31])
              : "r"(ta + 16u));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (cb + 32 >= n1) {
            // the pass's last columns are in registers: the accumulator is free
            asm volatile("tcgen05.fence::before_thread_sync;");
            warp_arrive(&acc_empty[mybuf]);
            released = true;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float4 mu = mean4[(cb >> 2) + j];
            float4 o;
            o.x = __uint_as_float(r[4 * j]) + mu.x;
            o.y = __uint_as_float(r[4 * j + 1]) + mu.y;
            o.z = __uint_as_float(r[4 * j + 2]) + mu.z;
            o.w = __uint_as_float(r[4 * j + 3]) + mu.w;
            *reinterpret_cast<float4*>(stg + (uint32_t)lane * 128u + ((j ^ (lane & 7)) << 4)) = o;
          }
          __syncwarp();
          if (cb + 4 * cc < a.d) {
            float* xp = a.X + (y0 + rsub) * a.d + cb + 4 * cc;
            const int64_t step = 4 * (int64_t)a.d;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const int rr = 4 * t + rsub;  // row of the staging tile
              const float4 o = *reinterpret_cast<const float4*>(stg + (uint32_t)rr * 128u + ((cc ^ (rr & 7)) << 4));
              if (y0 + rr < a.n) *reinterpret_cast<float4*>(xp) = o;
              xp += step;
            }
          }
          __syncwarp();
        }
        if (!released) {
          asm volatile("tcgen05.fence::before_thread_sync;");
          warp_arrive(&acc_empty[mybuf]);
        }
      }
    }
  }

  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ============================================================================
// WishartGen<float> (not inverse) Bartlett products on tcgen05, dims up to 64
// (MvNormal.h:236-277): per draw j, A_j = strictly-lower normals (column by
// column) + diagonal sqrt(chi^2(df - i)), T_j = L A_j, W_j = T_j T_j^T.
// Draws are stacked along M: a tile holds G = 128 / p draws, p the dim
// rounded up to a power of two (16, 32 or 64), 128 threads, lane (g, i) =
// thread g p + i.
//   1. lane (g, i) writes column i of A_g (its tf32 high and low parts) into
//      tensor memory: row (g, i) of the stacked A^T;
//   2. T^T = A^T L^T: tcgen05.mma, A from tensor memory, B = L (rows of L,
//      K-major, high and low parts resident in shared memory); accumulator
//      row (g, i), column r = T_g[r][i];
//   3. the accumulator is read back (tcgen05.ld) and written transposed into
//      shared memory as S[(g, r)][i] = T_g[r][i], split into tf32 parts,
//      K-major canonical layout;
//   4. S S^T: one M = 128, N = 128 product whose diagonal p x p blocks are
//      the draws' W_g (the cross blocks are not used);
//   5. lane (g, r) reads its draw's block of row (g, r) and stores W_g's
//      column-major elements (coalesced along r).
// 3xTF32 with FP32 accumulation in both products, as the mma.sync form.
namespace {

__device__ __forceinline__ void mma_tf32_ss(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_tf32_ts1(uint32_t dtmem, uint32_t atmem, uint64_t b, uint32_t idesc,
                                             uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "r"(atmem), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit1(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

constexpr int kWishUThreads = 128;

// Wait for an MMA commit by polling mbarrier.test_wait (non-blocking) from
// lane 0 of each warp; bounded like mbar_wait.
__device__ __forceinline__ bool wish_wait(uint64_t* bar, uint32_t parity, volatile int* abort, int32_t* status) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    uint32_t done = 0;
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; ++it) {
      asm volatile(
          "{\n\t.reg .pred p;\n\t"
          "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(smem_u32(bar)), "r"(parity)
          : "memory");
      if (done) break;
      if ((it & 255) == 0) {
        if (it == 0) t0 = gtimer();
        if (*abort) {
          ok = 0;
          break;
        }
        if (gtimer() - t0 > kWaitNs) {
          *abort = 1;
          atomicOr(status, (int)GR_DEV_MMA_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

}  // namespace

__global__ void __launch_bounds__(kWishUThreads)
    k_wishart_umma(const float* __restrict__ normals, const float* __restrict__ chis, const float* __restrict__ chol,
                   float* __restrict__ out, int d, int dp, int64_t samples, int32_t* status) {
  extern __shared__ __align__(1024) unsigned char wu_dyn[];
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)wu_dyn + 1023) & ~(uintptr_t)1023);
  float* Bhi = reinterpret_cast<float*>(base);  // L: dp rows x dp k
  float* Blo = Bhi + dp * dp;
  float* Xhi = Blo + dp * dp;  // A^T of the tile (128 rows x dp k), then S (stacked T)
  float* Xlo = Xhi + 128 * dp;
  float* stage0 = Xlo + 128 * dp;  // the tile's normals (G draws, contiguous in HBM), double buffered
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int G = 128 / dp;
  const uint32_t SBO = (uint32_t)dp * 32;  // bytes between 8-row groups: dp/4 core matrices of 128 bytes
  auto koff = [&](int row, int k) -> uint32_t {
    return ((uint32_t)(row >> 3) * SBO + (uint32_t)(k >> 2) * 128u + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 3) * 4u) >> 2;
  };
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(128u));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // the factor's rows: B[r][k] = L[r][k] (chol column-major), zero outside d x d
  for (int t = tid; t < dp * dp; t += kWishUThreads) {
    const int r = t / dp, k = t % dp;
    const float x = (r < d && k < d) ? chol[(size_t)k * d + r] : 0.0f;
    float hi, lo;
    split_tf32(x, hi, lo);
    Bhi[koff(r, k)] = hi;
    Blo[koff(r, k)] = lo;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  const uint32_t lane_addr = (uint32_t)(32 * warp) << 16;
  // tensor memory (128 columns): S S^T; T^T lives in its first dp columns
  // until the second product overwrites them
  const int g = tid / dp, i = tid % dp;
  const int64_t nper = (int64_t)d * (d - 1) / 2;
  const int64_t ntiles = (samples + G - 1) / G;
  const uint32_t idesc1 = umma_idesc_tf32(128, dp), idesc2 = umma_idesc_tf32(128, 128);
  const uint64_t dsc = kDescConstW(SBO);
  const uint64_t bh = dsc | (uint64_t)(smem_u32(Bhi) >> 4), bl = dsc | (uint64_t)(smem_u32(Blo) >> 4);
  const uint64_t xh = dsc | (uint64_t)(smem_u32(Xhi) >> 4), xl = dsc | (uint64_t)(smem_u32(Xlo) >> 4);
  const int stage_len = (G * (int)nper + 3) & ~3;
  float* stages[2] = {stage0, stage0 + stage_len};
  // a tile's normals into a stage buffer with cp.async (4-byte copies: the
  // tile's start need not be 16-byte aligned); lands while the previous tile
  // is processed
  auto prefetch = [&](int64_t t, float* dst) {
    if (t < ntiles) {
      const int64_t j0 = t * G, nd = (samples - j0 < G ? samples - j0 : G);
      const int cnt = (int)(nd * nper);
      const float* src = normals + j0 * nper;
      for (int q = tid; q < cnt; q += kWishUThreads)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst + q)), "l"(src + q) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  prefetch(blockIdx.x, stages[0]);
  int sb = 0;
  uint32_t phase = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles && !s_abort; tile += gridDim.x) {
    const int64_t j = tile * G + g;
    const bool jok = j < samples;
    const float diag = (jok && i < d) ? sqrtf(chis[(int64_t)i * samples + j]) : 0.0f;
    // ---- 1. this tile's normals (prefetched), the next tile's on their way,
    // then row (g, i) of the stacked A^T = column i of A_g, tf32 parts, into
    // shared memory
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    prefetch(tile + gridDim.x, stages[sb ^ 1]);
    const float* stage = stages[sb];
    sb ^= 1;
    const int nb = g * (int)nper + i * (d - 1) - i * (i - 1) / 2;  // its normals start here in the stage
    for (int k0 = 0; k0 < dp; k0 += 4) {
      float4 h, l;
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = k0 + q;
        v[q] = 0.0f;
        if (jok && i < d && k < d) {
          if (k > i) v[q] = stage[nb + (k - i - 1)];
          else if (k == i) v[q] = diag;
        }
      }
      split_tf32(v[0], h.x, l.x);
      split_tf32(v[1], h.y, l.y);
      split_tf32(v[2], h.z, l.z);
      split_tf32(v[3], h.w, l.w);
      *reinterpret_cast<float4*>(Xhi + koff(tid, k0)) = h;
      *reinterpret_cast<float4*>(Xlo + koff(tid, k0)) = l;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // ---- 2. T^T = A^T L^T
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int ks = 0; ks < dp / 8; ++ks) {
        const uint64_t o = 16u * (uint64_t)ks;
        mma_tf32_ss(tmem, xl + o, bh + o, idesc1, ks > 0 ? 1u : 0u);
        mma_tf32_ss(tmem, xh + o, bl + o, idesc1, 1u);
        mma_tf32_ss(tmem, xh + o, bh + o, idesc1, 1u);
      }
      commit1(&bar);
    }
    if (!wish_wait(&bar, phase, &s_abort, status)) break;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // ---- 3. S[(g, r)][i] = T_g[r][i], split, over A^T (consumed)
    for (int c0 = 0; c0 < dp; c0 += 16) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(tmem + lane_addr + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float hf, lf;
        split_tf32(__uint_as_float(r[q]), hf, lf);
        const uint32_t o = koff(g * dp + c0 + q, i);
        Xhi[o] = hf;
        Xlo[o] = lf;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // ---- 4. S S^T (the diagonal p x p blocks are the draws' W)
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int ks = 0; ks < dp / 8; ++ks) {
        const uint64_t o = 16u * (uint64_t)ks;
        mma_tf32_ss(tmem, xl + o, xh + o, idesc2, ks > 0 ? 1u : 0u);
        mma_tf32_ss(tmem, xh + o, xl + o, idesc2, 1u);
        mma_tf32_ss(tmem, xh + o, xh + o, idesc2, 1u);
      }
      commit1(&bar);
    }
    if (!wish_wait(&bar, phase, &s_abort, status)) break;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // ---- 5. lane (g, r): row (g, r) of its draw's block, W_g[r][s] at column g p + s
    {
      const int r = i;
      const int c0 = dp >= 32 ? (32 * warp / dp) * dp : 32 * warp;  // the warp's first column (warp-uniform)
      const int width = dp >= 32 ? dp : 32;
      float* o = out + j * (int64_t)d * d;
      for (int cc = 0; cc < width; cc += 16) {
        uint32_t v[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(tmem + lane_addr + (uint32_t)(c0 + cc)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int sc = c0 + cc + q - g * dp;  // column within the draw's block
          if (jok && r < d && sc >= 0 && sc < d) o[(int64_t)sc * d + r] = __uint_as_float(v[q]);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
  }
  // copies and products in flight finish before the CTA leaves
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (tid == 0) {
    commit1(&bar);
    mbar_wait(&bar, phase, &s_abort, status);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u));
  }
}

bool wishart_umma_usable(int d, int dtype, int inverse) {
  return dtype == GR_F32 && !inverse && d >= 1 && d <= kWishUmmaMaxDim;
}

cudaError_t launch_wishart_umma(const float* normals, const float* chis, const float* chol, float* out, int d,
                                int64_t samples, int32_t* status, cudaStream_t s) {
  if (d < 1 || d > kWishUmmaMaxDim || samples <= 0) return samples == 0 ? cudaSuccess : cudaErrorInvalidValue;
  int dp = 16;
  while (dp < d) dp <<= 1;
  const int G = 128 / dp;
  // 128 tensor-memory columns per CTA: four CTAs per SM; shared memory is
  // sized so that no more than four are resident (a fifth would wait in
  // tcgen05.alloc), fewer where a CTA needs more
  const size_t stage_len = ((size_t)G * d * (d - 1) / 2 + 3) & ~(size_t)3;
  size_t smem = 1024 + (size_t)(2 * dp * dp + 2 * 128 * dp + 2 * stage_len) * sizeof(float);
  if (smem < 52 * 1024) smem = 52 * 1024;
  int dev = 0, sms = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem + 4096 > (size_t)optin) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_wishart_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // all of the SM's unified L1 / shared memory as shared memory, so that
  // several CTAs fit
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_wishart_umma, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  // resident CTAs per SM from the SM's shared memory (the occupancy API
  // answers 1 for this kernel whatever the size, while the SM holds three at
  // dim 32); tensor memory (512 columns, 128 per CTA) caps it at four
  int sm_smem = 0, reserved = 0;
  cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, k_wishart_umma);
  if (e != cudaSuccess) return e;
  const size_t per_cta = smem + fa.sharedSizeBytes + (size_t)reserved;
  int per = (int)((size_t)sm_smem / per_cta);
  if (per < 1) per = 1;
  if (per > 4) per = 4;
  const int64_t tiles = (samples + G - 1) / G;
  const int64_t cap = (int64_t)sms * per;
  const int64_t grid = tiles < cap ? tiles : cap;
  k_wishart_umma<<<(unsigned)grid, kWishUThreads, smem, s>>>(normals, chis, chol, out, d, dp, samples, status);
  return cudaGetLastError();
}

int umma_padded_dim(int d) { return (d + 15) / 16 * 16; }
int umma_chunks(int d) { return (d + kUmmaKC - 1) / kUmmaKC; }

size_t umma_prep_floats(int d, int tri) {
  const int D = umma_padded_dim(d), C = umma_chunks(d);
  return (size_t)chunk_off(C, D, tri) / 4;
}

cudaError_t launch_prep_lt_umma(const double* L, float* out, int d, int tri, cudaStream_t s) {
  const int D = umma_padded_dim(d), C = umma_chunks(d);
  k_prep_lt_umma<<<256, 256, 0, s>>>(L, out, d, D, C, tri);
  return cudaGetLastError();
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// X viewed as n rows of d floats; box of 128 rows x 32 columns, 128-byte swizzle
bool encode_rows(CUtensorMap* m, float* X, int d, int64_t n) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)d, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)d * 4};
  const cuuint32_t box[2] = {(cuuint32_t)kUmmaKC, (cuuint32_t)kUmmaM};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, X, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the items of one tile, in the order every role walks them: pass p over
// outputs [128 p, min(D, 128 p + 128)), chunks c whose rows reach the pass
int build_items(UmmaItem* items, int d, int D, int C, int tri) {
  const int P = (D + kUmmaPassN - 1) / kUmmaPassN;
  int k = 0;
  for (int p = 0; p < P; ++p) {
    const int n0 = kUmmaPassN * p, n1 = D < n0 + kUmmaPassN ? D : n0 + kUmmaPassN;
    const int kfirst = k;
    for (int c = 0; c < C; ++c) {
      const int r0 = chunk_row0(c, tri);
      if (r0 >= n1) break;
      const int rs = r0 > n0 ? r0 : n0;
      UmmaItem& e = items[k++];
      e.x0 = (uint32_t)(kUmmaKC * c);
      e.boff = chunk_off(c, D, tri) + (uint32_t)(rs - r0) * 128u;
      e.part = (uint32_t)(D - r0) * 128u;
      e.sl = (uint32_t)(n1 - rs) * 128u;
      e.idesc = umma_idesc_tf32(kUmmaM, n1 - rs);
      e.dcol = (uint32_t)(rs - n0);
      e.n0 = (uint32_t)n0;
      e.n1 = (uint32_t)n1;
      e.flags = 0;
      const int kvalid = d - kUmmaKC * c < kUmmaKC ? d - kUmmaKC * c : kUmmaKC;
      e.nks = (uint32_t)((kvalid + 7) / 8);
    }
    items[kfirst].flags |= kItemFirst;
    items[k - 1].flags |= kItemLast;
  }
  return k;
}

}  // namespace

bool umma_usable(int d, const void* X, int64_t n) {
  return d >= 4 && d <= kUmmaMaxDim && (d & 3) == 0 && ((uintptr_t)X & 15) == 0 && n > 0 && n < (1ll << 31) &&
         encode_fn() != nullptr;
}

cudaError_t launch_mvn_umma(const float* Lp, int tri, const float* mean, float* X, int d, int64_t n, int32_t* status,
                            cudaStream_t s) {
  if (!umma_usable(d, X, n)) return cudaErrorInvalidValue;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  int sms = 0, optin = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  optin -= 4096;  // the kernel's static shared memory (barriers, item table) comes out of the same budget
  MvnUmmaArgs a;
  a.Lp = Lp;
  a.mean = mean;
  a.X = X;
  a.n = n;
  a.status = status;
  a.d = d;
  const int D = umma_padded_dim(d), C = umma_chunks(d);
  tri = tri ? 1 : 0;
  a.btotal = chunk_off(C, D, tri);
  a.nitems = build_items(a.items, d, D, C, tri);
  // shared memory: the raw Z ring (4 .. 12 slots of 16 KiB), the epilogue's
  // staging tiles, the mean, and the factor (whole, or a ring of slices)
  const size_t fixed = 1024 + (size_t)kOutBytes + kMeanBytes;
  const size_t ring_min = (size_t)kRawSlotsMin * kRawBytes;
  a.resident = fixed + ring_min + a.btotal <= (size_t)optin ? 1 : 0;
  size_t bbytes = a.btotal;
  a.nb = 0;
  if (!a.resident) {
    a.nb = (int)(((size_t)optin - fixed - ring_min) / kBSlotBytes);
    if (a.nb > kBSlotsMax) a.nb = kBSlotsMax;
    bbytes = (size_t)a.nb * kBSlotBytes;
    if (a.nb < 2) return cudaErrorInvalidValue;
  }
  size_t nr = ((size_t)optin - fixed - bbytes) / kRawBytes;
  if (nr > (size_t)kRawSlotsMax) nr = kRawSlotsMax;
  // even: raw slot s then always serves items of one parity, i.e. one
  // converter group, which waits on its phases in order (a parity wait must
  // never run two phases ahead)
  nr &= ~(size_t)1;
  a.nr = (int)nr;
  // accumulator buffers: the pass width rounded up to 32 columns (the
  // epilogue reads 32-column blocks), as many as fit in 256 columns (<= 8)
  const int W = D < kUmmaPassN ? D : kUmmaPassN;
  a.acc_stride = (W + 31) / 32 * 32;
  a.nacc = 256 / a.acc_stride;
  if (a.nacc > kAccMax) a.nacc = kAccMax;
  a.nacc &= ~1;  // even: buffer b always belongs to the same epilogue group
  size_t smem = fixed + bbytes + nr * kRawBytes;
  // at least 120 KiB: one CTA per SM, so that it owns the 512 tensor-memory columns
  if (smem < 120 * 1024) smem = 120 * 1024;
  if (smem > (size_t)optin) return cudaErrorInvalidValue;
  static bool attr[64] = {};
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_mvn_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  CUtensorMap zmap;
  if (!encode_rows(&zmap, X, d, n)) return cudaErrorInvalidValue;
  const int64_t tiles = (n + kUmmaM - 1) / kUmmaM;
  const int64_t grid = tiles < (int64_t)sms ? tiles : (int64_t)sms;
  k_mvn_umma<<<(unsigned)grid, kThreads, smem, s>>>(zmap, a);
  return cudaGetLastError();
}

}  // namespace gr
