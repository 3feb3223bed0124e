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
//   warp 12 (one thread)  TMA: the tile's Z chunk (32 columns x 128 samples,
//                         128-byte swizzle) into a ring of raw slots; the
//                         factor's chunk slice into shared memory (once per
//                         CTA when the whole prepared factor fits, else per
//                         item into a ring of slices);
//   warps 4..11           read a raw slot (row = sample, conflict-free thanks
//                         to the swizzle), split, and tcgen05.st the high and
//                         low parts into an A stage in tensor memory;
//   warp 13 (one thread)  tcgen05.mma, A from tensor memory, B (the factor)
//                         from shared memory, into an accumulator in tensor
//                         memory; tcgen05.commit frees the stages and
//                         publishes finished accumulators;
//   warps 0..3            epilogue: tcgen05.ld (warp w owns lanes 32w..),
//                         + mean, into a swizzled staging tile, TMA store.
// Tensor memory (512 columns): two accumulators of 128 columns (double
// buffered, so one tile's epilogue overlaps the next tile's products) and four
// A stages of 64 columns (32 high + 32 low).
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

constexpr int kUmmaM = 128;   // samples per tile (tensor-memory lanes)
constexpr int kUmmaKC = 32;   // K per chunk (one 128-byte swizzle row of float)
constexpr int kUmmaPassN = 128;  // output columns per pass (accumulator width)
constexpr int kRawSlots = 4;
constexpr int kAStages = 4;
constexpr int kBSlotsMax = 4;
constexpr int kThreads = 448;  // 14 warps
constexpr int kEpiWarps = 4, kCvtWarp0 = 4, kCvtWarps = 8, kTmaWarp = 12, kMmaWarp = 13;
constexpr uint32_t kRawBytes = kUmmaM * kUmmaKC * 4;              // 16 KiB
constexpr uint32_t kBSlotBytes = kUmmaPassN * kUmmaKC * 4 * 2;     // 32 KiB (high + low)
constexpr uint32_t kStageOutBytes = 32 * 128;                      // 32 rows x 32 floats
constexpr uint32_t kOutBytes = kEpiWarps * 2 * kStageOutBytes;     // 32 KiB
constexpr uint32_t kMeanBytes = 1024 + 128;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kAccCol0 = 0, kACol0 = 2 * kUmmaPassN;  // A stage s at kACol0 + 64 s
constexpr unsigned long long kWaitNs = 2000000000ull;      // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension
// byte offset (K direction for K-major) and stride-dimension byte offset (the
// next 8-row group), all in 16-byte units; version 1; no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor: FP32 accumulator, tf32 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
  return (1u << 4)                      // D format: F32
         | (2u << 7)                    // A format: TF32
         | (2u << 10)                   // B format: TF32
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

// D[tmem] (+)= A[tmem] * B[smem]^T
__device__ __forceinline__ void mma_tf32_ts(uint32_t dtmem, uint32_t atmem, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "r"(atmem), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort, int32_t* status) {
  if (mbar_try(bar, parity)) return true;
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

// one unit of work: tile t's chunk c for pass p (outputs [n0, n1))
struct Item {
  int c, rs, n0, n1;  // rs: first output row the chunk contributes to in this pass
};

struct ItemIter {
  int C, D, P, tri;
  int64_t tile, ntiles, tstep;
  int p, c;
  __device__ bool valid() const { return tile < ntiles; }
  __device__ Item get() const {
    Item it;
    it.c = c;
    it.n0 = kUmmaPassN * p;
    it.n1 = min(D, it.n0 + kUmmaPassN);
    it.rs = max(it.n0, chunk_row0(c, tri));
    return it;
  }
  __device__ bool first_of_pass() const { return c == 0; }
  // advance; returns true when the item just left was the last of its pass
  __device__ bool next() {
    const int n1 = min(D, kUmmaPassN * p + kUmmaPassN);
    ++c;
    if (c < C && (!tri || kUmmaKC * c < n1)) return false;
    c = 0;
    if (++p >= P) {
      p = 0;
      tile += tstep;
    }
    return true;
  }
};

__device__ __forceinline__ ItemIter make_iter(int C, int D, int tri, int64_t ntiles) {
  ItemIter it;
  it.C = C;
  it.D = D;
  it.P = (D + kUmmaPassN - 1) / kUmmaPassN;
  it.tri = tri;
  it.tile = blockIdx.x;
  it.ntiles = ntiles;
  it.tstep = gridDim.x;
  it.p = 0;
  it.c = 0;
  return it;
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

struct MvnUmmaArgs {
  const float* Lp;
  const float* mean;
  int64_t n;
  int32_t* status;
  int d, D, C, tri;
  int resident;  // the whole prepared factor sits in shared memory
  int nb;        // slice slots when it does not
  uint32_t btotal;
};

__global__ void __launch_bounds__(kThreads, 1)
    k_mvn_umma(const __grid_constant__ CUtensorMap zmap, const __grid_constant__ CUtensorMap xmap,
               const MvnUmmaArgs a) {
  extern __shared__ __align__(1024) unsigned char um_dyn[];
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)um_dyn + 1023) & ~(uintptr_t)1023);
  unsigned char* raw = base;                                   // kRawSlots x 16 KiB
  unsigned char* outst = raw + kRawSlots * kRawBytes;          // 4 warps x 2 x 4 KiB
  float* smean = reinterpret_cast<float*>(outst + kOutBytes);  // D floats (+ padding)
  unsigned char* bsm = outst + kOutBytes + kMeanBytes;         // factor (resident) or slices

  __shared__ __align__(8) uint64_t raw_full[kRawSlots], raw_empty[kRawSlots];
  __shared__ __align__(8) uint64_t a_full[kAStages], a_empty[kAStages];
  __shared__ __align__(8) uint64_t b_full[kBSlotsMax], b_empty[kBSlotsMax];
  __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], fin_bar;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t ntiles = (a.n + kUmmaM - 1) / kUmmaM;
  int32_t* status = a.status;

  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kRawSlots; ++i) {
      mbar_init(&raw_full[i], 1);
      mbar_init(&raw_empty[i], kCvtWarps * 32);
    }
    for (int i = 0; i < kAStages; ++i) {
      mbar_init(&a_full[i], kCvtWarps * 32);
      mbar_init(&a_empty[i], 1);
    }
    for (int i = 0; i < kBSlotsMax; ++i) {
      mbar_init(&b_full[i], 1);
      mbar_init(&b_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], kEpiWarps * 32);
    }
    mbar_init(&fin_bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  for (int i = tid; i < (int)(kMeanBytes / 4); i += kThreads) smean[i] = i < a.d ? a.mean[i] : 0.0f;
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;

  if (warp == kTmaWarp) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&zmap) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(&xmap) : "memory");
      if (a.resident) {
        // the whole prepared factor, once (pieces of at most 64 KiB)
        mbar_expect_tx(&b_full[0], a.btotal);
        for (uint32_t off = 0; off < a.btotal; off += 65536u) {
          const uint32_t sz = min(65536u, a.btotal - off);
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                  smem_u32(bsm + off)),
              "l"(reinterpret_cast<const unsigned char*>(a.Lp) + off), "r"(sz), "r"(smem_u32(&b_full[0]))
              : "memory");
        }
      }
      ItemIter it = make_iter(a.C, a.D, a.tri, ntiles);
      uint32_t seq = 0;
      while (it.valid() && !s_abort) {
        const Item x = it.get();
        // both slots free before either copy is issued
        const int bs = a.resident ? 0 : (int)(seq % (uint32_t)a.nb);
        if (!a.resident) {
          const uint32_t use = seq / (uint32_t)a.nb;
          if (use > 0 && !mbar_wait(&b_empty[bs], (use - 1) & 1u, &s_abort, status)) break;
        }
        const int rsl = (int)(seq % kRawSlots);
        const uint32_t ruse = seq / kRawSlots;
        if (ruse > 0 && !mbar_wait(&raw_empty[rsl], (ruse - 1) & 1u, &s_abort, status)) break;
        if (!a.resident) {
          const int r0 = chunk_row0(x.c, a.tri);
          const uint32_t part = (uint32_t)(a.D - r0) * 128u;   // bytes per part of the chunk
          const uint32_t sl = (uint32_t)(x.n1 - x.rs) * 128u;  // bytes per part of the slice
          const unsigned char* src =
              reinterpret_cast<const unsigned char*>(a.Lp) + chunk_off(x.c, a.D, a.tri) + (uint32_t)(x.rs - r0) * 128u;
          unsigned char* dst = bsm + (uint32_t)bs * kBSlotBytes;
          mbar_expect_tx(&b_full[bs], 2 * sl);
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                  smem_u32(dst)),
              "l"(src), "r"(sl), "r"(smem_u32(&b_full[bs]))
              : "memory");
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                  smem_u32(dst + sl)),
              "l"(src + part), "r"(sl), "r"(smem_u32(&b_full[bs]))
              : "memory");
        }
        mbar_expect_tx(&raw_full[rsl], kRawBytes);
        const int x0 = kUmmaKC * x.c;
        const int y0 = (int)(it.tile * kUmmaM);
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
            "[%4];" ::"r"(smem_u32(raw + (uint32_t)rsl * kRawBytes)),
            "l"(&zmap), "r"(x0), "r"(y0), "r"(smem_u32(&raw_full[rsl]))
            : "memory");
        ++seq;
        it.next();
      }
      // let every copy in flight land before the CTA can leave
      for (uint32_t s = 0; s < kRawSlots && s < seq; ++s) {
        const uint32_t last = seq - 1 - ((seq - 1 - s) % kRawSlots);  // last item that used slot s
        mbar_wait(&raw_full[s], (last / kRawSlots) & 1u, &s_abort, status);
      }
      if (!a.resident)
        for (uint32_t s = 0; s < (uint32_t)a.nb && s < seq; ++s) {
          const uint32_t last = seq - 1 - ((seq - 1 - s) % (uint32_t)a.nb);
          mbar_wait(&b_full[s], (last / (uint32_t)a.nb) & 1u, &s_abort, status);
        }
      else
        mbar_wait(&b_full[0], 0, &s_abort, status);
    }
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool ok = !a.resident || mbar_wait(&b_full[0], 0, &s_abort, status);
      ItemIter it = make_iter(a.C, a.D, a.tri, ntiles);
      uint32_t seq = 0, q = 0;  // q: passes started
      while (ok && it.valid() && !s_abort) {
        const Item x = it.get();
        const uint32_t abuf = q & 1u;
        if (it.first_of_pass()) {
          const uint32_t use = q >> 1;
          if (use > 0 && !mbar_wait(&acc_empty[abuf], (use - 1) & 1u, &s_abort, status)) break;
          asm volatile("tcgen05.fence::after_thread_sync;");
        }
        const int as = (int)(seq % kAStages);
        if (!mbar_wait(&a_full[as], (seq / kAStages) & 1u, &s_abort, status)) break;
        int bs = 0;
        uint32_t bhi, blo;
        const uint32_t sl = (uint32_t)(x.n1 - x.rs) * 128u;
        if (a.resident) {
          const int r0 = chunk_row0(x.c, a.tri);
          const uint32_t part = (uint32_t)(a.D - r0) * 128u;
          bhi = smem_u32(bsm) + chunk_off(x.c, a.D, a.tri) + (uint32_t)(x.rs - r0) * 128u;
          blo = bhi + part;
        } else {
          bs = (int)(seq % (uint32_t)a.nb);
          if (!mbar_wait(&b_full[bs], (seq / (uint32_t)a.nb) & 1u, &s_abort, status)) break;
          bhi = smem_u32(bsm + (uint32_t)bs * kBSlotBytes);
          blo = bhi + sl;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t idesc = umma_idesc_tf32(kUmmaM, x.n1 - x.rs);
        const uint32_t dcol = tmem + kAccCol0 + abuf * kUmmaPassN + (uint32_t)(x.rs - x.n0);
        const uint32_t ahi = tmem + kACol0 + (uint32_t)as * 64u, alo = ahi + 32u;
        const bool first = it.first_of_pass();
#pragma unroll
        for (int ks = 0; ks < kUmmaKC / 8; ++ks) {
          const uint32_t ko = (uint32_t)ks * 256;  // two 128-byte core matrices per K step of 8
          const uint64_t dbh = umma_desc(bhi + ko, 128, 1024), dbl = umma_desc(blo + ko, 128, 1024);
          mma_tf32_ts(dcol, alo + 8u * ks, dbh, idesc, (first && ks == 0) ? 0u : 1u);
          mma_tf32_ts(dcol, ahi + 8u * ks, dbl, idesc, 1u);
          mma_tf32_ts(dcol, ahi + 8u * ks, dbh, idesc, 1u);
        }
        mma_commit(&a_empty[as]);
        if (!a.resident) mma_commit(&b_empty[bs]);
        ++seq;
        if (it.next()) {
          mma_commit(&acc_full[abuf]);
          ++q;
        }
      }
      // every product issued has finished before the tensor memory is freed
      mma_commit(&fin_bar);
      mbar_wait(&fin_bar, 0, &s_abort, status);
    }
  } else if (warp >= kCvtWarp0) {
    // ------------------------------------------------------------ converters
    const int quad = warp & 3, half = (warp - kCvtWarp0) >> 2;
    const int row = 32 * quad + lane;  // sample within the tile = tensor-memory lane
    const uint32_t lane_addr = (uint32_t)(32 * quad) << 16;
    ItemIter it = make_iter(a.C, a.D, a.tri, ntiles);
    uint32_t seq = 0;
    while (it.valid() && !s_abort) {
      const int rsl = (int)(seq % kRawSlots);
      if (!mbar_wait(&raw_full[rsl], (seq / kRawSlots) & 1u, &s_abort, status)) break;
      const int as = (int)(seq % kAStages);
      const uint32_t ause = seq / kAStages;
      if (ause > 0 && !mbar_wait(&a_empty[as], (ause - 1) & 1u, &s_abort, status)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      // 16 columns of this sample's row: 16-byte chunks 4 half .. 4 half + 3,
      // chunk j of row r stored at chunk position j ^ (r % 8) (128-byte swizzle)
      const unsigned char* rrow = raw + (uint32_t)rsl * kRawBytes + (uint32_t)row * 128u;
      float v[16];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float4 f = *reinterpret_cast<const float4*>(rrow + (((4 * half + j) ^ (row & 7)) << 4));
        v[4 * j] = f.x;
        v[4 * j + 1] = f.y;
        v[4 * j + 2] = f.z;
        v[4 * j + 3] = f.w;
      }
      mbar_arrive(&raw_empty[rsl]);
      uint32_t h[16], l[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float hf, lf;
        split_tf32(v[j], hf, lf);
        h[j] = __float_as_uint(hf);
        l[j] = __float_as_uint(lf);
      }
      const uint32_t ta = tmem + lane_addr + kACol0 + (uint32_t)as * 64u + 16u * half;
      asm volatile(
          "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
              ta),
          "r"(h[0]), "r"(h[1]), "r"(h[2]), "r"(h[3]), "r"(h[4]), "r"(h[5]), "r"(h[6]), "r"(h[7]), "r"(h[8]),
          "r"(h[9]), "r"(h[10]), "r"(h[11]), "r"(h[12]), "r"(h[13]), "r"(h[14]), "r"(h[15]));
      asm volatile(
          "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
              ta + 32u),
          "r"(l[0]), "r"(l[1]), "r"(l[2]), "r"(l[3]), "r"(l[4]), "r"(l[5]), "r"(l[6]), "r"(l[7]), "r"(l[8]),
          "r"(l[9]), "r"(l[10]), "r"(l[11]), "r"(l[12]), "r"(l[13]), "r"(l[14]), "r"(l[15]));
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(&a_full[as]);
      ++seq;
      it.next();
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const uint32_t lane_addr = (uint32_t)(32 * warp) << 16;
    unsigned char* st0 = outst + (uint32_t)warp * 2 * kStageOutBytes;
    ItemIter it = make_iter(a.C, a.D, a.tri, ntiles);
    uint32_t q = 0, nst = 0;
    while (it.valid() && !s_abort) {
      const Item x = it.get();
      const int64_t tile = it.tile;
      const uint32_t abuf = q & 1u;
      if (!mbar_wait(&acc_full[abuf], (q >> 1) & 1u, &s_abort, status)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int64_t y0 = tile * kUmmaM + 32 * warp;
      // a warp whose 32 samples all lie past the end has nothing to store
      for (int cb = x.n0; cb < x.n1 && y0 < a.n; cb += 32) {
        uint32_t r[32];
        const uint32_t ta = tmem + lane_addr + kAccCol0 + abuf * kUmmaPassN + (uint32_t)(cb - x.n0);
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
        // staging tile nst & 1: wait until the store that last read it is done
        unsigned char* stg = st0 + (nst & 1u) * kStageOutBytes;
        if (lane == 0 && nst >= 2) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float4 o;
          o.x = __uint_as_float(r[4 * j]) + smean[cb + 4 * j];
          o.y = __uint_as_float(r[4 * j + 1]) + smean[cb + 4 * j + 1];
          o.z = __uint_as_float(r[4 * j + 2]) + smean[cb + 4 * j + 2];
          o.w = __uint_as_float(r[4 * j + 3]) + smean[cb + 4 * j + 3];
          *reinterpret_cast<float4*>(stg + (uint32_t)lane * 128u + ((j ^ (lane & 7)) << 4)) = o;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          asm volatile(
              "cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(&xmap),
              "r"(cb), "r"((int)y0), "r"(smem_u32(stg))
              : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
        ++nst;
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(&acc_empty[abuf]);
      ++q;
      // skip to the next pass
      while (!it.next()) {
      }
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    __syncwarp();
  }

  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
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

// X viewed as n rows of d floats; box of `rows` rows x 32 columns, 128-byte swizzle
bool encode_rows(CUtensorMap* m, float* X, int d, int64_t n, uint32_t rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)d, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)d * 4};
  const cuuint32_t box[2] = {(cuuint32_t)kUmmaKC, rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, X, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
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
  optin -= 2048;  // the kernel's static shared memory (barriers) comes out of the same budget
  MvnUmmaArgs a;
  a.Lp = Lp;
  a.mean = mean;
  a.n = n;
  a.status = status;
  a.d = d;
  a.D = umma_padded_dim(d);
  a.C = umma_chunks(d);
  a.tri = tri ? 1 : 0;
  a.btotal = chunk_off(a.C, a.D, a.tri);
  const size_t fixed = 1024 + (size_t)kRawSlots * kRawBytes + kOutBytes + kMeanBytes;
  a.resident = fixed + a.btotal <= (size_t)optin ? 1 : 0;
  a.nb = 0;
  size_t smem = fixed + a.btotal;
  if (!a.resident) {
    a.nb = (int)(((size_t)optin - fixed) / kBSlotBytes);
    if (a.nb > kBSlotsMax) a.nb = kBSlotsMax;
    if (a.nb < 2) return cudaErrorInvalidValue;
    smem = fixed + (size_t)a.nb * kBSlotBytes;
  }
  // at least 120 KiB: one CTA per SM, so that it owns the 512 tensor-memory columns
  if (smem < 120 * 1024) smem = 120 * 1024;
  if (smem > (size_t)optin) return cudaErrorInvalidValue;
  static bool attr[64] = {};
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_mvn_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  CUtensorMap zmap, xmap;
  if (!encode_rows(&zmap, X, d, n, kUmmaM) || !encode_rows(&xmap, X, d, n, 32)) return cudaErrorInvalidValue;
  const int64_t tiles = (n + kUmmaM - 1) / kUmmaM;
  const int64_t grid = tiles < (int64_t)sms ? tiles : (int64_t)sms;
  k_mvn_umma<<<(unsigned)grid, kThreads, smem, s>>>(zmap, xmap, a);
  return cudaGetLastError();
}

}  // namespace gr
