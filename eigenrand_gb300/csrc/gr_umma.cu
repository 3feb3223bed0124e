// X = L Z + mean for MvNormalGen<float> on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// The product is computed as X^T = Z^T L^T: the samples are the M dimension
// (Z holds sample j's dim normals contiguously, EigenRand/MvDists/MvNormal.h:
// 103-108), the output dimension is N and the input dimension K.  A CTA owns
// 128 samples; K runs in chunks of 32.  Per chunk:
//   - every thread loads its sample's 32 values of Z, splits them into tf32
//     high and low parts (cvt.rna.tf32) and stores both into shared memory in
//     the no-swizzle K-major canonical layout (core matrices of 8 rows x 16
//     bytes; K-adjacent core matrices 128 bytes apart, 8-row groups 1024
//     bytes apart);
//   - the factor's chunk, prepared once per generator in the same layout and
//     split the same way, is copied in;
//   - one thread issues, per K step of 8, three tcgen05.mma.kind::tf32 (low x
//     high, high x low, high x high: 3xTF32 with FP32 accumulation) into a
//     128 x D accumulator in tensor memory and commits them to an mbarrier
//     that every thread waits on (a bounded wait: on timeout the kernel
//     records an error bit and stops).
// The epilogue reads the accumulator back with tcgen05.ld (warp w reads
// tensor-memory lanes 32w .. 32w + 31, one sample per thread), adds the mean
// and writes X over Z (a CTA has read all of its samples' Z before it
// writes).  Dimensions up to 256 (N = D, the dimension rounded up to 16).
#include <cuda_runtime.h>

#include <cstdint>

#include "gr_internal.h"
#include "gr_mv.cuh"

namespace gr {

namespace {

constexpr int kUmmaM = 128;   // samples per CTA (tensor-memory lanes)
constexpr int kUmmaKC = 32;   // K per chunk (128 bytes of float per row)
constexpr int kUmmaThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 26;  // mbarrier polls before the kernel gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
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

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// true once the phase with this parity has completed; gives up after kWaitLimit polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
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

}  // namespace

// The factor as the B operand: chunk c, part h (0 high, 1 low), row n, column
// k of the chunk at ((c * 2 + h) * D * 32) floats + kmaj_off(n, k) / 4.
// B[n][k] = L[n][32 c + k] (L column-major FP64), zero outside dim x dim.
__global__ void k_prep_lt_umma(const double* L, float* out, int d, int D, int nchunks) {
  const int64_t total = (int64_t)nchunks * D * kUmmaKC;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / ((int64_t)D * kUmmaKC));
    const int rem = (int)(t % ((int64_t)D * kUmmaKC));
    const int n = rem / kUmmaKC, k = rem % kUmmaKC;
    const int kk = c * kUmmaKC + k;
    const float x = (n < d && kk < d) ? (float)L[(size_t)kk * d + n] : 0.0f;
    float hi, lo;
    split_tf32(x, hi, lo);
    float* base = out + (size_t)c * 2 * D * kUmmaKC;
    base[kmaj_off(n, k) / 4] = hi;
    base[(size_t)D * kUmmaKC + kmaj_off(n, k) / 4] = lo;
  }
}

__global__ void __launch_bounds__(kUmmaThreads) k_mvn_umma(const float* __restrict__ Lp, const float* __restrict__ mean,
                                                          float* X, int d, int D, int nchunks, uint32_t tcols,
                                                          int64_t n, int32_t* status) {
  extern __shared__ __align__(1024) unsigned char um_dyn[];
  // 1024-byte aligned operand tiles
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)um_dyn + 1023) & ~(uintptr_t)1023);
  float* Ahi = reinterpret_cast<float*>(base);
  float* Alo = Ahi + kUmmaM * kUmmaKC;
  float* Bhi = Alo + kUmmaM * kUmmaKC;
  float* Blo = Bhi + D * kUmmaKC;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(tcols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = umma_idesc_tf32(kUmmaM, D);
  uint32_t phase = 0;
  const int64_t ntiles = (n + kUmmaM - 1) / kUmmaM;
  const bool vec = (d & 3) == 0;

  for (int64_t tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x) {
    const int64_t m = tile * kUmmaM + tid;  // this thread's sample
    const bool mval = m < n;
    for (int c = 0; c < nchunks; ++c) {
      // ---- A: this sample's 32 values of the chunk, split into tf32 parts
      const int k0 = c * kUmmaKC;
#pragma unroll
      for (int q = 0; q < kUmmaKC / 4; ++q) {
        float v[4];
        const int kk = k0 + 4 * q;
        if (mval && vec && kk + 3 < d) {
          const float4 f = *reinterpret_cast<const float4*>(X + m * d + kk);
          v[0] = f.x;
          v[1] = f.y;
          v[2] = f.z;
          v[3] = f.w;
        } else {
#pragma unroll
          for (int j = 0; j < 4; ++j) v[j] = (mval && kk + j < d) ? X[m * d + kk + j] : 0.0f;
        }
        float4 h, l;
        split_tf32(v[0], h.x, l.x);
        split_tf32(v[1], h.y, l.y);
        split_tf32(v[2], h.z, l.z);
        split_tf32(v[3], h.w, l.w);
        const uint32_t off = kmaj_off(tid, 4 * q) / 4;
        *reinterpret_cast<float4*>(Ahi + off) = h;
        *reinterpret_cast<float4*>(Alo + off) = l;
      }
      // ---- B: the factor's chunk (both parts), a straight copy
      const float4* src = reinterpret_cast<const float4*>(Lp + (size_t)c * 2 * D * kUmmaKC);
      float4* dst = reinterpret_cast<float4*>(Bhi);  // Bhi and Blo are adjacent
      for (int i = tid; i < 2 * D * kUmmaKC / 4; i += kUmmaThreads) dst[i] = __ldg(src + i);
      // the generic-proxy writes become visible to the tensor cores' reads
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo), bh = smem_u32(Bhi), bl = smem_u32(Blo);
#pragma unroll
        for (int ks = 0; ks < kUmmaKC / 8; ++ks) {
          const uint32_t ko = (uint32_t)ks * 256;  // two 128-byte core matrices per K step of 8
          const uint64_t dah = umma_desc(ah + ko, 128, 1024), dal = umma_desc(al + ko, 128, 1024);
          const uint64_t dbh = umma_desc(bh + ko, 128, 1024), dbl = umma_desc(bl + ko, 128, 1024);
          const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
          mma_tf32(tmem, dal, dbh, idesc, acc0);
          mma_tf32(tmem, dah, dbl, idesc, 1u);
          mma_tf32(tmem, dah, dbh, idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&s_bar))
                     : "memory");
      }
      // the products have read the operands (and written the accumulator)
      if (!mbar_wait(&s_bar, phase)) {
        atomicOr(status, (int)GR_DEV_MMA_TIMEOUT);
        s_fail = 1;
      }
      phase ^= 1;
      __syncthreads();
      if (s_fail) break;
    }
    if (s_fail) break;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // ---- epilogue: sample `m` is tensor-memory lane tid (warp w reads lanes 32w ..)
    for (int cb = 0; cb < D / 16; ++cb) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cb * 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (mval) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = cb * 16 + j;
          if (col < d) X[m * d + col] = __uint_as_float(r[j]) + __ldg(mean + col);
        }
      }
    }
    (void)lane;
    // the next tile's first products overwrite the accumulator
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  // after a timed-out wait, give the products in flight one more bounded
  // wait before the tensor memory is freed
  if (s_fail && tid == 0) mbar_wait(&s_bar, phase ^ 1u);
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols));
}

int umma_padded_dim(int d) { return (d + 15) / 16 * 16; }
int umma_chunks(int d) { return (d + kUmmaKC - 1) / kUmmaKC; }

cudaError_t launch_prep_lt_umma(const double* L, float* out, int d, cudaStream_t s) {
  const int D = umma_padded_dim(d), C = umma_chunks(d);
  k_prep_lt_umma<<<256, 256, 0, s>>>(L, out, d, D, C);
  return cudaGetLastError();
}

static size_t umma_smem(int D) {
  return 1024 + (size_t)2 * kUmmaM * kUmmaKC * 4 + (size_t)2 * D * kUmmaKC * 4;
}

cudaError_t launch_mvn_umma(const float* Lp, const float* mean, float* X, int d, int64_t n, int32_t* status,
                            cudaStream_t s) {
  if (d < 1 || d > kUmmaMaxDim) return cudaErrorInvalidValue;
  if (n <= 0) return cudaSuccess;
  const int D = umma_padded_dim(d), C = umma_chunks(d);
  uint32_t tcols = 32;
  while ((int)tcols < D) tcols <<= 1;
  const size_t smem = umma_smem(D);
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(k_mvn_umma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)umma_smem(kUmmaMaxDim));
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mvn_umma, kUmmaThreads, smem);
  // every resident CTA holds tcols tensor-memory columns of the SM's 512
  per = per < 1 ? 1 : per;
  if ((int64_t)per * tcols > 512) per = (int)(512 / tcols);
  const int64_t tiles = (n + kUmmaM - 1) / kUmmaM;
  const int64_t grid = tiles < (int64_t)sms * per ? tiles : (int64_t)sms * per;
  k_mvn_umma<<<(unsigned)grid, kUmmaThreads, smem, s>>>(Lp, mean, X, d, D, C, tcols, n, status);
  return cudaGetLastError();
}

}  // namespace gr
