// TruncMvNormalGen::generate(urng, samples) (EigenRand/MvDists/
// TruncMvNormal.h:171-209): every column is an independent Gibbs chain
// started at clamp(mean, lower, upper); a sweep updates component i of every
// chain from the truncated normal of its conditional given the others,
// through the precision matrix H:
//   cond_mean = mean_i - (1 / H_ii) (H_i. diff - H_ii diff_i),
//   u = phi(a) + (phi(b) - phi(a)) ur,  x_i = -sqrt2 erfinv(1 - 2u) sd_i + cond_mean.
// The draws are scalar (one packet each, lane 0 kept) in the order
// sweep, component, chain, so the draw of (step t, chain j) of a stream that
// owns n chains is that stream's draw t n + j: the draws of a run of steps are
// made first (draw_first_words) and one thread per chain runs the steps.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_math.cuh"
#include "gr_mv.cuh"

namespace gr {
namespace {

constexpr int kTmvThreads = 128;

__device__ __forceinline__ float tm_erfc(float x) { return erfcf(x); }
__device__ __forceinline__ double tm_erfc(double x) { return erfc(x); }
__device__ __forceinline__ float tm_erfinv(float x) { return erfinvf_(x); }
__device__ __forceinline__ double tm_erfinv(double x) { return erfinv_(x); }
// BitScalar::to_ur of the draw's first element: the low 32 bits (float) or
// the whole lane (double)
__device__ __forceinline__ float tm_ur(uint64_t w, float) {
  return __uint_as_float(((uint32_t)w & 0x7fffffu) | (127u << 23)) - 1.0f;
}
__device__ __forceinline__ double tm_ur(uint64_t w, double) {
  return __longlong_as_double((long long)((w & 0xfffffffffffffull) | (1023ull << 52))) - 1.0;
}

template <class T>
__global__ void __launch_bounds__(kTmvThreads) k_tmvn(TmvArgs a) {
  extern __shared__ __align__(16) unsigned char tm_dyn[];
  const int d = a.dim;
  T* H = reinterpret_cast<T*>(tm_dyn);  // column-major d x d
  T* mu = H + d * d;
  T* lo = mu + d;
  T* hi = lo + d;
  T* idg = hi + d;
  T* csd = idg + d;
  for (int i = threadIdx.x; i < d * d; i += blockDim.x) H[i] = static_cast<const T*>(a.H)[i];
  for (int i = threadIdx.x; i < d; i += blockDim.x) {
    mu[i] = static_cast<const T*>(a.mean)[i];
    lo[i] = static_cast<const T*>(a.lo)[i];
    hi[i] = static_cast<const T*>(a.hi)[i];
    idg[i] = static_cast<const T*>(a.inv_diag)[i];
    csd[i] = static_cast<const T*>(a.cond_sd)[i];
  }
  __syncthreads();
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.samples) return;
  // the stream that owns chain s, split as any call splits its outputs
  const int64_t base = a.samples / a.K, rem = a.samples % a.K;
  const int64_t k = s < rem * (base + 1) ? s / (base + 1) : rem + (s - rem * (base + 1)) / base;
  const int64_t s0 = k * base + (k < rem ? k : rem), nk = base + (k < rem ? 1 : 0);
  const uint64_t* w = a.draws + s0 * a.tc + (s - s0);
  T* X = static_cast<T*>(a.x) + s * d;
  T x[kTmvMaxDim], df[kTmvMaxDim];
  for (int i = 0; i < d; ++i) {
    x[i] = X[i];
    df[i] = x[i] - mu[i];
  }
  const T rs2 = (T)(1.0 / 1.4142135623730951), ms2 = (T)(-1.4142135623730951);
  int i = (int)(a.t0 % d);
  for (int64_t t = 0; t < a.tc; ++t) {
    T h = H[i] * df[0];
    for (int j = 1; j < d; ++j) h = h + H[j * d + i] * df[j];
    const T cm = mu[i] - idg[i] * (h - H[i * d + i] * df[i]);
    const T an = (lo[i] - cm) / csd[i], bn = (hi[i] - cm) / csd[i];
    const T pa = (T)0.5 * tm_erfc(-an * rs2), pb = (T)0.5 * tm_erfc(-bn * rs2);
    const T u = pa + (pb - pa) * tm_ur(__ldg(w + t * nk), T());
    const T z = ms2 * tm_erfinv((T)1 - (T)2 * u);
    const T nx = z * csd[i] + cm;
    df[i] = nx - mu[i];
    x[i] = nx;
    if (++i == d) i = 0;
  }
  for (int q = 0; q < d; ++q) X[q] = x[q];
}

template <class T>
__global__ void k_tmvn_init(const T* init, T* x, int d, int64_t samples) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < samples * d) x[e] = init[e % d];
}

template <class T>
cudaError_t run_tmvn(const TmvArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(T) * ((size_t)a.dim * a.dim + 5 * (size_t)a.dim);
  const unsigned blocks = (unsigned)((a.samples + kTmvThreads - 1) / kTmvThreads);
  k_tmvn<T><<<blocks, kTmvThreads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tmvn_init(int dtype, const void* init, void* x, int dim, int64_t samples, cudaStream_t s) {
  const int64_t n = samples * dim;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (dtype == GR_F64)
    k_tmvn_init<double><<<blocks, 256, 0, s>>>(static_cast<const double*>(init), static_cast<double*>(x), dim, samples);
  else
    k_tmvn_init<float><<<blocks, 256, 0, s>>>(static_cast<const float*>(init), static_cast<float*>(x), dim, samples);
  return cudaGetLastError();
}

cudaError_t launch_tmvn(int dtype, const TmvArgs& a, cudaStream_t s) {
  if (a.dim < 1 || a.dim > kTmvMaxDim || a.samples <= 0 || a.tc <= 0) return cudaErrorInvalidValue;
  return dtype == GR_F64 ? run_tmvn<double>(a, s) : run_tmvn<float>(a, s);
}

}  // namespace gr
