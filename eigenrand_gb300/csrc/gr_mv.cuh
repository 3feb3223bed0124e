// Interface of the multivariate kernels (gr_mv.cu) for the host library.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "gr_internal.h"
#include "gr_kernels.cuh"

namespace gr {

constexpr int kWishTcMaxDim = 128;           // tensor-core Wishart products up to this dimension
constexpr size_t kMvMaxSmem = 200 * 1024;    // shared memory cap of the SIMT fallbacks
constexpr int kMvMaxDim = 2048;              // largest MvNormal dimension (in-place product)
constexpr int kMnMaxSampleWords = 2464;      // multinomial sample must fit the two-block ring

// Lower-triangular fragment count: sum over m-tiles of min(2mt + 2, KS).
__host__ __device__ inline int64_t mv_tri_frags(int MT, int KS) {
  int64_t t = 0;
  for (int m = 0; m < MT; ++m) t += (2 * m + 2 < KS) ? 2 * m + 2 : KS;
  return t;
}

// ---- multinomial word layout (MultinomialGen::generate, Multinomial.h:95-118)
// Per sample: nP = trials / 4 DiscreteGen packet draws (16 at a time, then the
// tail's whole packets) followed by ns = trials % 4 scalar draws.  State c =
// DiscreteGen cache full (1) or empty (0) when the sample starts.
struct MnLayout {
  int nP, ns;  // packet draws, scalar draws
  int spu;     // period of the state sequence in samples (1 or 2)
  int c0;      // state of the first sample
  int64_t W0, W1;  // u32 words consumed by a sample in state 0 / 1
};

__host__ __device__ inline MnLayout mn_layout(int trials, int c0) {
  MnLayout L;
  L.nP = trials >> 2;
  L.ns = trials & 3;
  L.c0 = c0;
  L.W0 = 8 * (int64_t)((L.nP + 1) / 2 + L.ns);  // ceil(nP/2) packets + ns scalar packets
  L.W1 = 8 * (int64_t)(L.nP / 2 + L.ns);        // first draw from the cache: ceil((nP-1)/2)
  L.spu = (L.nP & 1) ? 2 : 1;                   // odd nP flips the cache every sample
  return L;
}
__host__ __device__ inline int mn_state(const MnLayout& L, int64_t i) {
  return L.spu == 2 ? (L.c0 ^ (int)(i & 1)) : L.c0;
}
// words before sample i (relative to the engine slice)
__host__ __device__ inline int64_t mn_base(const MnLayout& L, int64_t i) {
  if (L.spu == 1) return i * (L.c0 ? L.W1 : L.W0);
  return (i >> 1) * (L.W0 + L.W1) + ((i & 1) ? (L.c0 ? L.W1 : L.W0) : 0);
}
// word offset (within a sample of state c) of the half packet it leaves cached
__host__ __device__ inline int64_t mn_cache_off(const MnLayout& L, int c) {
  return c == 0 ? 4 * (int64_t)L.nP : 4 * (int64_t)L.nP - 4;
}
// word offset of the first scalar draw's packet
__host__ __device__ inline int64_t mn_scalar_off(const MnLayout& L, int c) {
  return c == 0 ? 8 * (int64_t)((L.nP + 1) / 2) : 8 * (int64_t)(L.nP / 2);
}

struct MnArgs {
  const int32_t* prob;   // alias probabilities, or the CDF when ncdf > 0
  const int32_t* alias;
  uint32_t bitmask;
  int32_t ncdf;
  int32_t dim;
  int32_t trials;
  int64_t Us;            // state periods per jump segment
  int32_t* out;          // dim x samples, column-major
};

// MultinomialGen's conditional-binomial path (gr_mncond.cu): rows binomial
// rows of p[row] over the engine's samples (granule 8), out dim x samples.
struct McArgs {
  const float* p;      // p of each drawn row, float (device)
  int32_t rows;        // rows drawn: max(dim - 1, 1)
  int32_t dim;
  int32_t trials;
  int32_t* out;        // dim x samples, column-major
  int64_t max_blocks;  // engine blocks per engine before the status word is set
};
cudaError_t launch_mn_cond(const Plan& p, const McArgs& a, cudaStream_t s);

// TruncMvNormalGen's Gibbs chains (gr_tmvn.cu), one thread per chain, steps
// [t0, t0 + tc) of sweep-major (sweep, component) order.  Arrays are device
// arrays in the object's type.
constexpr int kTmvMaxDim = 64;
struct TmvArgs {
  const void* H;         // precision matrix, column-major dim x dim
  const void* mean;
  const void* lo;
  const void* hi;
  const void* inv_diag;  // 1 / H_ii
  const void* cond_sd;   // sqrt(1 / H_ii)
  int32_t dim;
  int32_t K;             // engine streams (chain slices as any call splits them)
  int64_t samples;
  int64_t t0, tc;
  const uint64_t* draws; // stream k's draws of the run: s0_k * tc + (t - t0) * n_k + j
  void* x;               // dim x samples, the chains' state and the result
};
cudaError_t launch_tmvn(int dtype, const TmvArgs& a, cudaStream_t s);
cudaError_t launch_tmvn_init(int dtype, const void* init, void* x, int dim, int64_t samples, cudaStream_t s);

cudaError_t launch_inverse_f64(double* A, double* W, int d, int32_t* status, cudaStream_t s);
cudaError_t launch_chol_f64(double* A, int d, int32_t* status, cudaStream_t s);
cudaError_t launch_jacobi_f64(double* A, double* V, double* L, int d, int32_t* status, cudaStream_t s);
cudaError_t launch_pack_lt(const double* L, float* out, int d, int tri, cudaStream_t s);
cudaError_t launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t s);
cudaError_t launch_mvn(const float* Lf, int tri, const float* mean, float* X, int d, int64_t n, cudaStream_t s);
// X = L Z + mean (float) with tcgen05.mma (gr_umma.cu), dim <= kUmmaMaxDim:
// the factor prepared once by launch_prep_lt_umma into umma_prep_floats(d,
// tri) floats (tri: L lower triangular, its zero blocks left out);
// umma_usable says whether a call can take this path (dim a multiple of 4,
// X 16-byte aligned, fewer than 2^31 samples); device errors go to *status.
constexpr int kUmmaMaxDim = 256;
constexpr int kUmmaAutoMinDim = 20;  // smallest dim the tcgen05 product is used for by default
// WishartGen<float> (not inverse) Bartlett products T = L A, W = T T^T on
// tcgen05 (gr_umma.cu), dims up to kWishUmmaMaxDim; device errors go to *status
constexpr int kWishUmmaMaxDim = 64;
bool wishart_umma_usable(int d, int dtype, int inverse);
cudaError_t launch_wishart_umma(const float* normals, const float* chis, const float* chol, float* out, int d,
                                int64_t samples, int32_t* status, cudaStream_t s);
int umma_padded_dim(int d);
int umma_chunks(int d);
size_t umma_prep_floats(int d, int tri);
bool umma_usable(int d, const void* X, int64_t n);
cudaError_t launch_prep_lt_umma(const double* L, float* out, int d, int tri, cudaStream_t s);
cudaError_t launch_mvn_umma(const float* Lp, int tri, const float* mean, float* X, int d, int64_t n, int32_t* status,
                            cudaStream_t s);
cudaError_t launch_mvn_f64(const double* L, int tri, const double* mean, double* X, int d, int64_t n, cudaStream_t s);
size_t wishart_smem(int d, int dtype);
cudaError_t launch_wishart(const void* normals, const void* chis, const void* chol, void* out, int d, int64_t samples,
                           int inverse, int dtype, cudaStream_t s);
size_t dirichlet_smem(int K, int dtype);
cudaError_t launch_dirichlet(const void* rows, void* out, int K, int64_t n, int dtype, cudaStream_t s);
cudaError_t launch_multinomial(const Plan& p, const MnArgs& a, const CallSnap* snap, cudaStream_t s);

// Host side (gr_api.cu): DiscreteGen's CDF / alias table (Discrete.h:23-207).
gr_status build_discrete_table(const std::vector<double>& w, std::vector<int32_t>& prob, std::vector<int32_t>& alias,
                               int& ncdf, uint32_t& bitmask);
// Host side (gr_api.cu): plans and launches k_multinomial on an engine, with
// the same slice / jump-segment split as the fixed-consumption samplers.
gr_status run_multinomial(gr_engine* e, GenState* gst, const MnArgs& a, int64_t samples, cudaStream_t s);
// Host side (gr_api.cu): pre-allocates an engine's segmented-call scratch.
gr_status engine_reserve(gr_engine* e, int max_segments);
// Host side (gr_mvapi.cu): a second MvNormalGen with the same mean and factor
// (no refactorisation) and its own StdNormalGen.
gr_status mvnormal_clone(const gr_mvnormal* src, gr_mvnormal** out);
int mvnormal_dim(const gr_mvnormal* g);

}  // namespace gr
