// C ABI of the multivariate generators (include/gpurand.h, EigenRand/MvDists).
//
// Each object owns the FP64 factor of its matrix (computed on the GPU at
// creation), device copies of its parameters and the member generators whose
// caches persist across calls.  A call issues the member generators' draws in
// the reference's order (gr_generate on the caller's engine), then the
// assembly kernels of gr_mv.cu.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_mv.cuh"

using namespace gr;

namespace {

gr_status mv_fail(gr_status s, const std::string& m) { return set_last_error(s, m); }

#define MV_CUDA(call)                                                                                 \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) return set_last_error(GR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int packet_width(int dtype) { return dtype == GR_F32 ? 8 : 4; }
size_t elem_size(int dtype) { return dtype == GR_F32 ? sizeof(float) : sizeof(double); }

// Eigen 3.4's sum() of a dynamic double vector compiled with AVX (packets of
// 4, the LinearVectorizedTraversal redux): two packet accumulators over pairs
// of packets, added, plus one more packet when the aligned part holds an odd
// number of them; the packet reduced as (a0 + a2) + (a1 + a3); then the
// remaining elements in order.  Below one packet it is a plain left-to-right
// sum.  Eigen's storage is 32-byte aligned, so the aligned part starts at 0.
// MultinomialGen normalises its weights by this sum.
double eigen_sum_avx(const double* v, int n) {
  constexpr int ps = 4;
  const int as2 = (n / (2 * ps)) * (2 * ps), as = (n / ps) * ps;
  if (as == 0) {
    double r = v[0];
    for (int i = 1; i < n; ++i) r = r + v[i];
    return r;
  }
  double acc0[ps], acc1[ps];
  for (int j = 0; j < ps; ++j) acc0[j] = v[j];
  if (as > ps) {
    for (int j = 0; j < ps; ++j) acc1[j] = v[ps + j];
    for (int i = 2 * ps; i < as2; i += 2 * ps) {
      for (int j = 0; j < ps; ++j) {
        acc0[j] = acc0[j] + v[i + j];
        acc1[j] = acc1[j] + v[i + ps + j];
      }
    }
    for (int j = 0; j < ps; ++j) acc0[j] = acc0[j] + acc1[j];
    if (as > as2)
      for (int j = 0; j < ps; ++j) acc0[j] = acc0[j] + v[as2 + j];
  }
  double r = (acc0[0] + acc0[2]) + (acc0[1] + acc0[3]);
  for (int i = as; i < n; ++i) r = r + v[i];
  return r;
}

// The constructor's per-dimension values in the scalar type T
// (TruncMvNormal.h:76-91): H = L^-T L^-1 from the lower triangle of the
// factor (computed in FP64, then rounded to T), 1 / H_ii, sqrt of that, and
// clamp(mean, lower, upper).
template <typename T>
std::vector<T> tmvn_values(int d, const std::vector<double>& H, const double* mean, const double* lower,
                           const double* upper) {
  std::vector<T> v((size_t)d * d + 6 * (size_t)d);
  T* Ht = v.data();
  T* mu = Ht + (size_t)d * d;
  T* lo = mu + d;
  T* hi = lo + d;
  T* idg = hi + d;
  T* csd = idg + d;
  T* init = csd + d;
  for (size_t i = 0; i < (size_t)d * d; ++i) Ht[i] = (T)H[i];
  for (int i = 0; i < d; ++i) {
    mu[i] = (T)mean[i];
    lo[i] = (T)lower[i];
    hi[i] = (T)upper[i];
    idg[i] = (T)1 / Ht[(size_t)i * d + i];
    csd[i] = std::sqrt(idg[i]);
    init[i] = std::max(lo[i], std::min(mu[i], hi[i]));
  }
  return v;
}

bool all_finite(const double* v, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

// RAII for the temporaries of one factorisation.
struct DevBufs {
  std::vector<void*> p;
  cudaStream_t s = nullptr;
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
    if (s) cudaStreamDestroy(s);
  }
  template <class T>
  cudaError_t alloc(T** out, size_t n) {
    cudaError_t e = cudaMalloc((void**)out, sizeof(T) * n);
    if (e == cudaSuccess) p.push_back(*out);
    return e;
  }
};

// The factor get_lt (MvNormal.h:21-38) computes, in FP64 on the GPU:
// Cholesky of the lower triangle, else V diag(sqrt(max(lambda, 0))) of the
// symmetric matrix the lower triangle defines.  invert: factor of matrix^-1
// (InvWishartGen, MvNormal.h:387-391).  GR_MATRIX_LOWER: the matrix is the
// factor.  *tri = 1 when the factor is lower triangular.
gr_status factor_f64(int d, const double* host, int form, bool invert, double** out_dev, int* tri) {
  const size_t dd = (size_t)d * d;
  std::vector<double> h(host, host + dd);
  double* L = nullptr;
  MV_CUDA(cudaMalloc(&L, sizeof(double) * dd));
  if (form == GR_MATRIX_LOWER) {
    int is_tri = 1;
    for (int c = 0; c < d; ++c)
      for (int r = 0; r < c; ++r)
        if (h[(size_t)c * d + r] != 0.0) is_tri = 0;
    cudaError_t e = cudaMemcpy(L, h.data(), sizeof(double) * dd, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(L);
      return mv_fail(GR_ERR_CUDA, std::string("factor upload: ") + cudaGetErrorString(e));
    }
    *out_dev = L;
    *tri = is_tri;
    return GR_OK;
  }
  DevBufs b;
  b.p.push_back(L);  // freed on error; released below on success
  double *A = nullptr, *W = nullptr;
  int32_t* status = nullptr;
  MV_CUDA(b.alloc(&A, dd));
  MV_CUDA(b.alloc(&W, dd));
  MV_CUDA(b.alloc(&status, 1));
  MV_CUDA(cudaStreamCreateWithFlags(&b.s, cudaStreamNonBlocking));
  int32_t hs = 0;
  MV_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), b.s));
  if (invert) {
    MV_CUDA(cudaMemcpyAsync(A, h.data(), sizeof(double) * dd, cudaMemcpyHostToDevice, b.s));
    MV_CUDA(launch_inverse_f64(A, W, d, status, b.s));
    MV_CUDA(cudaMemcpyAsync(h.data(), A, sizeof(double) * dd, cudaMemcpyDeviceToHost, b.s));
    MV_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int32_t), cudaMemcpyDeviceToHost, b.s));
    MV_CUDA(cudaStreamSynchronize(b.s));
    if (hs & 1) return mv_fail(GR_ERR_NOT_PD, "the scale matrix is singular");
  }
  // LLT and SelfAdjointEigenSolver read the lower triangle only
  for (int c = 0; c < d; ++c)
    for (int r = 0; r < c; ++r) h[(size_t)c * d + r] = h[(size_t)r * d + c];
  MV_CUDA(cudaMemcpyAsync(A, h.data(), sizeof(double) * dd, cudaMemcpyHostToDevice, b.s));
  MV_CUDA(launch_chol_f64(A, d, status, b.s));
  MV_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int32_t), cudaMemcpyDeviceToHost, b.s));
  MV_CUDA(cudaStreamSynchronize(b.s));
  if (!(hs & 2)) {
    MV_CUDA(cudaMemcpyAsync(L, A, sizeof(double) * dd, cudaMemcpyDeviceToDevice, b.s));
    *tri = 1;
  } else {
    MV_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), b.s));
    MV_CUDA(cudaMemcpyAsync(A, h.data(), sizeof(double) * dd, cudaMemcpyHostToDevice, b.s));
    MV_CUDA(launch_jacobi_f64(A, W, L, d, status, b.s));
    MV_CUDA(cudaMemcpyAsync(&hs, status, sizeof(int32_t), cudaMemcpyDeviceToHost, b.s));
    MV_CUDA(cudaStreamSynchronize(b.s));
    if (hs & 4) return mv_fail(GR_ERR_NOT_PD, "The matrix cannot be solved! (eigen decomposition did not converge)");
    *tri = 0;
  }
  MV_CUDA(cudaStreamSynchronize(b.s));
  b.p.erase(b.p.begin());  // keep L
  *out_dev = L;
  return GR_OK;
}

gr_status make_gen(gr_gen** out, int kind, int dtype, double a, double b = 0.0) {
  gr_dist_desc d{};
  d.kind = kind;
  d.dtype = dtype;
  d.a = a;
  d.b = b;
  return gr_gen_create(out, &d);
}

// device scratch owned by an object, grown on demand
struct Scratch {
  void* p = nullptr;
  size_t bytes = 0;
  gr_status need(size_t n) {
    if (n <= bytes) return GR_OK;
    cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) return mv_fail(GR_ERR_NOMEM, std::string("scratch: ") + cudaGetErrorString(e));
    bytes = n;
    return GR_OK;
  }
  ~Scratch() { cudaFree(p); }
};

}  // namespace

struct gr_mvnormal {
  int dim = 0, dtype = GR_F32, tri = 1;
  double* L64 = nullptr;
  float* Lf = nullptr;  // packed float fragments (float objects)
  float* Lu = nullptr;  // the factor as the tcgen05 B operand (float objects, dim <= kUmmaMaxDim)
  void* mean = nullptr;
  gr_gen* normal = nullptr;
};

struct gr_wishart {
  int dim = 0, dtype = GR_F32, inverse = 0;
  int64_t df = 0;
  double* L64 = nullptr;
  void* chol = nullptr;  // factor in the object's type (aliases L64 for double)
  gr_gen* normal = nullptr;
  std::vector<gr_gen*> chis;
  Scratch scratch;
};

struct gr_dirichlet {
  int dim = 0, dtype = GR_F32;
  std::vector<gr_gen*> gammas;
  Scratch scratch;
};

struct gr_truncmvn {
  int dim = 0, dtype = GR_F32;
  int64_t burn_in = 0;
  // device, the object's type: H (dim x dim), mean, lower, upper, 1/H_ii,
  // sqrt(1/H_ii), initial state
  void* buf = nullptr;
};

struct gr_multinomial {
  int dim = 0, trials = 0;
  // conditional-binomial path: p of each drawn row (device floats)
  bool cond = false;
  float* pdev = nullptr;
  int rows = 0;
  int32_t* table = nullptr;  // prob (or CDF) then alias
  int32_t ncdf = 0;
  uint32_t bitmask = 0;
  size_t nprob = 0;
  GenState* gst = nullptr;
  int gst_K = 0;
};

namespace gr {

int mvnormal_dim(const gr_mvnormal* g) { return g ? g->dim : 0; }

gr_status mvnormal_clone(const gr_mvnormal* src, gr_mvnormal** out) {
  if (!src || !out) return mv_fail(GR_ERR_INVALID, "NULL argument");
  gr_mvnormal* g = new gr_mvnormal;
  g->dim = src->dim;
  g->dtype = src->dtype;
  g->tri = src->tri;
  const size_t dd = (size_t)src->dim * src->dim;
  const size_t es = elem_size(src->dtype);
  cudaError_t e = cudaMalloc(&g->L64, sizeof(double) * dd);
  if (e == cudaSuccess) e = cudaMemcpy(g->L64, src->L64, sizeof(double) * dd, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess && src->Lf) {
    const int MT = (src->dim + 15) / 16, KS = (src->dim + 7) / 8;
    const int64_t nfr = src->tri ? mv_tri_frags(MT, KS) : (int64_t)MT * KS;
    e = cudaMalloc(&g->Lf, sizeof(float) * (size_t)nfr * 128);
    if (e == cudaSuccess) e = cudaMemcpy(g->Lf, src->Lf, sizeof(float) * (size_t)nfr * 128, cudaMemcpyDeviceToDevice);
  }
  if (e == cudaSuccess && src->Lu) {
    const size_t nu = umma_prep_floats(src->dim, src->tri);
    e = cudaMalloc(&g->Lu, sizeof(float) * nu);
    if (e == cudaSuccess) e = cudaMemcpy(g->Lu, src->Lu, sizeof(float) * nu, cudaMemcpyDeviceToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc(&g->mean, es * src->dim);
  if (e == cudaSuccess) e = cudaMemcpy(g->mean, src->mean, es * src->dim, cudaMemcpyDeviceToDevice);
  // device-to-device copies return before they finish, and the clone's
  // users launch on streams that do not wait for the legacy stream
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  gr_status st = e == cudaSuccess ? GR_OK : mv_fail(GR_ERR_CUDA, std::string("MvNormalGen copy: ") + cudaGetErrorString(e));
  if (st == GR_OK) st = make_gen(&g->normal, GR_NORMAL_STD, g->dtype, 0.0);
  if (st != GR_OK) {
    gr_mvnormal_destroy(g);
    return st;
  }
  *out = g;
  return GR_OK;
}

}  // namespace gr

extern "C" {

// ---------------------------------------------------------------- MvNormalGen
gr_status gr_mvnormal_destroy(gr_mvnormal* g) {
  if (!g) return GR_OK;
  cudaFree(g->L64);
  cudaFree(g->Lf);
  cudaFree(g->Lu);
  cudaFree(g->mean);
  gr_gen_destroy(g->normal);
  delete g;
  return GR_OK;
}

gr_status gr_mvnormal_create(gr_mvnormal** out, int32_t dtype, int32_t dim, const double* mean, const double* matrix,
                             int32_t matrix_form) {
  if (!out || !mean || !matrix) return mv_fail(GR_ERR_INVALID, "NULL argument");
  if (dtype != GR_F32 && dtype != GR_F64) return mv_fail(GR_ERR_INVALID, "MvNormalGen needs a float or double type");
  if (matrix_form != GR_MATRIX_FULL && matrix_form != GR_MATRIX_LOWER) return mv_fail(GR_ERR_INVALID, "bad matrix form");
  if (dim < 1) return mv_fail(GR_ERR_INVALID, "dim must be >= 1");
  if (dtype == GR_F32 && dim > kMvMaxDim) return mv_fail(GR_ERR_UNSUPPORTED, "float MvNormalGen: dim <= 2048");
  if (dtype == GR_F64 && (size_t)32 * dim * sizeof(double) > kMvMaxSmem)
    return mv_fail(GR_ERR_UNSUPPORTED, "double MvNormalGen: dim <= 800");
  if (!all_finite(mean, dim) || !all_finite(matrix, (size_t)dim * dim))
    return mv_fail(GR_ERR_INVALID, "non-finite mean or matrix");
  gr_mvnormal* g = new gr_mvnormal;
  g->dim = dim;
  g->dtype = dtype;
  gr_status st = factor_f64(dim, matrix, matrix_form, false, &g->L64, &g->tri);
  // test hook: GR_MVN_FULL_FORM=1 treats a triangular factor as a full matrix
  // (the products then run over every block, as for the eigen form)
  if (const char* ff = std::getenv("GR_MVN_FULL_FORM"))
    if (ff[0] == '1') g->tri = 0;
  if (st == GR_OK) {
    cudaError_t e = cudaSuccess;
    if (dtype == GR_F32) {
      const int MT = (dim + 15) / 16, KS = (dim + 7) / 8;
      const int64_t nfr = g->tri ? mv_tri_frags(MT, KS) : (int64_t)MT * KS;
      e = cudaMalloc(&g->Lf, sizeof(float) * (size_t)nfr * 128);
      if (e == cudaSuccess) e = launch_pack_lt(g->L64, g->Lf, dim, g->tri, nullptr);
      if (e == cudaSuccess && dim <= kUmmaMaxDim) {
        const size_t nu = umma_prep_floats(dim, g->tri);
        e = cudaMalloc(&g->Lu, sizeof(float) * nu);
        if (e == cudaSuccess) e = launch_prep_lt_umma(g->L64, g->Lu, dim, g->tri, nullptr);
      }
      std::vector<float> mf(mean, mean + dim);
      if (e == cudaSuccess) e = cudaMalloc(&g->mean, sizeof(float) * dim);
      if (e == cudaSuccess) e = cudaMemcpy(g->mean, mf.data(), sizeof(float) * dim, cudaMemcpyHostToDevice);
    } else {
      e = cudaMalloc(&g->mean, sizeof(double) * dim);
      if (e == cudaSuccess) e = cudaMemcpy(g->mean, mean, sizeof(double) * dim, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) st = mv_fail(GR_ERR_CUDA, std::string("MvNormalGen set-up: ") + cudaGetErrorString(e));
  }
  if (st == GR_OK) st = make_gen(&g->normal, GR_NORMAL_STD, dtype, 0.0);
  if (st != GR_OK) {
    gr_mvnormal_destroy(g);
    return st;
  }
  *out = g;
  return GR_OK;
}

gr_status gr_mvnormal_sample(gr_mvnormal* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream) {
  if (need_four_lanes(e, "MvNormalGen") != GR_OK) return GR_ERR_UNSUPPORTED;
  if (!g || !e) return mv_fail(GR_ERR_INVALID, "NULL generator or engine");
  if (samples == 0) return GR_OK;
  if (!dev_out) return mv_fail(GR_ERR_INVALID, "output is NULL");
  const size_t n = (size_t)g->dim * samples;
  if (n % (size_t)packet_width(g->dtype))
    return mv_fail(GR_ERR_INVALID, "dim * samples must be a multiple of the packet width");
  cudaStream_t s = (cudaStream_t)stream;
  // Z = StdNormalGen draws (dim x samples), then X = L Z + mean in place
  gr_status st = gr_generate(g->normal, e, dev_out, n, stream);
  if (st != GR_OK) return st;
  cudaError_t err;
  // the tcgen05 product from kUmmaAutoMinDim up (below it the mma.sync form
  // is as fast); test hook GR_MVN_PRODUCT=tcgen05 | mma_sync picks one form
  bool umma = g->dim >= kUmmaAutoMinDim;
  if (const char* pv = std::getenv("GR_MVN_PRODUCT")) {
    if (std::strcmp(pv, "tcgen05") == 0) umma = true;
    if (std::strcmp(pv, "mma_sync") == 0) umma = false;
  }
  if (g->dtype == GR_F32 && g->Lu && umma && umma_usable(g->dim, dev_out, (int64_t)samples))
    err = launch_mvn_umma(g->Lu, g->tri, (const float*)g->mean, (float*)dev_out, g->dim, (int64_t)samples,
                          &engine_state_ptr(e)->status, s);
  else if (g->dtype == GR_F32)
    err = launch_mvn(g->Lf, g->tri, (const float*)g->mean, (float*)dev_out, g->dim, (int64_t)samples, s);
  else
    err = launch_mvn_f64(g->L64, g->tri, (const double*)g->mean, (double*)dev_out, g->dim, (int64_t)samples, s);
  if (err != cudaSuccess) return mv_fail(GR_ERR_CUDA, std::string("MvNormal product: ") + cudaGetErrorString(err));
  return GR_OK;
}

// ---------------------------------------------------------------- Wishart / InvWishart
gr_status gr_wishart_destroy(gr_wishart* g) {
  if (!g) return GR_OK;
  if (g->chol != g->L64) cudaFree(g->chol);
  cudaFree(g->L64);
  gr_gen_destroy(g->normal);
  for (gr_gen* c : g->chis) gr_gen_destroy(c);
  delete g;
  return GR_OK;
}

gr_status gr_wishart_create(gr_wishart** out, int32_t dtype, int32_t dim, int64_t df, const double* matrix,
                            int32_t matrix_form, int32_t inverse) {
  if (!out || !matrix) return mv_fail(GR_ERR_INVALID, "NULL argument");
  if (dtype != GR_F32 && dtype != GR_F64) return mv_fail(GR_ERR_INVALID, "WishartGen needs a float or double type");
  if (matrix_form != GR_MATRIX_FULL && matrix_form != GR_MATRIX_LOWER) return mv_fail(GR_ERR_INVALID, "bad matrix form");
  if (dim < 1) return mv_fail(GR_ERR_INVALID, "dim must be >= 1");
  if (df <= dim - 1) return mv_fail(GR_ERR_INVALID, "df must be > dim - 1");
  if (wishart_smem(dim, dtype) > kMvMaxSmem) return mv_fail(GR_ERR_UNSUPPORTED, "Wishart dimension too large");
  if (!all_finite(matrix, (size_t)dim * dim)) return mv_fail(GR_ERR_INVALID, "non-finite matrix");
  gr_wishart* g = new gr_wishart;
  g->dim = dim;
  g->dtype = dtype;
  g->df = df;
  g->inverse = inverse ? 1 : 0;
  int tri = 0;
  gr_status st = factor_f64(dim, matrix, matrix_form, g->inverse && matrix_form == GR_MATRIX_FULL, &g->L64, &tri);
  if (st == GR_OK) {
    if (dtype == GR_F64) {
      g->chol = g->L64;
    } else {
      cudaError_t e = cudaMalloc(&g->chol, sizeof(float) * (size_t)dim * dim);
      if (e == cudaSuccess) e = launch_f64_to_f32(g->L64, (float*)g->chol, (int64_t)dim * dim, nullptr);
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
      if (e != cudaSuccess) st = mv_fail(GR_ERR_CUDA, std::string("WishartGen set-up: ") + cudaGetErrorString(e));
    }
  }
  if (st == GR_OK) st = make_gen(&g->normal, GR_NORMAL_STD, dtype, 0.0);
  for (int i = 0; st == GR_OK && i < dim; ++i) {  // ChiSquaredGen(df - i)
    gr_gen* c = nullptr;
    st = make_gen(&c, GR_CHI_SQUARED, dtype, (double)(df - i));
    if (st == GR_OK) g->chis.push_back(c);
  }
  if (st != GR_OK) {
    gr_wishart_destroy(g);
    return st;
  }
  *out = g;
  return GR_OK;
}

gr_status gr_wishart_sample(gr_wishart* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream) {
  if (need_four_lanes(e, "WishartGen") != GR_OK) return GR_ERR_UNSUPPORTED;
  if (!g || !e) return mv_fail(GR_ERR_INVALID, "NULL generator or engine");
  if (samples == 0) return GR_OK;
  if (!dev_out) return mv_fail(GR_ERR_INVALID, "output is NULL");
  if ((uintptr_t)dev_out % 16) return mv_fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  const int d = g->dim;
  const size_t P = (size_t)packet_width(g->dtype);
  const size_t nnorm = samples * (size_t)d * (size_t)(d - 1) / 2;
  if (samples % P || nnorm % P)
    return mv_fail(GR_ERR_INVALID, "samples and samples * dim * (dim - 1) / 2 must be multiples of the packet width");
  const size_t es = elem_size(g->dtype);
  gr_status st = g->scratch.need((nnorm + (size_t)d * samples) * es);
  if (st != GR_OK) return st;
  char* normals = (char*)g->scratch.p;
  char* chis = normals + nnorm * es;
  // draw order of WishartGen::generate: all normals, then one chi^2 row per diagonal
  if (nnorm) {
    st = gr_generate(g->normal, e, normals, nnorm, stream);
    if (st != GR_OK) return st;
  }
  for (int i = 0; i < d; ++i) {
    st = gr_generate(g->chis[i], e, chis + (size_t)i * samples * es, samples, stream);
    if (st != GR_OK) return st;
  }
  // the tcgen05 products for float WishartGen up to dim 64; test hook
  // GR_WISHART_PRODUCT=mma_sync picks the mma.sync form
  bool umma = wishart_umma_usable(d, g->dtype, g->inverse);
  if (const char* pv = std::getenv("GR_WISHART_PRODUCT"))
    if (std::strcmp(pv, "mma_sync") == 0) umma = false;
  cudaError_t err = umma ? launch_wishart_umma((const float*)normals, (const float*)chis, (const float*)g->chol,
                                               (float*)dev_out, d, (int64_t)samples, &engine_state_ptr(e)->status,
                                               (cudaStream_t)stream)
                         : launch_wishart(normals, chis, g->chol, dev_out, d, (int64_t)samples, g->inverse, g->dtype,
                                          (cudaStream_t)stream);
  if (err != cudaSuccess) return mv_fail(GR_ERR_CUDA, std::string("Wishart products: ") + cudaGetErrorString(err));
  return GR_OK;
}

// ---------------------------------------------------------------- DirichletGen
gr_status gr_dirichlet_destroy(gr_dirichlet* g) {
  if (!g) return GR_OK;
  for (gr_gen* x : g->gammas) gr_gen_destroy(x);
  delete g;
  return GR_OK;
}

gr_status gr_dirichlet_create(gr_dirichlet** out, int32_t dtype, int32_t dim, const double* alpha) {
  if (!out || !alpha) return mv_fail(GR_ERR_INVALID, "NULL argument");
  if (dtype != GR_F32 && dtype != GR_F64) return mv_fail(GR_ERR_INVALID, "DirichletGen needs a float or double type");
  if (dim < 1) return mv_fail(GR_ERR_INVALID, "dim must be >= 1");
  if (dirichlet_smem(dim, dtype) > kMvMaxSmem) return mv_fail(GR_ERR_UNSUPPORTED, "Dirichlet dimension too large");
  for (int i = 0; i < dim; ++i)
    if (!(alpha[i] > 0) || !std::isfinite(alpha[i])) return mv_fail(GR_ERR_INVALID, "alpha must be > 0");
  gr_dirichlet* g = new gr_dirichlet;
  g->dim = dim;
  g->dtype = dtype;
  gr_status st = GR_OK;
  for (int i = 0; st == GR_OK && i < dim; ++i) {  // GammaGen(alpha[i]) per category
    gr_gen* x = nullptr;
    st = make_gen(&x, GR_GAMMA, dtype, alpha[i], 1.0);
    if (st == GR_OK) g->gammas.push_back(x);
  }
  if (st != GR_OK) {
    gr_dirichlet_destroy(g);
    return st;
  }
  *out = g;
  return GR_OK;
}

gr_status gr_dirichlet_sample(gr_dirichlet* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream) {
  if (need_four_lanes(e, "DirichletGen") != GR_OK) return GR_ERR_UNSUPPORTED;
  if (!g || !e) return mv_fail(GR_ERR_INVALID, "NULL generator or engine");
  if (samples == 0) return GR_OK;
  if (!dev_out) return mv_fail(GR_ERR_INVALID, "output is NULL");
  if ((uintptr_t)dev_out % 16) return mv_fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  if (samples % (size_t)packet_width(g->dtype)) return mv_fail(GR_ERR_INVALID, "samples must be a multiple of the packet width");
  const size_t es = elem_size(g->dtype);
  gr_status st = g->scratch.need((size_t)g->dim * samples * es);
  if (st != GR_OK) return st;
  char* rows = (char*)g->scratch.p;
  for (int i = 0; i < g->dim; ++i) {
    st = gr_generate(g->gammas[i], e, rows + (size_t)i * samples * es, samples, stream);
    if (st != GR_OK) return st;
  }
  cudaError_t err = launch_dirichlet(rows, dev_out, g->dim, (int64_t)samples, g->dtype, (cudaStream_t)stream);
  if (err != cudaSuccess) return mv_fail(GR_ERR_CUDA, std::string("Dirichlet normalisation: ") + cudaGetErrorString(err));
  return GR_OK;
}

// ---------------------------------------------------------------- TruncMvNormalGen
gr_status gr_truncmvn_destroy(gr_truncmvn* g) {
  if (!g) return GR_OK;
  cudaFree(g->buf);
  delete g;
  return GR_OK;
}

gr_status gr_truncmvn_create(gr_truncmvn** out, int32_t dtype, int32_t dim, const double* mean, const double* matrix,
                             int32_t matrix_form, const double* lower, const double* upper, int64_t burn_in) {
  if (!out || !mean || !matrix || !lower || !upper) return mv_fail(GR_ERR_INVALID, "NULL argument");
  if (dtype != GR_F32 && dtype != GR_F64) return mv_fail(GR_ERR_INVALID, "TruncMvNormalGen needs a float or double type");
  if (matrix_form != GR_MATRIX_FULL && matrix_form != GR_MATRIX_LOWER) return mv_fail(GR_ERR_INVALID, "bad matrix form");
  if (dim < 1 || dim > kTmvMaxDim) return mv_fail(GR_ERR_UNSUPPORTED, "TruncMvNormalGen: 1 <= dim <= 64");
  if (burn_in < 0) return mv_fail(GR_ERR_INVALID, "burn_in must be >= 0");
  if (!all_finite(mean, dim) || !all_finite(matrix, (size_t)dim * dim))
    return mv_fail(GR_ERR_INVALID, "non-finite mean or matrix");
  for (int i = 0; i < dim; ++i) {
    const bool ok = dtype == GR_F32 ? (float)lower[i] < (float)upper[i] : lower[i] < upper[i];
    if (!ok) return mv_fail(GR_ERR_INVALID, "support needs lower[i] < upper[i]");
  }
  const size_t dd = (size_t)dim * dim;
  double* Ldev = nullptr;
  int tri = 1;
  gr_status st = factor_f64(dim, matrix, matrix_form, false, &Ldev, &tri);
  if (st != GR_OK) return st;
  std::vector<double> L(dd);
  cudaError_t e = cudaMemcpy(L.data(), Ldev, sizeof(double) * dd, cudaMemcpyDeviceToHost);
  cudaFree(Ldev);
  if (e != cudaSuccess) return mv_fail(GR_ERR_CUDA, std::string("factor download: ") + cudaGetErrorString(e));
  // inv = lower(L)^-1 by forward substitution, column by column; H = inv^T inv
  std::vector<double> inv(dd, 0.0), H(dd, 0.0);
  for (int c = 0; c < dim; ++c)
    for (int r = c; r < dim; ++r) {
      double v = r == c ? 1.0 : 0.0;
      for (int k = c; k < r; ++k) v -= L[(size_t)k * dim + r] * inv[(size_t)c * dim + k];
      inv[(size_t)c * dim + r] = v / L[(size_t)r * dim + r];
    }
  for (int j = 0; j < dim; ++j)
    for (int i = 0; i < dim; ++i) {
      double v = 0.0;
      for (int k = std::max(i, j); k < dim; ++k) v += inv[(size_t)i * dim + k] * inv[(size_t)j * dim + k];
      H[(size_t)j * dim + i] = v;
    }
  if (!all_finite(H.data(), dd)) return mv_fail(GR_ERR_NOT_PD, "the covariance factor is singular");
  gr_truncmvn* g = new gr_truncmvn;
  g->dim = dim;
  g->dtype = dtype;
  g->burn_in = burn_in == 0 ? 5 * (int64_t)dim : burn_in;
  if (dtype == GR_F32) {
    const std::vector<float> v = tmvn_values<float>(dim, H, mean, lower, upper);
    e = cudaMalloc(&g->buf, sizeof(float) * v.size());
    if (e == cudaSuccess) e = cudaMemcpy(g->buf, v.data(), sizeof(float) * v.size(), cudaMemcpyHostToDevice);
  } else {
    const std::vector<double> v = tmvn_values<double>(dim, H, mean, lower, upper);
    e = cudaMalloc(&g->buf, sizeof(double) * v.size());
    if (e == cudaSuccess) e = cudaMemcpy(g->buf, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    gr_truncmvn_destroy(g);
    return mv_fail(GR_ERR_CUDA, std::string("TruncMvNormalGen set-up: ") + cudaGetErrorString(e));
  }
  *out = g;
  return GR_OK;
}

gr_status gr_truncmvn_sample(gr_truncmvn* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream) {
  if (need_four_lanes(e, "TruncMvNormalGen") != GR_OK) return GR_ERR_UNSUPPORTED;
  if (!g || !e) return mv_fail(GR_ERR_INVALID, "NULL generator or engine");
  if (samples == 0) return GR_OK;
  if (!dev_out) return mv_fail(GR_ERR_INVALID, "output is NULL");
  if ((uintptr_t)dev_out % 16) return mv_fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  const int d = g->dim;
  const size_t es = elem_size(g->dtype);
  const char* b = static_cast<const char*>(g->buf);
  TmvArgs a{};
  a.H = b;
  a.mean = b + es * (size_t)d * d;
  a.lo = b + es * ((size_t)d * d + d);
  a.hi = b + es * ((size_t)d * d + 2 * d);
  a.inv_diag = b + es * ((size_t)d * d + 3 * d);
  a.cond_sd = b + es * ((size_t)d * d + 4 * d);
  const void* init = b + es * ((size_t)d * d + 5 * d);
  a.dim = d;
  a.K = gr_engine_streams(e);
  a.samples = (int64_t)samples;
  a.x = dev_out;
  MV_CUDA(launch_tmvn_init(g->dtype, init, dev_out, d, (int64_t)samples, s));
  // the draws of up to 2^25 (step, chain) pairs at a time
  const int64_t steps = g->burn_in * d;
  const int64_t tc = std::max<int64_t>(1, std::min<int64_t>(steps, ((int64_t)1 << 25) / (int64_t)samples));
  uint64_t* draws = nullptr;
  MV_CUDA(cudaMallocAsync(&draws, sizeof(uint64_t) * (size_t)tc * samples, s));
  gr_status st = GR_OK;
  for (int64_t t0 = 0; t0 < steps && st == GR_OK; t0 += tc) {
    const int64_t n = std::min(tc, steps - t0);
    st = draw_first_words(e, draws, n, (int64_t)samples, s);
    if (st != GR_OK) break;
    a.t0 = t0;
    a.tc = n;
    a.draws = draws;
    const cudaError_t err = launch_tmvn(g->dtype, a, s);
    if (err != cudaSuccess) st = mv_fail(GR_ERR_CUDA, std::string("TruncMvNormal kernel: ") + cudaGetErrorString(err));
  }
  cudaFreeAsync(draws, s);
  return st;
}

// ---------------------------------------------------------------- MultinomialGen
gr_status gr_multinomial_destroy(gr_multinomial* g) {
  if (!g) return GR_OK;
  cudaFree(g->pdev);
  cudaFree(g->table);
  cudaFree(g->gst);
  delete g;
  return GR_OK;
}

gr_status gr_multinomial_create(gr_multinomial** out, int32_t dim, int32_t trials, const double* weights) {
  if (!out || !weights) return mv_fail(GR_ERR_INVALID, "NULL argument");
  if (dim < 1) return mv_fail(GR_ERR_INVALID, "dim must be >= 1");
  if (trials < 0) return mv_fail(GR_ERR_INVALID, "trials must be >= 0");
  for (int i = 0; i < dim; ++i)
    if (!(weights[i] >= 0)) return mv_fail(GR_ERR_INVALID, "weights must be >= 0");
  if ((int64_t)trials >= std::max<int64_t>(30 * (int64_t)(dim - 1), 100)) {
    // probs = weights / probs.sum() (Multinomial.h:41-49), then the p of
    // each drawn row: probs[0], and probs[i] / rest_p with rest_p = 1 -
    // probs[0] - ... - probs[i-1] in double, converted to float
    const double sum = eigen_sum_avx(weights, dim);
    std::vector<double> probs(weights, weights + dim);
    for (double& q : probs) q = q / sum;
    const int rows = std::max(dim - 1, 1);
    std::vector<float> pr(rows);
    double rest = 1 - probs[0];
    pr[0] = (float)probs[0];
    for (int i = 1; i < rows; ++i) {
      pr[i] = (float)(probs[i] / rest);
      rest -= probs[i];
    }
    gr_multinomial* g = new gr_multinomial;
    g->dim = dim;
    g->trials = trials;
    g->cond = true;
    g->rows = rows;
    cudaError_t e = cudaMalloc(&g->pdev, sizeof(float) * rows);
    if (e == cudaSuccess) e = cudaMemcpy(g->pdev, pr.data(), sizeof(float) * rows, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      gr_multinomial_destroy(g);
      return mv_fail(GR_ERR_CUDA, std::string("multinomial p: ") + cudaGetErrorString(e));
    }
    *out = g;
    return GR_OK;
  }
  const MnLayout L = mn_layout(trials, 0);
  if (L.W0 > kMnMaxSampleWords || L.W1 > kMnMaxSampleWords)
    return mv_fail(GR_ERR_UNSUPPORTED, "multinomial: trials above 2400");
  if ((size_t)5 * dim * sizeof(int32_t) > 160 * 1024) return mv_fail(GR_ERR_UNSUPPORTED, "multinomial: dim too large");
  std::vector<double> w(weights, weights + dim);
  std::vector<int32_t> prob, alias;
  int ncdf = 0;
  uint32_t mask = 0;
  gr_status st = build_discrete_table(w, prob, alias, ncdf, mask);
  if (st != GR_OK) return st;
  gr_multinomial* g = new gr_multinomial;
  g->dim = dim;
  g->trials = trials;
  g->ncdf = ncdf;
  g->bitmask = mask;
  g->nprob = prob.size();
  std::vector<int32_t> both(prob);
  both.insert(both.end(), alias.begin(), alias.end());
  both.push_back(0);
  cudaError_t e = cudaMalloc(&g->table, sizeof(int32_t) * both.size());
  if (e == cudaSuccess) e = cudaMemcpy(g->table, both.data(), sizeof(int32_t) * both.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gr_multinomial_destroy(g);
    return mv_fail(GR_ERR_CUDA, std::string("multinomial table: ") + cudaGetErrorString(e));
  }
  *out = g;
  return GR_OK;
}

gr_status gr_multinomial_sample(gr_multinomial* g, gr_engine* e, int32_t* dev_out, size_t samples,
                                gr_stream_t stream) {
  if (need_four_lanes(e, "MultinomialGen") != GR_OK) return GR_ERR_UNSUPPORTED;
  if (!g || !e) return mv_fail(GR_ERR_INVALID, "NULL generator or engine");
  if (samples == 0) return GR_OK;
  if (!dev_out) return mv_fail(GR_ERR_INVALID, "output is NULL");
  if ((uintptr_t)dev_out % 16) return mv_fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  if (g->trials == 0) {  // no draws: every count is 0
    MV_CUDA(cudaMemsetAsync(dev_out, 0, sizeof(int32_t) * (size_t)g->dim * samples, s));
    return GR_OK;
  }
  const int K = gr_engine_streams(e);
  if (g->cond) {
    if (samples % 8)
      return mv_fail(GR_ERR_INVALID, "the conditional-binomial multinomial path needs samples % 8 == 0 "
                                     "(BinomialVGen<float> packets of 8 samples)");
    const int64_t gran = (int64_t)(samples / 8);
    Plan p{};
    p.eng = engine_state_ptr(e);
    p.K = K;
    p.gran = 8;
    p.gran_per_k = gran / K;
    p.gran_rem = gran % K;
    McArgs a{};
    a.p = g->pdev;
    a.rows = g->rows;
    a.dim = g->dim;
    a.trials = g->trials;
    a.out = dev_out;
    // Poisson loop about mean + 1 packets, tan rejection about 2.5 trials of
    // two packets; the cap is far above either
    const int64_t pk = (p.gran_per_k + 1) * (int64_t)g->rows;
    a.max_blocks = (pk * 64) / kN + 64;
    const cudaError_t err = launch_mn_cond(p, a, s);
    if (err != cudaSuccess) return mv_fail(GR_ERR_CUDA, std::string("multinomial kernel: ") + cudaGetErrorString(err));
    return GR_OK;
  }
  if (g->gst_K != K) {  // DiscreteGen cache per engine stream
    cudaFree(g->gst);
    g->gst = nullptr;
    g->gst_K = 0;
    MV_CUDA(cudaMalloc(&g->gst, sizeof(GenState) * (size_t)K));
    MV_CUDA(cudaMemsetAsync(g->gst, 0, sizeof(GenState) * (size_t)K, s));
    g->gst_K = K;
  }
  MnArgs a{};
  a.prob = g->table;
  a.alias = g->table + g->nprob;
  a.bitmask = g->bitmask;
  a.ncdf = g->ncdf;
  a.dim = g->dim;
  a.trials = g->trials;
  a.out = dev_out;
  return run_multinomial(e, g->gst, a, (int64_t)samples, s);
}

}  // extern "C"
