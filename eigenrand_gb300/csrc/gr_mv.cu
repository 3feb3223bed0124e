// Multivariate generators (EigenRand/MvDists): MvNormalGen, WishartGen,
// InvWishartGen, DirichletGen, MultinomialGen.
//
// The normal / chi-squared / gamma draws come from the univariate kernels, in
// the reference's call order, so their streams are the reference's.  This
// file holds the rest:
//   k_inverse_f64, k_chol_f64, k_jacobi_f64
//       the covariance / scale factor in FP64 on the GPU (MvNormal.h:21-38
//       get_lt: LLT, else the eigen decomposition V sqrt(max(lambda, 0))).
//   k_pack_lt     the factor rounded to float in mma.sync A-fragment order.
//   k_mvn_tc      X = L Z + mean, in place over Z, 3xTF32 on the tensor cores
//                 (MvNormal.h:103-108).
//   k_wishart_tc  Bartlett products T = chol A, W = T T^T (MvNormal.h:236-277)
//                 and the inverse form U = T^-1, W = U^T U (:400-442).
//   k_dirichlet   column normalisation of the K gamma rows (Multinomial.h:190-203).
//   k_multinomial trials alias / CDF draws per sample into a histogram, with
//                 DiscreteGen's packet cache and scalar tail reproduced
//                 (Multinomial.h:95-118, Discrete.h:420-485).
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_mt.cuh"
#include "gr_mv.cuh"

namespace gr {

__host__ __device__ __forceinline__ int64_t i64min(int64_t a, int64_t b) { return a < b ? a : b; }

// =================================================================== FP64 factorisation
// Matrices are col-major d x d in global memory; one CTA does the whole job
// (set-up work, O(d^3)).

// Gauss-Jordan inverse with partial pivoting: A is replaced by A^-1, W is
// d x d scratch.  status |= 1 when a pivot is zero.
__global__ void __launch_bounds__(1024) k_inverse_f64(double* A, double* W, int d, int32_t* status) {
  __shared__ int piv;
  __shared__ double red_v[32];
  __shared__ int red_i[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < d * d; t += nt) W[t] = ((t % d) == (t / d)) ? 1.0 : 0.0;
  __syncthreads();
  for (int j = 0; j < d; ++j) {
    // pivot: max |A[i][j]| for i >= j
    double bv = -1.0;
    int bi = j;
    for (int i = j + tid; i < d; i += nt) {
      const double v = fabs(A[(size_t)j * d + i]);
      if (v > bv) {
        bv = v;
        bi = i;
      }
    }
    for (int o = 16; o; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, bv, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if ((tid & 31) == 0) {
      red_v[tid >> 5] = bv;
      red_i[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < nt / 32; ++w)
        if (red_v[w] > red_v[0] || (red_v[w] == red_v[0] && red_i[w] < red_i[0])) {
          red_v[0] = red_v[w];
          red_i[0] = red_i[w];
        }
      piv = red_i[0];
      if (!(red_v[0] > 0.0)) *status |= 1;
    }
    __syncthreads();
    const int p = piv;
    if (p != j) {  // swap rows p and j of A and W
      for (int c = tid; c < 2 * d; c += nt) {
        double* M = c < d ? A : W;
        const int cc = c < d ? c : c - d;
        const double t = M[(size_t)cc * d + j];
        M[(size_t)cc * d + j] = M[(size_t)cc * d + p];
        M[(size_t)cc * d + p] = t;
      }
    }
    __syncthreads();
    const double pv = A[(size_t)j * d + j];
    const double inv = pv != 0.0 ? 1.0 / pv : 0.0;
    __syncthreads();
    for (int c = tid; c < 2 * d; c += nt) {  // scale row j
      double* M = c < d ? A : W;
      const int cc = c < d ? c : c - d;
      M[(size_t)cc * d + j] *= inv;
    }
    __syncthreads();
    // eliminate column j from the other rows (column j of A itself is
    // cleared afterwards, so the factors A[i][j] stay intact meanwhile)
    for (int t = tid; t < d * 2 * d; t += nt) {
      const int i = t % d, c = t / d;
      if (i == j || c == j) continue;
      double* M = c < d ? A : W;
      const int cc = c < d ? c : c - d;
      const double f = A[(size_t)j * d + i];
      M[(size_t)cc * d + i] -= f * M[(size_t)cc * d + j];
    }
    __syncthreads();
    for (int i = tid; i < d; i += nt)
      if (i != j) A[(size_t)j * d + i] = 0.0;
    __syncthreads();
  }
  for (int t = tid; t < d * d; t += nt) A[t] = W[t];
}

// Cholesky: the lower factor replaces A, the strict upper part is zeroed.
// status |= 2 when A is not positive definite.
__global__ void __launch_bounds__(1024) k_chol_f64(double* A, int d, int32_t* status) {
  __shared__ double diag;
  __shared__ int bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < d; ++j) {
    for (int i = j + tid; i < d; i += nt) {
      double s = A[(size_t)j * d + i];
      for (int k = 0; k < j; ++k) s -= A[(size_t)k * d + i] * A[(size_t)k * d + j];
      A[(size_t)j * d + i] = s;
    }
    __syncthreads();
    if (tid == 0) {
      const double s = A[(size_t)j * d + j];
      if (!(s > 0.0)) bad = 1;
      diag = s > 0.0 ? sqrt(s) : 1.0;
      A[(size_t)j * d + j] = diag;
    }
    __syncthreads();
    const double dj = diag;
    for (int i = j + 1 + tid; i < d; i += nt) A[(size_t)j * d + i] /= dj;
    __syncthreads();
    if (bad) break;  // uniform: read after the barrier
  }
  for (int t = tid; t < d * d; t += nt)
    if ((t % d) < (t / d)) A[t] = 0.0;
  if (tid == 0 && bad) *status |= 2;
}

// Symmetric eigen decomposition by parallel cyclic Jacobi (round-robin pair
// ordering, (d+1)/2 disjoint rotations per step).  A (symmetric) is
// overwritten; on return L = V diag(sqrt(max(lambda, 0))) is written to Lout.
// V is d x d scratch.  At most kJacobiSweeps sweeps; status |= 4 if the
// off-diagonal mass did not vanish.
constexpr int kJacobiSweeps = 40;
__global__ void __launch_bounds__(1024) k_jacobi_f64(double* A, double* V, double* Lout, int d, int32_t* status) {
  extern __shared__ double jsm[];  // c[np], s[np]
  __shared__ int pp_[1024], qq_[1024];
  __shared__ double red[32];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int m = d + (d & 1);
  const int np = m / 2;
  double* cs = jsm;
  double* sn = jsm + np;
  for (int t = tid; t < d * d; t += nt) V[t] = ((t % d) == (t / d)) ? 1.0 : 0.0;
  auto block_sum = [&](double v) -> double {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int w = 0; w < nt / 32; ++w) s += red[w];
    return s;
  };
  double tv = 0;
  for (int t = tid; t < d * d; t += nt) tv += A[t] * A[t];
  const double tot = block_sum(tv);
  bool converged = false;
  for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
    double v = 0;
    for (int t = tid; t < d * d; t += nt)
      if ((t % d) != (t / d)) v += A[t] * A[t];
    const double offn = block_sum(v);
    // RMS off-diagonal entry below ~1e-15 of the Frobenius norm (the
    // rounding floor of the rotations themselves)
    if (!(offn > 1e-30 * tot * (double)d * (double)d)) {
      converged = true;
      break;
    }
    for (int r = 0; r < m - 1; ++r) {
      // round r pairs player 0 with r % (m-1) + 1 and, for i >= 1,
      // (r+i) % (m-1) + 1 with (r-i) % (m-1) + 1; player d (odd d) sits out
      for (int i = tid; i < np; i += nt) {
        int p, q;
        if (i == 0) {
          p = 0;
          q = r % (m - 1) + 1;
        } else {
          p = (r + i) % (m - 1) + 1;
          q = (r - i + (m - 1)) % (m - 1) + 1;
        }
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, sv = 0.0;
        if (q < d) {
          const double apq = A[(size_t)q * d + p];
          if (apq != 0.0) {
            const double tau = (A[(size_t)q * d + q] - A[(size_t)p * d + p]) / (2.0 * apq);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            sv = t * c;
          }
        }
        pp_[i] = p;
        qq_[i] = q;
        cs[i] = c;
        sn[i] = sv;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int t = tid; t < np * d; t += nt) {
        const int i = t / d, k = t % d;
        const int p = pp_[i], q = qq_[i];
        if (q >= d || sn[i] == 0.0) continue;
        const double c = cs[i], sv = sn[i];
        const double akp = A[(size_t)p * d + k], akq = A[(size_t)q * d + k];
        A[(size_t)p * d + k] = c * akp - sv * akq;
        A[(size_t)q * d + k] = sv * akp + c * akq;
        const double vkp = V[(size_t)p * d + k], vkq = V[(size_t)q * d + k];
        V[(size_t)p * d + k] = c * vkp - sv * vkq;
        V[(size_t)q * d + k] = sv * vkp + c * vkq;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int t = tid; t < np * d; t += nt) {
        const int i = t / d, k = t % d;
        const int p = pp_[i], q = qq_[i];
        if (q >= d || sn[i] == 0.0) continue;
        const double c = cs[i], sv = sn[i];
        const double apk = A[(size_t)k * d + p], aqk = A[(size_t)k * d + q];
        A[(size_t)k * d + p] = c * apk - sv * aqk;
        A[(size_t)k * d + q] = sv * apk + c * aqk;
      }
      __syncthreads();
    }
  }
  for (int t = tid; t < d * d; t += nt) {
    const int col = t / d;
    const double lam = A[(size_t)col * d + col];
    Lout[t] = V[t] * sqrt(lam > 0.0 ? lam : 0.0);
  }
  if (tid == 0 && !converged) *status |= 4;
}

// =================================================================== L fragments
// Fragment (mt, ks) of the float factor: rows 16mt.., cols 8ks.., 32 lanes x 4
// values in mma.sync m16n8k8 A order (a0 (g, t), a1 (g+8, t), a2 (g, t+4),
// a3 (g+8, t+4); g = lane/4, t = lane%4).  Lower-triangular factors store
// only ks < min(2mt+2, KS); fragment (mt, ks) then sits at mt(mt+1) + ks
// (every m-tile but the last has 2mt + 2 <= KS fragments).
__global__ void k_pack_lt(const double* L, float* out, int d, int tri) {
  const int MT = (d + 15) / 16, KS = (d + 7) / 8;
  const int64_t nfr = tri ? mv_tri_frags(MT, KS) : (int64_t)MT * KS;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nfr * 128;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / 128;
    const int lane = (int)((t % 128) / 4), e = (int)(t % 4);
    int mt, ks;
    if (tri) {
      mt = 0;
      while (mt + 1 < MT && (int64_t)(mt + 1) * (mt + 2) <= f) ++mt;
      ks = (int)(f - (int64_t)mt * (mt + 1));
    } else {
      mt = (int)(f / KS);
      ks = (int)(f % KS);
    }
    const int g = lane >> 2, tq = lane & 3;
    const int row = 16 * mt + g + ((e & 1) ? 8 : 0);
    const int col = 8 * ks + tq + ((e & 2) ? 4 : 0);
    out[t] = (row < d && col < d) ? (float)L[(size_t)col * d + row] : 0.0f;
  }
}

__global__ void k_f64_to_f32(const double* a, float* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// =================================================================== tensor-core helpers
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  const float r = x - __uint_as_float(h);
  uint32_t l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  hi = h;
  lo = l;
}

__device__ __forceinline__ void mma_tf32(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// c += a * b with a, b split into tf32 hi + lo: lo*hi + hi*lo + hi*hi
__device__ __forceinline__ void mma_3xtf32(float* c, const uint32_t* ah, const uint32_t* al, const uint32_t* bh,
                                           const uint32_t* bl) {
  mma_tf32(c, al, bh);
  mma_tf32(c, ah, bl);
  mma_tf32(c, ah, bh);
}

// =================================================================== X = L Z + mean
// CTA: 8 warps as WM (m) x WN (n); a warp owns MTW m-tiles (stride WM) and NTW
// consecutive n-tiles.  Block of BN = 8 * NTW * WN samples; the Z block is
// staged in shared memory as Zs[sample][k] (row stride d_pad + 4: B fragment
// reads are bank-conflict free), replaced by the result, and written back
// over Z.  Persistent: CTAs stride over the sample blocks.
template <int WM, int WN, int MTW, int NTW, bool TRI>
__global__ void __launch_bounds__(256) k_mvn_tc(const float* __restrict__ Lf, const float* __restrict__ mean,
                                                float* X, int d, int64_t n) {
  constexpr int BN = 8 * NTW * WN;
  extern __shared__ float Zs[];
  const int MT = (d + 15) / 16, KS = (d + 7) / 8;
  const int dp = 16 * MT, ZS = dp + 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp % WM, wn = warp / WM;
  const int g = lane >> 2, tq = lane & 3;
  const int64_t nblk = (n + BN - 1) / BN;
  const bool vec = (d & 3) == 0 && ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(mean)) & 15) == 0;
  int ks_end = 0;
#pragma unroll
  for (int i = 0; i < MTW; ++i) {
    const int mt = wm + i * WM;
    if (mt < MT) ks_end = max(ks_end, TRI ? min(2 * mt + 2, KS) : KS);
  }
  for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t s0 = blk * BN;
    const int nv = (int)i64min(BN, n - s0);
    const float* src = X + s0 * d;
    // ---- stage Z (zero padded)
    if (vec) {
      const int q = d >> 2, qp = dp >> 2;
      for (int t = tid; t < BN * qp; t += 256) {
        const int c = t / qp, k4 = t % qp;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c < nv && k4 < q) v = reinterpret_cast<const float4*>(src)[(size_t)c * q + k4];
        *reinterpret_cast<float4*>(&Zs[c * ZS + 4 * k4]) = v;
      }
    } else {
      for (int t = tid; t < BN * dp; t += 256) {
        const int c = t / dp, k = t % dp;
        Zs[c * ZS + k] = (c < nv && k < d) ? src[(size_t)c * d + k] : 0.0f;
      }
    }
    __syncthreads();
    float acc[MTW][NTW][4];
#pragma unroll
    for (int i = 0; i < MTW; ++i)
#pragma unroll
      for (int j = 0; j < NTW; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0f;
    for (int ks = 0; ks < ks_end; ++ks) {
      uint32_t bh[NTW][2], bl[NTW][2];
#pragma unroll
      for (int j = 0; j < NTW; ++j) {
        const int c = (wn * NTW + j) * 8 + g;
        split_tf32(Zs[c * ZS + 8 * ks + tq], bh[j][0], bl[j][0]);
        split_tf32(Zs[c * ZS + 8 * ks + tq + 4], bh[j][1], bl[j][1]);
      }
#pragma unroll
      for (int i = 0; i < MTW; ++i) {
        const int mt = wm + i * WM;
        if (mt >= MT) continue;
        if (TRI && ks >= min(2 * mt + 2, KS)) continue;
        const int64_t fr = TRI ? (int64_t)mt * (mt + 1) + ks : (int64_t)mt * KS + ks;
        const float4 av = __ldg(reinterpret_cast<const float4*>(Lf) + fr * 32 + lane);
        uint32_t ah[4], al[4];
        split_tf32(av.x, ah[0], al[0]);
        split_tf32(av.y, ah[1], al[1]);
        split_tf32(av.z, ah[2], al[2]);
        split_tf32(av.w, ah[3], al[3]);
#pragma unroll
        for (int j = 0; j < NTW; ++j) mma_3xtf32(acc[i][j], ah, al, bh[j], bl[j]);
      }
    }
    __syncthreads();  // every warp is done reading Z
#pragma unroll
    for (int i = 0; i < MTW; ++i) {
      const int mt = wm + i * WM;
      if (mt >= MT) continue;
#pragma unroll
      for (int j = 0; j < NTW; ++j) {
        const int r = 16 * mt + g, c = (wn * NTW + j) * 8 + 2 * tq;
        Zs[c * ZS + r] = acc[i][j][0];
        Zs[(c + 1) * ZS + r] = acc[i][j][1];
        Zs[c * ZS + r + 8] = acc[i][j][2];
        Zs[(c + 1) * ZS + r + 8] = acc[i][j][3];
      }
    }
    __syncthreads();
    float* dst = X + s0 * d;
    if (vec) {
      const int q = d >> 2;
      for (int t = tid; t < nv * q; t += 256) {
        const int c = t / q, k4 = t % q;
        float4 v = *reinterpret_cast<const float4*>(&Zs[c * ZS + 4 * k4]);
        const float4 mu = __ldg(reinterpret_cast<const float4*>(mean) + k4);
        v.x += mu.x;
        v.y += mu.y;
        v.z += mu.z;
        v.w += mu.w;
        reinterpret_cast<float4*>(dst)[(size_t)c * q + k4] = v;
      }
    } else {
      for (int t = tid; t < nv * d; t += 256) {
        const int c = t / d, k = t % d;
        dst[(size_t)c * d + k] = Zs[c * ZS + k] + __ldg(mean + k);
      }
    }
    __syncthreads();
  }
}

// FP64 generators: plain FP64 FMAs (the FP64 tensor rate of this part is no
// faster).  One CTA per block of 32 samples; Z block in shared memory.
__global__ void __launch_bounds__(256) k_mvn_f64(const double* __restrict__ L, const double* __restrict__ mean,
                                                 double* X, int d, int64_t n, int tri) {
  extern __shared__ double Zd[];
  const int64_t s0 = (int64_t)blockIdx.x * 32;
  const int nv = (int)i64min(32, n - s0);
  double* col = X + s0 * d;
  for (int t = threadIdx.x; t < nv * d; t += blockDim.x) Zd[t] = col[t];
  __syncthreads();
  for (int t = threadIdx.x; t < nv * d; t += blockDim.x) {
    const int c = t / d, r = t % d;
    const int kend = tri ? r + 1 : d;
    double s = 0.0;
    for (int k = 0; k < kend; ++k) s = fma(__ldg(L + (size_t)k * d + r), Zd[c * d + k], s);
    col[t] = s + __ldg(mean + r);
  }
}

// =================================================================== Wishart
// Per draw j:  A = strictly-lower normals (column by column, MvNormal.h:243-251)
// + diagonal sqrt(chi^2(df - i)) (:253-261);  T = chol A;
//   Wishart:     W = T T^T
//   InvWishart:  U = (lower part of T)^-1,  W = U^T U
// Tensor path (float, d <= 128): 4 warps per CTA, one draw at a time per CTA,
// matrices in shared memory stored so that both mma operands read
// k-contiguous rows: Cr = chol row-major, As = A col-major, Tr = T row-major
// (T is both operands of T T^T), U col-major.  Row stride ld = dp + 4 (dp =
// d rounded up to 16): fragment reads are bank-conflict free.
constexpr int kWishThreads = 128;

// Cout(r, c) = sum_k Am[r*ld + k] * Bm[c*ld + k] over dp x dp, 3xTF32
__device__ __forceinline__ void wish_gemm(const float* Am, const float* Bm, float* Cout, int dp, int ld,
                                          bool out_colmajor) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  const int MT = dp / 16, NT = dp / 8, KS = dp / 8;
  for (int tile = warp; tile < MT * NT; tile += kWishThreads / 32) {
    const int mt = tile / NT, nt = tile % NT;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int ks = 0; ks < KS; ++ks) {
      uint32_t ah[4], al[4], bh[2], bl[2];
      const int r = 16 * mt + g, k = 8 * ks + tq, c = 8 * nt + g;
      split_tf32(Am[r * ld + k], ah[0], al[0]);
      split_tf32(Am[(r + 8) * ld + k], ah[1], al[1]);
      split_tf32(Am[r * ld + k + 4], ah[2], al[2]);
      split_tf32(Am[(r + 8) * ld + k + 4], ah[3], al[3]);
      split_tf32(Bm[c * ld + k], bh[0], bl[0]);
      split_tf32(Bm[c * ld + k + 4], bh[1], bl[1]);
      mma_3xtf32(acc, ah, al, bh, bl);
    }
    const int r = 16 * mt + g, c = 8 * nt + 2 * tq;
    if (out_colmajor) {
      Cout[c * ld + r] = acc[0];
      Cout[(c + 1) * ld + r] = acc[1];
      Cout[c * ld + r + 8] = acc[2];
      Cout[(c + 1) * ld + r + 8] = acc[3];
    } else {
      Cout[r * ld + c] = acc[0];
      Cout[r * ld + c + 1] = acc[1];
      Cout[(r + 8) * ld + c] = acc[2];
      Cout[(r + 8) * ld + c + 1] = acc[3];
    }
  }
}

__global__ void __launch_bounds__(kWishThreads)
    k_wishart_tc(const float* __restrict__ normals, const float* __restrict__ chis, const float* __restrict__ chol,
                 float* __restrict__ out, int d, int64_t samples, int inverse) {
  extern __shared__ float wsm[];
  const int dp = (d + 15) / 16 * 16, ld = dp + 4;
  float* Cr = wsm;
  float* As = wsm + dp * ld;  // A (col-major), then W (col-major)
  float* Tr = wsm + 2 * dp * ld;
  const int tid = threadIdx.x;
  const int64_t nper = (int64_t)d * (d - 1) / 2;
  for (int t = tid; t < dp * ld; t += kWishThreads) {
    const int r = t / ld, k = t % ld;
    Cr[t] = (r < d && k < d) ? chol[(size_t)k * d + r] : 0.0f;
  }
  for (int64_t j = blockIdx.x; j < samples; j += gridDim.x) {
    __syncthreads();
    for (int t = tid; t < dp * ld; t += kWishThreads) {
      const int col = t / ld, row = t % ld;
      float v = 0.0f;
      if (row < d && col < d) {
        if (row > col) {
          const int before = col * (d - 1) - col * (col - 1) / 2;
          v = normals[j * nper + before + (row - col - 1)];
        } else if (row == col) {
          v = sqrtf(chis[(int64_t)row * samples + j]);
        }
      }
      As[t] = v;
    }
    __syncthreads();
    wish_gemm(Cr, As, Tr, dp, ld, false);  // T = chol A, row-major
    __syncthreads();
    if (!inverse) {
      wish_gemm(Tr, Tr, As, dp, ld, true);  // W = T T^T, col-major
    } else {
      // U = T^-1 (lower triangle of T), column c by forward substitution:
      // U[i][c] = (delta_ic - sum_{c<=k<i} T[i][k] U[k][c]) / T[i][i]
      for (int c = tid; c < dp; c += kWishThreads) {
        float* u = As + c * ld;  // U col-major
        for (int i = 0; i < dp; ++i) {
          float v = 0.0f;
          if (i < d && c < d && i >= c) {
            float s = (i == c) ? 1.0f : 0.0f;
            for (int k = c; k < i; ++k) s -= Tr[i * ld + k] * u[k];
            v = s / Tr[i * ld + i];
          }
          u[i] = v;
        }
      }
      __syncthreads();
      // W = U^T U: both operands read U col-major as [r][k] = U[k][r]
      wish_gemm(As, As, Tr, dp, ld, true);
      __syncthreads();
      for (int t = tid; t < dp * ld; t += kWishThreads) As[t] = Tr[t];
    }
    __syncthreads();
    float* o = out + j * (int64_t)d * d;
    for (int t = tid; t < d * d; t += kWishThreads) {
      const int c = t / d, r = t % d;
      o[t] = As[c * ld + r];
    }
  }
}

// SIMT form for FP64 and for float above the tensor path's size: A and T in
// shared memory, chol read through L1.
template <typename T>
__global__ void __launch_bounds__(256)
    k_wishart_simt(const T* __restrict__ normals, const T* __restrict__ chis, const T* __restrict__ chol,
                   T* __restrict__ out, int d, int64_t samples, int inverse) {
  extern __shared__ unsigned char wsm_raw[];
  T* As = reinterpret_cast<T*>(wsm_raw);  // col-major
  T* Ts = As + (size_t)d * d;              // col-major
  const int tid = threadIdx.x, nt = blockDim.x;
  const int64_t nper = (int64_t)d * (d - 1) / 2;
  for (int64_t j = blockIdx.x; j < samples; j += gridDim.x) {
    __syncthreads();
    for (int t = tid; t < d * d; t += nt) {
      const int col = t / d, row = t % d;
      T v = 0;
      if (row > col) {
        const int before = col * (d - 1) - col * (col - 1) / 2;
        v = normals[j * nper + before + (row - col - 1)];
      } else if (row == col) {
        v = sqrt(chis[(int64_t)row * samples + j]);
      }
      As[t] = v;
    }
    __syncthreads();
    for (int t = tid; t < d * d; t += nt) {
      const int col = t / d, row = t % d;
      T s = 0;
      for (int k = 0; k < d; ++k) s = fma(__ldg(chol + (size_t)k * d + row), As[col * d + k], s);
      Ts[t] = s;
    }
    __syncthreads();
    T* o = out + j * (int64_t)d * d;
    if (!inverse) {
      for (int t = tid; t < d * d; t += nt) {
        const int col = t / d, row = t % d;
        T s = 0;
        for (int k = 0; k < d; ++k) s = fma(Ts[k * d + row], Ts[k * d + col], s);
        o[t] = s;
      }
    } else {
      for (int c = tid; c < d; c += nt) {  // U col-major into As
        T* u = As + (size_t)c * d;
        for (int i = 0; i < d; ++i) {
          T v = 0;
          if (i >= c) {
            T s = (i == c) ? T(1) : T(0);
            for (int k = c; k < i; ++k) s -= Ts[k * d + i] * u[k];
            v = s / Ts[i * d + i];
          }
          u[i] = v;
        }
      }
      __syncthreads();
      for (int t = tid; t < d * d; t += nt) {
        const int col = t / d, row = t % d;
        T s = 0;
        for (int k = 0; k < d; ++k) s = fma(As[row * d + k], As[col * d + k], s);
        o[t] = s;
      }
    }
  }
}

// =================================================================== Dirichlet
// rows: K x n row-major (category i's gamma draws in row i); out: K x n
// col-major.  Tile of 32 samples: coalesced row reads, one column sum per
// sample, contiguous writes of 32 K-vectors.
template <typename T>
__global__ void __launch_bounds__(256) k_dirichlet(const T* __restrict__ rows, T* __restrict__ out, int K, int64_t n) {
  extern __shared__ unsigned char dsm_raw[];
  T* tile = reinterpret_cast<T*>(dsm_raw);  // [K][33]
  T* tot = tile + (size_t)K * 33;            // [32]
  const int64_t s0 = (int64_t)blockIdx.x * 32;
  const int nv = (int)i64min(32, n - s0);
  const int tid = threadIdx.x;
  for (int t = tid; t < K * 32; t += blockDim.x) {
    const int i = t / 32, c = t % 32;
    tile[i * 33 + c] = c < nv ? rows[(int64_t)i * n + s0 + c] : T(1);
  }
  __syncthreads();
  if (tid < 32) {
    T s = 0;
    for (int i = 0; i < K; ++i) s += tile[i * 33 + tid];
    tot[tid] = s;
  }
  __syncthreads();
  T* o = out + s0 * K;
  for (int t = tid; t < nv * K; t += blockDim.x) {
    const int c = t / K, i = t % K;
    o[t] = tile[i * 33 + c] / tot[c];
  }
}

// =================================================================== Multinomial
// Word layout per engine slice: see MnLayout (gr_mv.cuh).  A packet draw with
// DiscreteGen's cache empty takes a new rng() packet, returns the categories
// of its words 0..3 and caches those of 4..7; with the cache full it returns
// the cache.  A scalar draw takes a whole packet and uses word 0 through the
// scalar operator() (Discrete.h:420-441), whose comparisons differ from the
// packet path's.
__device__ __forceinline__ int32_t mn_packet_cat(uint32_t rx, const MnArgs& a) {
  if (a.ncdf > 0) {
    const int32_t x = (int32_t)(rx & 0x7fffffffu);
    int32_t r = a.ncdf - 1;
    for (int i = 0; i < a.ncdf - 1; ++i) r += (x < __ldg(a.prob + i)) ? -1 : 0;
    return r;
  }
  const int32_t albit = (int32_t)(rx & a.bitmask);
  return ((int32_t)(rx >> 1) < __ldg(a.prob + albit)) ? albit : __ldg(a.alias + albit);
}
__device__ __forceinline__ int32_t mn_scalar_cat(uint32_t w, const MnArgs& a) {
  const int32_t rx = (int32_t)w;
  if (a.ncdf > 0) {  // std::lower_bound over the uint32 cdf[0 .. n-2]
    const uint32_t x = (uint32_t)(rx & 0x7fffffff);
    int32_t r = 0;
    for (int i = 0; i < a.ncdf - 1; ++i) r += ((uint32_t)__ldg(a.prob + i) < x) ? 1 : 0;
    return r;
  }
  const int32_t albit = rx & (int32_t)a.bitmask;
  const uint32_t alx = (uint32_t)(rx >> 1);  // arithmetic shift of the signed draw
  return (alx < (uint32_t)__ldg(a.prob + albit)) ? albit : __ldg(a.alias + albit);
}

constexpr int kMnThreads = 160;

// CTA per (engine k, jump segment s); one warp per sample, lanes over trials,
// a shared-memory histogram per warp.  A sample is counted in the block step
// that generates its last packet; the two-block ring then still holds all of
// its words and the half packet its first draw may take from the sample
// before (host guarantees words per sample <= kMnMaxSampleWords).
__global__ void __launch_bounds__(kMnThreads) k_multinomial(Plan p, MnArgs a, const CallSnap* snap) {
  __shared__ uint64_t raw[2][kLanes][kN];
  __shared__ uint64_t tp[2][kN][kLanes];
  __shared__ int32_t cat0[4];
  extern __shared__ int32_t hist[];  // (kMnThreads / 32) x dim
  const int k = blockIdx.x / p.S, s = blockIdx.x % p.S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  EngState* st = p.eng + k;
  GenState* gs = p.gen + k;
  const int64_t g0 = (int64_t)k * p.gran_per_k + min((int64_t)k, p.gran_rem);
  const int64_t ng = p.gran_per_k + ((int64_t)k < p.gran_rem ? 1 : 0);  // samples of engine k
  if (ng == 0) return;
  const int c0 = p.S > 1 ? (snap[k].gen_valid ? 1 : 0) : (gs->s[0].valid ? 1 : 0);
  const MnLayout L = mn_layout(a.trials, c0);
  const int64_t i_beg = (int64_t)s * a.Us * L.spu;
  if (i_beg >= ng) return;
  const int64_t i_end = min(i_beg + a.Us * L.spu, ng);
  const bool last = (i_end == ng);
  const int64_t seg_p0 = (int64_t)s * p.J;  // == mn_base(L, i_beg) / 8
  const int64_t np_seg = mn_base(L, i_end) / 8 - seg_p0;

  if (s == 0 && p.S > 1) load_window(raw[0], p.prefix + (size_t)k * kLanes * kPrefixLen, kPrefixLen);
  else if (s == 0) load_window(raw[0], &st->win[0][0], kN);
  else load_window(raw[0], p.segwin + ((size_t)k * (p.S - 1) + (s - 1)) * kLanes * kN, kN);
  __syncthreads();
  // categories cached before the first sample (used if it starts in state 1)
  if (tid < 4) {
    int32_t v = 0;
    if (L.nP > 0 && mn_state(L, i_beg) == 1) {
      if (s == 0) {
        v = p.S > 1 ? (int32_t)snap[k].gen_cache[tid] : (int32_t)gs->s[0].cache[tid];
      } else {
        // the previous sample's cached half packet lies 1 + ns <= 4 packets
        // before the segment: rebuild it from the raw window
        const int64_t wc = mn_base(L, i_beg - 1) + mn_cache_off(L, mn_state(L, i_beg - 1));
        const int back = (int)(seg_p0 - (wc >> 3));
        const uint64_t rv = mt_temper(raw[0][2 + (tid >> 1)][kN - back]);
        v = mn_packet_cat((tid & 1) ? (uint32_t)(rv >> 32) : (uint32_t)rv, a);
      }
    }
    cat0[tid] = v;
  }
  __syncthreads();

  int64_t ring_new = 0;  // newest ring block's first packet (ring_packet)
  int ring_slot = 0;
  auto word = [&](int64_t w) -> uint32_t {  // slice word w, present in the ring
    const int64_t rel = (w >> 3) - seg_p0;
    const uint64_t v = ring_packet(tp, rel, ring_new, ring_slot)[(w & 7) >> 1];
    return (w & 1) ? (uint32_t)(v >> 32) : (uint32_t)v;
  };
  int32_t* h = hist + warp * a.dim;
  // count samples [lo, hi) (every word they use is in the ring)
  auto count = [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo + warp; i < hi; i += kMnThreads / 32) {
      for (int b = lane; b < a.dim; b += 32) h[b] = 0;
      __syncwarp();
      const int c = mn_state(L, i);
      const int64_t b0 = mn_base(L, i);
      const int64_t cw = (c == 1 && i > i_beg) ? mn_base(L, i - 1) + mn_cache_off(L, mn_state(L, i - 1)) : -1;
      const int64_t bs = b0 + mn_scalar_off(L, c);
      for (int t = lane; t < a.trials; t += 32) {
        int32_t cat;
        if (t < 4 * L.nP) {
          const int kk = t >> 2, e = t & 3;
          if (c == 0) cat = mn_packet_cat(word(b0 + 4 * kk + e), a);
          else if (kk == 0) cat = (cw >= 0) ? mn_packet_cat(word(cw + e), a) : cat0[e];
          else cat = mn_packet_cat(word(b0 + 4 * (kk - 1) + e), a);
        } else {
          cat = mn_scalar_cat(word(bs + 8 * (t - 4 * L.nP)), a);
        }
        if ((unsigned)cat < (unsigned)a.dim) atomicAdd(&h[cat], 1);
        else atomicOr(&st->status, (int32_t)GR_DEV_BAD_INPUT);  // table slot outside the categories
      }
      __syncwarp();
      int32_t* o = a.out + (g0 + i) * (int64_t)a.dim;
      for (int b = lane; b < a.dim; b += 32) o[b] = h[b];
      __syncwarp();
    }
  };
  int64_t i_next = i_beg;
  int cur = 0;
  const int64_t nblk = (np_seg + kN - 1) / kN;
  for (int64_t nb = 0; nb < nblk; ++nb) {
    const int slot = (int)(nb & 1);
    mt_block(raw[cur], raw[cur ^ 1], [&](int i, const uint64_t* pk) {
#pragma unroll
      for (int l = 0; l < kLanes; ++l) tp[slot][i][l] = pk[l];
    });
    cur ^= 1; ring_new = nb * kN; ring_slot = slot;
    const int64_t wavail = (seg_p0 + (nb + 1) * kN) * 8;  // words [.., wavail) exist
    int64_t i_ready = i_next;
    while (i_ready < i_end && mn_base(L, i_ready + 1) <= wavail) ++i_ready;
    count(i_next, i_ready);
    i_next = i_ready;
    __syncthreads();
  }
  // samples that take no new packet (a trailing state-1 sample of 4 trials)
  if (i_next < i_end) {
    count(i_next, i_end);
    __syncthreads();
  }

  if (last) {
    if (np_seg > 0) {
      const int rr = (int)(np_seg - (nblk - 1) * kN);
      store_window(st, raw[cur], raw[cur ^ 1], rr);
    }
    if (tid < 4 && L.nP > 0) {
      const int cf = mn_state(L, ng);  // state after the last sample
      if (cf == 1) {
        const int64_t wc = mn_base(L, ng - 1) + mn_cache_off(L, mn_state(L, ng - 1));
        gs->s[0].cache[tid] = (uint32_t)mn_packet_cat(word(wc + tid), a);
      }
      if (tid == 0) gs->s[0].valid = cf;
    }
    if (tid == 0) st->consumed += (uint64_t)(mn_base(L, ng) / 8);
  }
}

// =================================================================== launchers
cudaError_t launch_inverse_f64(double* A, double* W, int d, int32_t* status, cudaStream_t s) {
  k_inverse_f64<<<1, 1024, 0, s>>>(A, W, d, status);
  return cudaGetLastError();
}
cudaError_t launch_chol_f64(double* A, int d, int32_t* status, cudaStream_t s) {
  k_chol_f64<<<1, 1024, 0, s>>>(A, d, status);
  return cudaGetLastError();
}
cudaError_t launch_jacobi_f64(double* A, double* V, double* L, int d, int32_t* status, cudaStream_t s) {
  if (d > kMvMaxDim) return cudaErrorInvalidValue;
  const size_t smem = (size_t)(d + 1) * sizeof(double);  // c and s for (d+1)/2 pairs each
  k_jacobi_f64<<<1, 1024, smem, s>>>(A, V, L, d, status);
  return cudaGetLastError();
}
cudaError_t launch_pack_lt(const double* L, float* out, int d, int tri, cudaStream_t s) {
  k_pack_lt<<<256, 256, 0, s>>>(L, out, d, tri);
  return cudaGetLastError();
}
cudaError_t launch_f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t s) {
  k_f64_to_f32<<<(unsigned)i64min((n + 255) / 256, 4096), 256, 0, s>>>(a, b, n);
  return cudaGetLastError();
}

namespace {
int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n = v > 0 ? v : 1;
  }
  return n;
}

template <int WM, int WN, int MTW, int NTW, bool TRI>
cudaError_t run_mvn(const float* Lf, const float* mean, float* X, int d, int64_t n, cudaStream_t s) {
  constexpr int BN = 8 * NTW * WN;
  const int dp = (d + 15) / 16 * 16;
  const size_t smem = (size_t)BN * (dp + 4) * sizeof(float);
  auto kern = k_mvn_tc<WM, WN, MTW, NTW, TRI>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  if (e != cudaSuccess) return e;
  const int64_t nblk = (n + BN - 1) / BN;
  const int64_t grid = i64min(nblk, (int64_t)num_sms() * (per_sm > 1 ? per_sm : 1));
  kern<<<(unsigned)grid, 256, smem, s>>>(Lf, mean, X, d, n);
  return cudaGetLastError();
}

template <bool TRI>
cudaError_t mvn_dispatch(const float* Lf, const float* mean, float* X, int d, int64_t n, cudaStream_t s) {
  const int MT = (d + 15) / 16;
  if (MT <= 1) return run_mvn<1, 8, 1, 8, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 2) return run_mvn<2, 4, 1, 8, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 4) return run_mvn<4, 2, 1, 8, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 8) return run_mvn<8, 1, 1, 8, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 16) return run_mvn<8, 1, 2, 8, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 32) return run_mvn<8, 1, 4, 4, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 64) return run_mvn<8, 1, 8, 2, TRI>(Lf, mean, X, d, n, s);
  if (MT <= 128) return run_mvn<8, 1, 16, 1, TRI>(Lf, mean, X, d, n, s);
  return cudaErrorInvalidValue;
}
}  // namespace

cudaError_t launch_mvn(const float* Lf, int tri, const float* mean, float* X, int d, int64_t n, cudaStream_t s) {
  return tri ? mvn_dispatch<true>(Lf, mean, X, d, n, s) : mvn_dispatch<false>(Lf, mean, X, d, n, s);
}

cudaError_t launch_mvn_f64(const double* L, int tri, const double* mean, double* X, int d, int64_t n,
                           cudaStream_t s) {
  const size_t smem = (size_t)32 * d * sizeof(double);
  if (smem > kMvMaxSmem) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_mvn_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_mvn_f64<<<(unsigned)((n + 31) / 32), 256, smem, s>>>(L, mean, X, d, n, tri);
  return cudaGetLastError();
}

size_t wishart_smem(int d, int dtype) {
  if (dtype == GR_F32 && d <= kWishTcMaxDim) {
    const int dp = (d + 15) / 16 * 16;
    return (size_t)3 * dp * (dp + 4) * sizeof(float);
  }
  return (size_t)2 * d * d * (dtype == GR_F32 ? sizeof(float) : sizeof(double));
}

cudaError_t launch_wishart(const void* normals, const void* chis, const void* chol, void* out, int d, int64_t samples,
                           int inverse, int dtype, cudaStream_t s) {
  const size_t smem = wishart_smem(d, dtype);
  if (smem > kMvMaxSmem) return cudaErrorInvalidValue;
  const int64_t grid = i64min(samples, (int64_t)num_sms() * 8);
  if (dtype == GR_F32 && d <= kWishTcMaxDim) {
    cudaError_t e = cudaFuncSetAttribute(k_wishart_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_wishart_tc<<<(unsigned)grid, kWishThreads, smem, s>>>((const float*)normals, (const float*)chis,
                                                            (const float*)chol, (float*)out, d, samples, inverse);
  } else if (dtype == GR_F32) {
    cudaError_t e =
        cudaFuncSetAttribute(k_wishart_simt<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_wishart_simt<float><<<(unsigned)grid, 256, smem, s>>>((const float*)normals, (const float*)chis,
                                                           (const float*)chol, (float*)out, d, samples, inverse);
  } else {
    cudaError_t e =
        cudaFuncSetAttribute(k_wishart_simt<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_wishart_simt<double><<<(unsigned)grid, 256, smem, s>>>((const double*)normals, (const double*)chis,
                                                            (const double*)chol, (double*)out, d, samples,
                                                            inverse);
  }
  return cudaGetLastError();
}

size_t dirichlet_smem(int K, int dtype) {
  return ((size_t)K * 33 + 32) * (dtype == GR_F32 ? sizeof(float) : sizeof(double));
}

cudaError_t launch_dirichlet(const void* rows, void* out, int K, int64_t n, int dtype, cudaStream_t s) {
  const size_t smem = dirichlet_smem(K, dtype);
  if (smem > kMvMaxSmem) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((n + 31) / 32);
  if (dtype == GR_F32) {
    cudaError_t e = cudaFuncSetAttribute(k_dirichlet<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_dirichlet<float><<<grid, 256, smem, s>>>((const float*)rows, (float*)out, K, n);
  } else {
    cudaError_t e =
        cudaFuncSetAttribute(k_dirichlet<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_dirichlet<double><<<grid, 256, smem, s>>>((const double*)rows, (double*)out, K, n);
  }
  return cudaGetLastError();
}

cudaError_t launch_multinomial(const Plan& p, const MnArgs& a, const CallSnap* snap, cudaStream_t s) {
  const size_t smem = (size_t)(kMnThreads / 32) * a.dim * sizeof(int32_t);
  if (smem > 160 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_multinomial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_multinomial<<<p.K * p.S, kMnThreads, smem, s>>>(p, a, snap);
  return cudaGetLastError();
}

}  // namespace gr
