// C ABI of libgpurand.so (declared in include/gpurand.h).
//
// Host-side planning for one call: split the output over the engine's
// sub-engines (streams), split a long single-engine call into jump-ahead
// segments, compute the generator's constants exactly as the reference
// constructor does, and launch the kernels.  Nothing here touches sample data.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <random>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_mv.cuh"
#include "gr_poly.h"

using namespace gr;

namespace {

thread_local std::string g_err;

gr_status fail(gr_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

gr_status cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return GR_ERR_CUDA;
}

#define GR_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// Jump polynomials x^(s*J - delta) mod P for s = 1..count, per device,
// cached by (J, delta).
struct JumpCache {
  std::mutex mu;
  struct Entry {
    uint64_t* dev = nullptr;
    int count = 0;
  };
  std::map<std::tuple<int, int64_t, int>, Entry> tab;
};
JumpCache& jump_cache() {
  static JumpCache c;
  return c;
}

gr_status get_jump_polys(int dev, int64_t J, int delta, int need, const uint64_t** out) {
  JumpCache& jc = jump_cache();
  std::lock_guard<std::mutex> lk(jc.mu);
  auto& ent = jc.tab[std::make_tuple(dev, J, delta)];
  if (ent.count < need) {
    // every entry is made at full size (127 = the most segments a call uses)
    // so a buffer that running kernels may read is never replaced
    const int cnt = std::max({need, 2 * ent.count, 127});
    std::vector<uint64_t> exps(cnt);
    for (int s = 0; s < cnt; ++s) exps[s] = (uint64_t)(s + 1) * (uint64_t)J - (uint64_t)delta;
    if (charpoly_terms().size() != 284) return fail(GR_ERR_CUDA, "MT19937-64 characteristic polynomial recovery failed");
    std::vector<Poly> polys;
    pow_x_mod_many(exps, polys);
    uint64_t* d = nullptr;
    GR_CUDA(cudaMalloc(&d, sizeof(uint64_t) * kPolyWords * (size_t)cnt));
    GR_CUDA(cudaMemcpy(d, polys.data(), sizeof(uint64_t) * kPolyWords * (size_t)cnt, cudaMemcpyHostToDevice));
    if (ent.dev) cudaFree(ent.dev);
    ent.dev = d;
    ent.count = cnt;
  }
  *out = ent.dev;
  return GR_OK;
}

}  // namespace

struct gr_engine {
  int K = 1;
  int lanes = 4;  // 4: AVX2 profile (Packet8i); 2: SSE / NEON profile (Packet4i)
  int device = 0;
  uint64_t seed = 0;
  EngState* st = nullptr;
  // scratch for segmented (jump-ahead) calls
  uint64_t* prefix = nullptr;
  uint64_t* segwin = nullptr;
  size_t segwin_words = 0;
  CallSnap* snap = nullptr;
  GenState* scratch_gen = nullptr;  // caches of temporary generators (gr_sample)
  uint64_t* tailw = nullptr;        // draws of a call's partial last packet
};

struct gr_gen {
  gr_dist_desc desc{};
  std::vector<double> weights;
  DistParams dp{};
  int32_t* table = nullptr;  // prob + alias (or cdf)
  GenState* gst = nullptr;
  int gst_K = 0;
  // TruncGen over a base without a closed-form inverse CDF (Truncated.h:
  // 202-263): the base generator it holds, its support in the scalar type,
  // the carried lanes of its CompressMask, and the accepted-lane counts seen
  // so far (they size the next chunk of base packets)
  gr_gen* trunc_base = nullptr;
  GenSlot* trunc_carry = nullptr;
  double trunc_lo = 0, trunc_hi = 0;
  int64_t trunc_lanes = 0, trunc_acc = 0;
};

// A scalar engine as EigenRand's Urng.  std::mt19937_64(seed) is lane 0 of
// Vmt19937_64(seed) (PacketRandomEngine.h:230-239 seeds lane l with seed +
// l): a one-stream packet engine whose lane-0 words are the stream.
// P8_mt19937_64(seed) (:600-607) hands out the four lanes of a packet of
// Vmt19937_64(seed) and then of Vmt19937_64(seed + 4) in turn (:465-496): a
// two-stream packet engine (streams seed + 4k) plus the eight lanes being
// handed out and how many are gone.
struct gr_sengine {
  int kind = 0;
  gr_engine* eng = nullptr;
  uint64_t* pbuf = nullptr;  // P8: the current eight lanes (device)
  int cnt = 8;               // P8: lanes of pbuf handed out (8: none left)
};

namespace gr {
EngState* engine_state_ptr(gr_engine* e) { return e ? e->st : nullptr; }
gr_status need_four_lanes(const gr_engine* e, const char* what) {
  if (e && e->lanes != kLanes)
    return set_last_error(GR_ERR_UNSUPPORTED, std::string(what) + ": needs the 4-lane Vmt19937_64 (AVX2 profile)");
  return GR_OK;
}
gr_status set_last_error(gr_status s, const std::string& msg) { return fail(s, msg); }
}  // namespace gr

extern "C" {

const char* gr_last_error(void) { return g_err.c_str(); }
const char* gr_version(void) { return "gpurand 0.1 (sm_103a; EigenRand 0.6.0 AVX2/Eigen-3.4 stream profile)"; }

gr_status gr_engine_create(gr_engine** out, uint64_t seed, int32_t lanes, int32_t streams) {
  if (!out) return fail(GR_ERR_INVALID, "out is NULL");
  if (lanes != kLanes && lanes != 2)
    return fail(GR_ERR_UNSUPPORTED, "lanes must be 4 (AVX2 Vmt19937_64) or 2 (SSE / NEON Vmt19937_64)");
  if (streams < 1 || streams > (1 << 20)) return fail(GR_ERR_INVALID, "streams must be in [1, 2^20]");
  gr_engine* e = new gr_engine;
  e->K = streams;
  e->lanes = lanes;
  e->seed = seed;
  cudaGetDevice(&e->device);
  cudaError_t err = cudaMalloc(&e->st, sizeof(EngState) * (size_t)streams);
  if (err != cudaSuccess) {
    delete e;
    return cuda_fail(err, "cudaMalloc(engine state)");
  }
  err = launch_seed(e->st, e->K, seed, nullptr);
  if (err == cudaSuccess) err = cudaStreamSynchronize(nullptr);
  if (err != cudaSuccess) {
    cudaFree(e->st);
    delete e;
    return cuda_fail(err, "seed kernel");
  }
  *out = e;
  return GR_OK;
}

gr_status gr_engine_destroy(gr_engine* e) {
  if (!e) return GR_OK;
  cudaFree(e->st);
  cudaFree(e->prefix);
  cudaFree(e->segwin);
  cudaFree(e->snap);
  cudaFree(e->scratch_gen);
  cudaFree(e->tailw);
  delete e;
  return GR_OK;
}

gr_status gr_engine_seed(gr_engine* e, uint64_t seed, gr_stream_t stream) {
  if (!e) return fail(GR_ERR_INVALID, "engine is NULL");
  e->seed = seed;
  GR_CUDA(launch_seed(e->st, e->K, seed, (cudaStream_t)stream));
  return GR_OK;
}

int32_t gr_engine_streams(const gr_engine* e) { return e ? e->K : 0; }

size_t gr_engine_state_size(const gr_engine* e) { return e ? sizeof(EngState) * (size_t)e->K : 0; }

gr_status gr_engine_save(const gr_engine* e, void* host_buf, size_t size, gr_stream_t stream) {
  if (!e || !host_buf) return fail(GR_ERR_INVALID, "NULL argument");
  if (size < gr_engine_state_size(e)) return fail(GR_ERR_INVALID, "buffer too small");
  GR_CUDA(cudaMemcpyAsync(host_buf, e->st, gr_engine_state_size(e), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  GR_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return GR_OK;
}

gr_status gr_engine_restore(gr_engine* e, const void* host_buf, size_t size, gr_stream_t stream) {
  if (!e || !host_buf) return fail(GR_ERR_INVALID, "NULL argument");
  if (size != gr_engine_state_size(e)) return fail(GR_ERR_INVALID, "state size does not match this engine");
  GR_CUDA(cudaMemcpyAsync(e->st, host_buf, size, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  GR_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return GR_OK;
}

gr_status gr_engine_sync(gr_engine* e, gr_stream_t stream) {
  if (!e) return fail(GR_ERR_INVALID, "engine is NULL");
  GR_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  std::vector<int32_t> status(e->K);
  GR_CUDA(cudaMemcpy2D(status.data(), sizeof(int32_t), &e->st[0].status, sizeof(EngState), sizeof(int32_t),
                       (size_t)e->K, cudaMemcpyDeviceToHost));
  int32_t any = 0;
  for (int32_t s : status) any |= s;
  if (any) {
    GR_CUDA(cudaMemset2D(&e->st[0].status, sizeof(EngState), 0, sizeof(int32_t), (size_t)e->K));
    if (any & GR_DEV_REJECT_LIMIT) return fail(GR_ERR_REJECT_LIMIT, "a rejection loop hit its iteration cap");
    if (any & GR_DEV_MMA_TIMEOUT) return fail(GR_ERR_CUDA, "a tensor-core kernel timed out waiting for its products");
    return fail(GR_ERR_INVALID, "device reported invalid input");
  }
  return GR_OK;
}

}  // extern "C"

namespace {

// Per-call constants, as the reference generators compute them.
gr_status make_params(const gr_dist_desc& d, DistParams& p) {
  std::memset(&p, 0, sizeof p);
  p.kind = d.kind;
  p.dtype = d.dtype;
  const bool f = d.dtype == GR_F32;
  const double a = d.a, b = d.b;
  switch (d.kind) {
    case kRawKind:
    case GR_UNIFORM_REAL:
    case GR_BALANCED:
    case GR_NORMAL_STD:
    case GR_RANDBITS:
      break;
    case GR_UNIFORM_REAL2:  // UniformRealGen(min, max): bias=min, slope=max-min (Scalar)
    case GR_BALANCED2:      // Balanced2Gen(a, b): slope=b-a, bias=a
      p.fa = (float)b - (float)a;
      p.fb = (float)a;
      p.da = b - a;
      p.db = a;
      break;
    case GR_NORMAL:
    case GR_LOGNORMAL:  // mean=a, stdev=b
    case GR_CAUCHY:
    case GR_EXTREME_VALUE:
      p.fa = (float)a;
      p.fb = (float)b;
      p.da = a;
      p.db = b;
      break;
    case GR_EXPONENTIAL:
      p.fa = (float)a;
      p.da = a;
      break;
    case GR_BERNOULLI:  // BernoulliGen(p): (uint32_t)(p * 0x80000000), compared as int32 (Basic.h:680-684)
      if (!(a >= 0 && a <= 1)) return fail(GR_ERR_INVALID, "bernoulli needs 0 <= p <= 1");
      p.ia = (int32_t)(uint32_t)(a * 2147483648.0);
      break;
    case GR_GEOMETRIC:  // GeometricGen(p): rlog_q = 1 / log(1 - p), set as a float packet (Discrete.h:1353-1374)
      p.fa = (float)(1 / std::log(1 - a));
      break;
    case GR_NEGATIVE_BINOMIAL: {  // GammaGen<float>((float)trials, (float)((1 - p) / p)), GammaPoisson.h:42-45
      if (d.trials < 1 || !(a > 0 && a <= 1)) return fail(GR_ERR_INVALID, "negativeBinomial needs trials >= 1, 0 < p <= 1");
      const float af = (float)d.trials, bf = (float)((1 - a) / a);
      p.fa = af;
      p.fb = bf;
      p.fc = std::sqrt(2 * af - 1);  // GammaGen::sqrt, NormalExp.h:455-459
      p.fd = af - 1;
      const int cnt = (int)af;
      p.ia = cnt;
      p.ic = af == 1.0f ? 0 : (((float)cnt == af && cnt < 20) ? 1 : 2);  // exponential / product / tan
      break;
    }
    case GR_UNIFORM_INT: {  // UniformIntGen<int32_t>(min, max), Discrete.h:230-245 (size_t arithmetic)
      const int32_t mn = (int32_t)a, mx = (int32_t)b;
      // pdiff = (size_t)(_max - _min): the int32 difference, sign-extended
      const uint64_t pdiff = (uint64_t)(int64_t)(int32_t)((uint32_t)mx - (uint32_t)mn);
      uint64_t bits = 0;
      if (pdiff != 0) bits = (uint64_t)std::ceil(std::log2((double)(pdiff + 1 > pdiff ? pdiff + 1 : pdiff)));
      // bitmask = (_Scalar)(~0 >> (64 - bitsize)), stored back into a size_t
      const uint64_t bitmask = bits == 0 ? ~0ull : (uint64_t)(int64_t)(int32_t)(uint32_t)(~0ull >> (64 - bits));
      p.ia = mn;                                  // pmin
      p.bitmask = (uint32_t)bitmask;              // pset1<Packet4i>(bitmask)
      p.ic = (int32_t)(uint32_t)(pdiff + 1);      // plen = pset1<Packet4i>(pdiff + 1)
      p.ncdf = bits < 32 ? (int32_t)bits : 32;    // slice width (shifts only happen below 16)
      p.ib = pdiff == 0 ? 0 : (pdiff == bitmask ? 1 : 2);  // constant / masked bits / rejection
      break;
    }
    case GR_WEIBULL:  // pset1(1 / a) in the scalar type
      p.fa = 1.0f / (float)a;
      p.fb = (float)b;
      p.da = 1.0 / a;
      p.db = b;
      break;
    case GR_CHI_SQUARED:  // ChiSquaredGen(n) = GammaGen(n * 0.5, 2) in the scalar type
    case GR_GAMMA: {
      const bool chi = d.kind == GR_CHI_SQUARED;
      const float af = chi ? (float)a * 0.5f : (float)a;
      const double ad = chi ? a * 0.5 : a;
      const double bb = chi ? 2.0 : b;
      p.kind = GR_GAMMA;
      p.fa = af;
      p.fb = (float)bb;
      p.da = ad;
      p.db = bb;
      p.ia = f ? (af == 1.0f) : (ad == 1.0);
      // integer alpha < 20: product of alpha uniforms (NormalExp.h:577-587)
      const int cnt = f ? (int)af : (int)ad;
      const bool integral = f ? ((float)cnt == af) : ((double)cnt == ad);
      p.ib = (integral && cnt < 20 && cnt >= 2) ? cnt : 0;
      // rejection branches (NormalExp.h:453-458, 535-604): 1/alpha, alpha-1,
      // px = e/(alpha+e), sqrt(2 alpha - 1), all in the scalar type
      p.fc = 1 / af;
      p.fd = af - 1;
      p.fe = (float)(2.7182818284590452 / (af + 2.7182818284590452));
      p.ff = std::sqrt(2 * af - 1);
      p.dc = 1 / ad;
      p.dd = ad - 1;
      p.de = 2.7182818284590452 / (ad + 2.7182818284590452);
      p.df = std::sqrt(2 * ad - 1);
      p.ic = f ? (af < 1.0f) : (ad < 1.0);  // GS branch
      // relative band of the float pre-test of double GS trials (gs_filter_f64),
      // and ceil(px * 2^52) for the integer branch test, as the bits of dg
      p.fh = (float)(std::ldexp(1.0, -18) * (1.0 + 40.0 / ad));
      {
        const uint64_t tpx = (uint64_t)std::ceil(p.de * 0x1p52);
        std::memcpy(&p.dg, &tpx, sizeof tpx);
      }
      break;
    }
    case GR_FISHER_F:  // FisherFGen(m, n): BetaGen(m/2, n/2) in the scalar type, NormalExp.h:997-1000
    case GR_BETA: {    // BetaGen(a, b), NormalExp.h:949-976
      double ba = a, bb = b;
      if (d.kind == GR_FISHER_F) {
        if (f) {
          ba = (double)((float)a * 0.5f);
          bb = (double)((float)b * 0.5f);
        } else {
          ba = a * 0.5;
          bb = b * 0.5;
        }
        p.kind = GR_BETA;
        p.post = 1;  // (b/a) x / (1 - x), NormalExp.h:1016-1021
        p.fh = (float)bb / (float)ba;
        p.dh = bb / ba;
      }
      const float af = (float)ba, bf = (float)bb;
      p.fa = af;
      p.fb = bf;
      p.fc = 1 / af;
      p.fd = 1 / bf;
      p.da = ba;
      p.db = bb;
      p.dc = 1 / ba;
      p.dd = 1 / bb;
      p.ic = f ? (af < 1 && bf < 1) : (ba < 1 && bb < 1);
      break;
    }
    case GR_POISSON: {  // PoissonGen(mean), Discrete.h:806-812 (double), packet constants in float
      const double mean = a;
      p.da = mean;
      p.fa = (float)std::sqrt(2 * mean);
      p.fb = (float)mean;
      p.fc = (float)std::log(mean);
      p.fd = (float)(mean * std::log(mean) - std::lgamma(mean + 1));
      p.fe = (float)std::exp(-mean);
      p.ic = mean < 12;
      break;
    }
    case GR_STUDENT_T:  // n = a; pset1(-2 / n) in the scalar type
      p.fa = (float)a;
      p.fc = -2 / (float)a;
      p.da = a;
      p.dc = -2 / a;
      break;
    case GR_BINOMIAL: {  // BinomialGen(trials, p): a = p, Discrete.h:926-938
      const double pp = a, small_p = std::min(pp, 1 - pp), mean = d.trials * small_p;
      p.da = pp;
      p.ia = d.trials;
      p.db = mean;
      p.ib = pp != small_p;  // return trials - res
      if (d.trials < 25) {
        p.fa = (float)pp;
      } else if (mean < 1.0) {
        p.fe = (float)std::exp(-mean);
        p.ic = 1;  // poisson loop
      } else {
        const double sqrt_v = std::sqrt(2 * mean * (1 - small_p));
        p.fa = (float)sqrt_v;
        p.fb = (float)mean;
        p.fc = (float)std::log(small_p);
        p.fd = (float)std::log(1 - small_p);
        p.fg = (float)std::lgamma(d.trials + 1);
        p.fh = (float)d.trials;
      }
      break;
    }
    default:
      return fail(GR_ERR_UNSUPPORTED, "distribution kind not implemented yet");
  }
  // divisors and scales that are exactly 1 in the scalar type
  if (p.kind == GR_EXPONENTIAL && (f ? p.fa == 1.0f : p.da == 1.0)) p.flags |= kParamUnitDiv;
  if ((p.kind == GR_GAMMA || p.kind == GR_WEIBULL) && (f ? p.fb == 1.0f : p.db == 1.0)) p.flags |= kParamUnitScale;
  return GR_OK;
}

// AliasMethod::buildTable (Discrete.h:76-190) and the CDF of DiscreteGen
// (Discrete.h:385-412), int32 precision; restated on the host.
gr_status build_discrete(const std::vector<double>& w, std::vector<int32_t>& prob, std::vector<int32_t>& alias,
                         int& ncdf, uint32_t& bitmask) {
  const size_t n = w.size();
  if (n == 0) return fail(GR_ERR_INVALID, "no weights");
  if (n < 16) {
    std::vector<double> cdf;
    double acc = 0;
    for (double x : w) cdf.push_back(acc += x);
    prob.clear();
    for (double x : cdf) prob.push_back((int32_t)(uint32_t)(x / cdf.back() * 0x80000000));
    ncdf = (int)n;
    bitmask = 0;
    return GR_OK;
  }
  double sum = 0;
  for (double x : w) sum += x;
  if (!std::isfinite(sum)) return fail(GR_ERR_NAN_WEIGHT, "cannot build NaN value distribution");
  const size_t nb = (size_t)std::ceil(std::log2((double)n));
  const size_t ps = (size_t)1 << nb;
  bitmask = (uint32_t)(((size_t)-1) >> (sizeof(size_t) * 8 - nb));
  prob.assign(ps, 0);
  alias.assign(ps, 0);
  sum /= (double)ps;
  std::vector<double> f(ps, 0.0);
  for (size_t i = 0; i < n; ++i) f[i] = w[i] / sum;
  size_t over = 0, under = 0, mm;
  while (over < ps && f[over] < 1) ++over;
  while (under < ps && f[under] >= 1) ++under;
  mm = under + 1;
  while (over < ps && under < ps) {
    prob[under] = (int32_t)(f[under] * (2147483647 + 1.0));
    alias[under] = (int32_t)over;
    f[over] += f[under] - 1;
    if (f[over] >= 1 || mm <= over) {
      for (under = mm; under < ps && f[under] >= 1; ++under) {
      }
      mm = under + 1;
    } else {
      under = over;
    }
    while (over < ps && f[over] < 1) ++over;
  }
  for (; over < ps; ++over) {
    if (f[over] >= 1) {
      prob[over] = 2147483647;
      alias[over] = (int32_t)over;
    }
  }
  if (under < ps) {
    prob[under] = 2147483647;
    alias[under] = (int32_t)under;
    for (under = mm; under < n; ++under) {
      if (f[under] < 1) {
        prob[under] = 2147483647;
        alias[under] = (int32_t)under;
      }
    }
  }
  ncdf = 0;
  return GR_OK;
}

// Zeroed on the call's stream: a plain cudaMemset runs on the legacy stream,
// which streams created non-blocking (the serving loop's) do not wait for.
gr_status ensure_gen_state(gr_gen* g, int K, cudaStream_t s) {
  if (g->gst && g->gst_K == K) return GR_OK;
  cudaFree(g->gst);
  g->gst = nullptr;
  GR_CUDA(cudaMalloc(&g->gst, sizeof(GenState) * (size_t)K));
  GR_CUDA(cudaMemsetAsync(g->gst, 0, sizeof(GenState) * (size_t)K, s));
  g->gst_K = K;
  return GR_OK;
}

// Choose the jump-ahead segmentation for a single-engine-per-slice call.
void plan_segments(const gr_engine* e, int64_t packets_max, int ppu, int& S, int64_t& J) {
  S = 1;
  J = std::max<int64_t>(packets_max, 2);
  if (e->K >= 16 || packets_max < (int64_t)1 << 17) return;
  const int64_t target = std::max<int64_t>(1, 128 / e->K);
  int64_t j = (int64_t)1 << 14;
  while (j * target < packets_max) j <<= 1;
  if (ppu == 2 && (j & 1)) ++j;
  S = (int)((packets_max + j - 1) / j);
  J = j;
}

// How a kind's draws map onto the packet stream.
enum class Family { Direct, Staged, Reject, Walk, Unsupported };

// GammaGen branch of a component with shape `alpha` in the generator's scalar
// type: (branch << 8) | packets per draw or per trial (NormalExp.h:527-604).
int gamma_branch(double alpha, bool f32) {
  const double a = f32 ? (double)(float)alpha : alpha;
  if (a < 1) return (2 << 8) | 3;  // GS rejection, 3 packets per trial
  if (a == 1) return (0 << 8) | 1;  // exponential
  const int cnt = (int)a;
  if ((double)cnt == a && cnt < 20) return (1 << 8) | cnt;  // product of cnt uniforms
  return (3 << 8) | 2;  // tan proposal, 2 packets per trial
}

// Rejection family code for launch_reject, or -1.
int reject_code(const DistParams& dp) {
  if (dp.dtype == GR_I32) {
    if (dp.kind == GR_POISSON && !dp.ic) return 3;
    if (dp.kind == GR_BINOMIAL && dp.ia >= 25 && !dp.ic) return 4;
    return -1;
  }
  if (dp.kind == GR_GAMMA && dp.ia == 0 && dp.ib == 0) return dp.ic ? 0 : 1;
  if (dp.kind == GR_BETA && dp.ic) return 2;
  return -1;
}

Family family_of(const DistParams& dp) {
  if (kind_is_direct(dp.kind, dp.dtype, dp)) return Family::Direct;
  if (dp.kind == GR_GAMMA && dp.ib >= 2 && dp.dtype != GR_I32) return Family::Staged;
  if (dp.kind == GR_STUDENT_T && dp.dtype != GR_I32) return Family::Staged;
  if (dp.kind == GR_BINOMIAL && dp.dtype == GR_I32 && dp.ia < 25) return Family::Staged;
  if (reject_code(dp) >= 0) return Family::Reject;
  if (dp.dtype == GR_I32 && dp.kind == GR_POISSON && dp.ic) return Family::Walk;
  if (dp.dtype == GR_I32 && dp.kind == GR_BINOMIAL && dp.ia >= 25 && dp.ic) return Family::Walk;
  if (dp.dtype != GR_I32 && dp.kind == GR_BETA && !dp.ic) return Family::Walk;
  if (dp.dtype == GR_I32 && dp.kind == GR_UNIFORM_INT) return Family::Walk;  // constant or rejection
  if (dp.dtype == GR_I32 && dp.kind == GR_NEGATIVE_BINOMIAL) return Family::Walk;
  return Family::Unsupported;
}

// Sets up prefix / jump windows for an S-segment call; exponents s*J - delta.
gr_status prepare_segments(gr_engine* e, Plan& p, int S, int64_t J, int delta, cudaStream_t stream) {
  p.S = S;
  p.J = J;
  if (S <= 1) return GR_OK;
  if (!e->prefix) {
    GR_CUDA(cudaMalloc(&e->prefix, sizeof(uint64_t) * (size_t)kPrefixLen * kLanes * (size_t)e->K));
    GR_CUDA(cudaMalloc(&e->snap, sizeof(CallSnap) * (size_t)e->K));
  }
  const size_t need = (size_t)e->K * (S - 1) * kLanes * kN;
  if (e->segwin_words < need) {
    cudaFree(e->segwin);
    e->segwin = nullptr;
    GR_CUDA(cudaMalloc(&e->segwin, sizeof(uint64_t) * need));
    e->segwin_words = need;
  }
  const uint64_t* polys = nullptr;
  gr_status st = get_jump_polys(e->device, J, delta, S - 1, &polys);
  if (st != GR_OK) return st;
  GR_CUDA(launch_prefix(e->st, p.gen, e->K, e->prefix, e->snap, stream));
  GR_CUDA(launch_jump(e->prefix, polys, e->K, S, e->segwin, stream));
  p.segwin = e->segwin;
  p.prefix = e->prefix;
  return GR_OK;
}

// Fraction of accepted candidate lanes of a rejection family (the expected
// output packets per trial), estimated once per parameter set on the host by
// evaluating the acceptance test on 4096 pseudo-random lanes.  Used only to
// plan how many trials the segments of a long call cover; the result does not
// depend on it.
double reject_yield(int rk, const DistParams& d) {
  static std::mutex mu;
  static std::map<std::vector<double>, double> cache;
  const std::vector<double> key = {(double)rk, (double)d.dtype, d.fa, d.fb, d.fc, d.fd, d.fe, d.ff, d.fg, d.fh,
                                   d.da, d.db, (double)d.ia, (double)d.ib, (double)d.ic};
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  std::mt19937_64 rng(0x5eed);
  auto u = [&]() { return (double)(rng() >> 11) * (1.0 / 9007199254740992.0); };
  const double pi = 3.14159265358979323846, e1 = 2.7182818284590452;
  const double alpha = d.dtype == GR_F64 ? d.da : (double)d.fa;
  const int N = 4096;
  int acc = 0;
  for (int i = 0; i < N; ++i) {
    bool ok = false;
    if (rk == 0) {  // GammaGen alpha < 1
      const double ux = u(), vx = u() + 1e-12, ux2 = u();
      const double lv = std::log(vx);
      double xx, qx;
      if (ux < e1 / (alpha + e1)) {
        xx = std::exp(lv / alpha);
        qx = std::exp(-xx);
      } else {
        xx = 1.0 - lv;
        qx = std::exp(std::log(xx) * (alpha - 1));
      }
      ok = ux2 < qx;
    } else if (rk == 1) {  // GammaGen tan proposal
      const double yx = std::tan(pi * u()), ux = u();
      const double sq = std::sqrt(2 * alpha - 1), xx = sq * yx + (alpha - 1);
      ok = xx > 0 && ux <= (yx * yx + 1) * std::exp((alpha - 1) * std::log(xx / (alpha - 1)) - yx * sq);
    } else if (rk == 2) {  // BetaGen a, b < 1
      const double a = d.dtype == GR_F64 ? d.da : d.fa, b = d.dtype == GR_F64 ? d.db : d.fb;
      ok = std::pow(u(), 1 / a) + std::pow(u(), 1 / b) <= 1.0;
    } else if (rk == 3) {  // PoissonGen mean >= 12
      const double yx = std::tan(pi * u()), u2 = u();
      const double fres = std::trunc(d.fa * yx + d.fb);
      ok = fres >= 0 && u2 <= 0.9 * (yx * yx + 1) * std::exp(fres * d.fc - std::lgamma(fres + 1) - d.fd);
    } else {  // BinomialGen tan proposal
      const double yx = std::tan(pi * u()), u2 = u();
      const double fres = std::trunc(d.fa * yx + d.fb);
      if (fres >= 0 && fres <= d.fh) {
        const double tt = d.fg - std::lgamma(fres + 1) - std::lgamma(d.fh + 1 - fres) + fres * d.fc + (d.fh - fres) * d.fd;
        ok = u2 <= 1.2 * d.fa * (1 + yx * yx) * std::exp(tt);
      }
    }
    acc += ok ? 1 : 0;
  }
  const double q = std::max((double)acc / N, 1.0 / N);
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = q;
  return q;
}

// Expected half packets one PoissonGen packetOp consumes (the longest of
// its four lanes' multiplicative loops, threshold fe = exp(-mean) in float),
// estimated once per threshold on the host from 4096 simulated packets.  Used
// only to plan how many segments a long call covers; the result does not
// depend on it.
// The engine blocks a rejection or walk kernel may generate in one call
// (its iteration cap).  GR_MAX_BLOCKS (tests) lowers the cap so that a call
// runs into it: the kernel stops, records GR_DEV_REJECT_LIMIT in the engine's
// status word and returns, and gr_engine_sync reports GR_ERR_REJECT_LIMIT.
int64_t block_cap(int64_t planned) {
  const char* v = std::getenv("GR_MAX_BLOCKS");
  if (!v) return planned;
  const long long c = std::atoll(v);
  return c > 0 ? std::min<int64_t>(planned, (int64_t)c) : planned;
}

double poisson_step_halves(float fe) {
  static std::mutex mu;
  static std::map<float, double> cache;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(fe);
    if (it != cache.end()) return it->second;
  }
  std::mt19937_64 rng(0x5eed);
  auto u = [&]() { return (float)((double)(rng() >> 40) * (1.0 / 16777216.0)); };
  const int N = 4096;
  double tot = 0;
  for (int i = 0; i < N; ++i) {
    int L = 0;
    for (int j = 0; j < 4; ++j) {
      float v = 1.0f;
      int it = 0;
      do {
        v *= u();
        ++it;
      } while (fe < v && it < 64);
      L = std::max(L, it);
    }
    tot += L;
  }
  const double m = tot / N;
  std::lock_guard<std::mutex> lk(mu);
  cache[fe] = m;
  return m;
}

gr_status run_packets(gr_engine* e, gr_gen* g, const DistParams& dp, void* out, size_t n, cudaStream_t stream);

// The n % P elements after the last whole packet of a call: the scalar
// operator(), one engine packet each, drawn from the last stream (whose slice
// they extend), its first 64-bit lane transformed by launch_tail.
gr_status run_tail(gr_engine* e, const DistParams& dp, void* out, int r, cudaStream_t stream) {
  if (!e->tailw) GR_CUDA(cudaMalloc(&e->tailw, sizeof(uint64_t) * 8));
  DistParams rp{};
  rp.kind = kRawLane0Kind;
  rp.dtype = GR_U64;
  Plan p{};
  p.eng = e->st + (e->K - 1);
  p.K = 1;
  p.S = 1;
  p.J = r;
  p.gran = 4;  // four (virtual) outputs per packet: one draw
  p.gran_per_k = r;
  p.out = e->tailw;
  cudaError_t err = launch_direct(p, rp, nullptr, stream);
  if (err == cudaSuccess) err = launch_tail(e->tailw, out, r, dp, true, stream);
  if (err != cudaSuccess) return cuda_fail(err, "scalar tail");
  return GR_OK;
}

// The 2-lane Vmt19937_64 (SSE / NEON profile, Pmt19937_64<Packet4i>,
// PacketRandomEngine.h:585-588): lanes seed, seed + 1, a packet of two 64-bit
// lanes per draw, a Packet4f (4 floats) or Packet2d (2 doubles) per packet.
// Its lanes are the first two of the 4-lane engine with the same seed, so
// the kernels run the 4-lane engine and use lanes 0 and 1.  Served: the raw
// stream and the kinds whose packetOp transforms each 32-bit word (float) or
// 64-bit lane (double) on its own, whose values do not depend on the packet
// width.
gr_status run_two_lane(gr_engine* e, const DistParams& dp0, void* out, size_t n, cudaStream_t stream) {
  if (!kind_two_lane(dp0.kind, dp0.dtype) || (dp0.kind == GR_GAMMA && dp0.ia != 1))
    return fail(GR_ERR_UNSUPPORTED, "2-lane Vmt19937_64: the raw stream, uniformReal, exponential, cauchy, weibull, "
                                    "extremeValue and gamma(alpha = 1) in float and double, balanced and "
                                    "bernoulli in float");
  const int opp = (dp0.kind == kRawKind || dp0.dtype == GR_F64) ? 2 : 4;
  if (n % (size_t)opp)
    return fail(GR_ERR_INVALID, "size must be a multiple of " + std::to_string(opp) +
                                    " (the 2-lane packet width for this type)");
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  DistParams dp = dp0;
  dp.flags |= kParamTwoLane;
  const int64_t granules = (int64_t)(n / (size_t)opp);
  Plan p{};
  p.eng = e->st;
  p.K = e->K;
  p.gran = opp;
  p.gran_per_k = granules / e->K;
  p.gran_rem = granules % e->K;
  p.out = out;
  const int64_t packets_max = p.gran_per_k + (p.gran_rem ? 1 : 0);
  int S;
  int64_t J;
  plan_segments(e, packets_max, 1, S, J);
  gr_status st = prepare_segments(e, p, S, J, 0, stream);
  if (st != GR_OK) return st;
  cudaError_t err = launch_direct(p, dp, e->snap, stream);
  if (err != cudaSuccess) return cuda_fail(err, "2-lane sampling kernel");
  return GR_OK;
}

gr_status run_call(gr_engine* e, gr_gen* g, const DistParams& dp, void* out, size_t n, cudaStream_t stream) {
  // the kernels store whole packets with 16-byte vector stores
  if (n && ((uintptr_t)out % 16)) return fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  if (e->lanes == 2) return run_two_lane(e, dp, out, n, stream);
  const int gran = kind_granule(dp.kind, dp.dtype);
  const int r = (int)(n % (size_t)gran);
  if (r == 0) return run_packets(e, g, dp, out, n, stream);
  if (!kind_has_exact_tail(dp.kind, dp.dtype)) {
    return fail(GR_ERR_INVALID, "size must be a multiple of " + std::to_string(gran) +
                                    " (the reference packet width for this type); a partial last packet is "
                                    "supported for uniformReal, balanced, bernoulli and randBits, whose scalar "
                                    "form is exact");
  }
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  const size_t whole = n - (size_t)r;
  if (whole) {
    gr_status st = run_packets(e, g, dp, out, whole, stream);
    if (st != GR_OK) return st;
  }
  const size_t es = dp.dtype == GR_F64 ? 8 : 4;
  return run_tail(e, dp, static_cast<char*>(out) + whole * es, r, stream);
}

gr_status run_packets(gr_engine* e, gr_gen* g, const DistParams& dp, void* out, size_t n, cudaStream_t stream) {
  const int gran = kind_granule(dp.kind, dp.dtype);
  if (n % (size_t)gran) {
    return fail(GR_ERR_INVALID, "size must be a multiple of " + std::to_string(gran) +
                                    " (the reference packet width for this type)");
  }
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  const Family fam = family_of(dp);
  if (fam == Family::Unsupported) return fail(GR_ERR_UNSUPPORTED, "this parameter set is not implemented yet");
  if (dp.kind == GR_BINOMIAL && dp.ia <= 0) {
    // BinomialGen with 0 trials draws nothing and returns 0 (Discrete.h:1000-1009)
    GR_CUDA(cudaMemsetAsync(out, 0, n * sizeof(int32_t), stream));
    return GR_OK;
  }
  const int64_t granules = (int64_t)(n / (size_t)gran);
  Plan p{};
  p.eng = e->st;
  p.gen = g ? g->gst : nullptr;
  p.K = e->K;
  p.gran = gran;
  p.gran_per_k = granules / e->K;
  p.gran_rem = granules % e->K;
  p.out = out;
  const int64_t nk_max = (p.gran_per_k + (p.gran_rem ? 1 : 0)) * gran;

  if (fam == Family::Direct) {
    // packets per slice, upper bound (caches can only reduce it)
    int opp = 8;
    const int bk = dp.kind >= kVecBase ? dp.kind - kVecBase : dp.kind;
    if (bk == kRawKind || bk == kRawLane0Kind || (dp.dtype == GR_F64 && bk != GR_BALANCED && bk != GR_BALANCED2))
      opp = 4;
    const int ppu = kind_packets_per_unit(dp.kind, dp.dtype);
    int64_t packets_max = (nk_max + opp - 1) / opp;
    if (ppu == 2) packets_max += packets_max & 1;
    int S;
    int64_t J;
    plan_segments(e, packets_max, ppu, S, J);
    gr_status st = prepare_segments(e, p, S, J, 0, stream);
    if (st != GR_OK) return st;
    cudaError_t err = launch_direct(p, dp, e->snap, stream);
    if (err != cudaSuccess) return cuda_fail(err, "sampling kernel");
    return GR_OK;
  }

  if (fam == Family::Reject) {
    if (!p.gen) return fail(GR_ERR_INVALID, "rejection samplers need a generator state");
    const int P = (dp.dtype == GR_F32) ? 8 : 4;
    const int rk = reject_code(dp);
    const int64_t wt = rk == 0 ? 24 : (rk >= 3 ? 8 : 16);  // words per trial
    const int64_t npk = nk_max / P;
    const int64_t max_blocks = block_cap(((16 * npk + 4096) * wt) / (kN * 8) + 64);
    if (e->K < 16 && npk >= ((int64_t)1 << 12)) {
      // long call on few engines: jump-ahead segments over the trial stream
      const double q = reject_yield(rk, dp);
      // GR_REJECT_PLAN_SCALE (tests) scales the planned trials; below 1 the
      // last segment runs on past its plan, which must give the same result
      const char* sc = std::getenv("GR_REJECT_PLAN_SCALE");
      const double scale = sc ? std::max(0.0, std::atof(sc)) : 1.0;
      const int64_t t_need = (int64_t)std::ceil((double)npk / q * 1.04 * scale) + 256;
      const int64_t smax = std::max(2, 128 / e->K);
      const int64_t Ts = std::max<int64_t>((t_need + smax - 1) / smax, 2048);
      const int S = (int)((t_need + Ts - 1) / Ts);
      if (S >= 2) {
        const int64_t J = Ts * (wt / 8);
        gr_status st = prepare_segments(e, p, S, J, dp.dtype == GR_I32 ? 1 : 0, stream);
        if (st != GR_OK) return st;
        RsArgs a{};
        a.Ts = Ts;
        a.lane_cap = P * (npk + 2) + 16;
        a.pos_cap = npk + 2;
        a.max_blocks = max_blocks;
        const size_t K = (size_t)e->K;
        // lane buffer: K * lane_cap lanes of 8 (double) or 4 bytes
        const size_t lane_words = dp.dtype == GR_F64 ? K * (size_t)a.lane_cap : (K * (size_t)a.lane_cap + 1) / 2;
        const size_t words = K * S * 4 + K * 4 + lane_words + K * (size_t)a.pos_cap;
        int64_t* buf = nullptr;
        GR_CUDA(cudaMallocAsync(&buf, sizeof(int64_t) * words, stream));
        a.cnt = buf;
        a.start = buf + K * S * 2;
        a.fin = buf + K * S * 4;
        a.lanes = reinterpret_cast<uint64_t*>(buf + K * S * 4 + K * 4);
        a.pos = buf + K * S * 4 + K * 4 + lane_words;
        cudaError_t err = launch_reject_segmented(p, dp, rk, e->snap, a, a.lane_cap, stream);
        cudaFreeAsync(buf, stream);
        if (err != cudaSuccess) return cuda_fail(err, "segmented rejection kernels");
        return GR_OK;
      }
    }
    cudaError_t err = launch_reject(p, dp, rk, max_blocks, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rejection sampling kernel");
    return GR_OK;
  }

  if (fam == Family::Walk) {
    if (!p.gen) return fail(GR_ERR_INVALID, "these samplers need a generator state");
    const int P = (dp.dtype == GR_F32) ? 8 : 4;
    const int64_t npk = nk_max / P;
    DistParams wd = dp;
    int64_t max_blocks;
    if (dp.kind == GR_UNIFORM_INT) {
      // every draw accepts each lane with probability > 1/2
      max_blocks = (npk * 16) / (2 * kN) + 64;
    } else if (dp.kind == GR_NEGATIVE_BINOMIAL) {
      // gamma draws (< 20 or ~2.5 per trial) plus the Poisson loop or trials
      max_blocks = (npk * 160) / (2 * kN) + 64;
    } else if (dp.dtype == GR_I32) {
      // PoissonGen loop (mean < 12); BinomialGen with mean < 1 runs the same
      // loop on its poisson member and returns trials - res when p > 1/2
      wd.fe = dp.kind == GR_POISSON ? (float)std::exp(-dp.da) : dp.fe;
      wd.ia = dp.kind == GR_BINOMIAL ? dp.ia : 0;
      wd.ic = dp.kind == GR_BINOMIAL ? dp.ib : 0;
      max_blocks = block_cap((npk * 64) / (2 * kN) + 64);
      if (e->K < 16 && npk >= ((int64_t)1 << 14)) {
        // long call on few engines: the step chain over jump-ahead segments
        const int64_t J = (int64_t)1 << 15;
        const double hl = poisson_step_halves(wd.fe);
        // GR_WALK_PLAN_SCALE (tests) scales the planned packets: below 1 the
        // last segment runs on past its plan, above 1 the call ends in an
        // earlier segment; the result is the same
        const char* sc = std::getenv("GR_WALK_PLAN_SCALE");
        const double scale = sc ? std::max(0.0, std::atof(sc)) : 1.0;
        const int64_t need = (int64_t)std::ceil((double)npk * hl * 0.5 * 1.03 * scale) + 64;
        const int S = (int)std::max<int64_t>(2, (need + J - 1) / J);
        gr_status st = prepare_segments(e, p, S, J, 0, stream);
        if (st != GR_OK) return st;
        PwArgs a{};
        a.J = J;
        a.snap = e->snap;
        a.words_per_seg = (2 * J + 1) / 32 + 2;
        a.max_blocks = max_blocks;
        const size_t KS = (size_t)e->K * S;
        const size_t bytes = KS * (4 * 4 + kPwEntries * 2 * 4 + 3 * 8 + (size_t)a.words_per_seg * 4);
        char* buf = nullptr;
        GR_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&buf), bytes, stream));
        a.plan = reinterpret_cast<int64_t*>(buf);
        a.info = reinterpret_cast<int32_t*>(buf + KS * 3 * 8);
        a.ent = a.info + KS * 4;
        a.bits = reinterpret_cast<uint32_t*>(a.ent + KS * kPwEntries * 2);
        cudaError_t err = launch_poisson_segmented(p, wd, a, stream);
        cudaFreeAsync(buf, stream);
        if (err != cudaSuccess) return cuda_fail(err, "segmented Poisson kernels");
        return GR_OK;
      }
    } else {
      const bool f32 = dp.dtype == GR_F32;
      wd.ia = gamma_branch(dp.da, f32);
      wd.ib = gamma_branch(dp.db, f32);
      wd.fa = (float)dp.da;
      wd.fb = (float)dp.db;
      max_blocks = (npk * 64) / kN + 64;
    }
    max_blocks = block_cap(max_blocks);
    cudaError_t err = launch_walk(p, wd, max_blocks, stream);
    if (err != cudaSuccess) return cuda_fail(err, "walk sampling kernel");
    return GR_OK;
  }

  // staged: U packets (full kinds) or U half packets (int32) per unit of P outputs
  const int P = (dp.dtype == GR_F32) ? 8 : 4;
  const bool half = dp.dtype == GR_I32;
  int U = 0;
  if (dp.kind == GR_GAMMA) U = dp.ib;
  if (dp.kind == GR_STUDENT_T) U = 2;
  if (dp.kind == GR_BINOMIAL) U = dp.ia;
  const int64_t units = nk_max / P;
  const int64_t packets_max = half ? (units * U + 1) / 2 + 1 : units * U;
  int S = 1;
  int64_t Us = std::max<int64_t>(units, 1), J = packets_max;
  if (e->K < 16 && packets_max >= ((int64_t)1 << 17)) {
    const int64_t target = std::max<int64_t>(1, 128 / e->K);
    int64_t us = 2;
    while (us * target < units || (half ? us * U / 2 : us * U) < ((int64_t)1 << 14)) us <<= 1;
    Us = us;
    J = half ? us * U / 2 : us * U;
    S = (int)((units + us - 1) / us);
  }
  const int delta = half ? 1 : 0;
  gr_status st = prepare_segments(e, p, S, J, delta, stream);
  if (st != GR_OK) return st;
  cudaError_t err = launch_staged(p, dp, e->snap, U, Us, delta, stream);
  if (err != cudaSuccess) return cuda_fail(err, "staged sampling kernel");
  return GR_OK;
}

// TruncGen's constructors (Truncated.h) in the scalar type T.  Bases with a
// closed-form CDF become UniformRealGen(phi(lower), phi(upper)) followed by
// the inverse CDF: TruncNormalGen (:293-305, also for NormalGen :353-358 and
// StdNormalGen :793-798), lognormal (:565-575), exponential (:448-458),
// Cauchy (:507-515), extreme value (:621-630), Weibull (:679-690); the
// uniform family is a UniformRealGen over the intersected range (:741-751,
// :840-845, :888-893, :936-941).  `reject` is set for every other base:
// generic CompressMask rejection (:202-263).  std:: math in T, as the
// reference calls it.
template <typename T>
gr_status trunc_setup(const gr_dist_desc& d, T lo, T hi, DistParams& p, bool& reject) {
  reject = false;
  if (!(lo < hi)) return fail(GR_ERR_INVALID, "truncation support needs lower < upper");
  const T a = (T)d.a, b = (T)d.b;
  T bias = 0, top = 0, c0 = 0, c1 = 0;
  int kind = 0;
  switch (d.kind) {
    case GR_UNIFORM_REAL:
    case GR_UNIFORM_REAL2:
    case GR_BALANCED:
    case GR_BALANCED2: {
      // the base's bias and bias + slope
      T ob = 0, os = 1;
      if (d.kind == GR_BALANCED) ob = -1, os = 2;
      if (d.kind == GR_UNIFORM_REAL2 || d.kind == GR_BALANCED2) ob = a, os = b - a;
      const T mn = lo > ob ? lo : ob, mx = hi < ob + os ? hi : ob + os;
      if (!(mn < mx)) return fail(GR_ERR_INVALID, "truncation support does not meet the base's range");
      gr_dist_desc u{};
      u.kind = GR_UNIFORM_REAL2;
      u.dtype = d.dtype;
      u.a = (double)mn;
      u.b = (double)mx;
      return make_params(u, p);
    }
    case GR_NORMAL_STD:
    case GR_NORMAL:
    case GR_LOGNORMAL: {
      const T mean = d.kind == GR_NORMAL_STD ? (T)0 : a, sd = d.kind == GR_NORMAL_STD ? (T)1 : b;
      if (!(sd > 0)) return fail(GR_ERR_INVALID, "truncated normal needs stdev > 0");
      if (d.kind == GR_LOGNORMAL) {
        lo = lo <= 0 ? std::numeric_limits<T>::lowest() : std::log(lo);
        hi = std::log(hi);
        if (!(lo < hi)) return fail(GR_ERR_INVALID, "truncation support needs lower < upper");
      }
      const T an = (lo - mean) / sd, bn = (hi - mean) / sd, k = (T)(1.0 / 1.4142135623730951);
      bias = (T)0.5 * std::erfc(-an * k);
      top = (T)0.5 * std::erfc(-bn * k);
      c0 = sd;
      c1 = mean;
      kind = d.kind == GR_LOGNORMAL ? kTruncLognormalKind : kTruncNormalKind;
      break;
    }
    case GR_EXPONENTIAL: {
      const T el = lo < 0 ? (T)0 : lo;
      bias = (T)1 - std::exp(-a * el);
      top = (T)1 - std::exp(-a * hi);
      c0 = (T)1 / a;
      kind = kTruncExponentialKind;
      break;
    }
    case GR_CAUCHY:
      bias = (T)0.5 + std::atan((lo - a) / b) / (T)3.1415926535897932;
      top = (T)0.5 + std::atan((hi - a) / b) / (T)3.1415926535897932;
      c0 = a;
      c1 = b;
      kind = kTruncCauchyKind;
      break;
    case GR_EXTREME_VALUE:
      bias = std::exp(-std::exp(-(lo - a) / b));
      top = std::exp(-std::exp(-(hi - a) / b));
      c0 = a;
      c1 = b;
      kind = kTruncExtremeKind;
      break;
    case GR_WEIBULL: {
      const T el = lo < 0 ? (T)0 : lo;
      bias = (T)1 - std::exp(-std::pow(el / b, a));
      top = (T)1 - std::exp(-std::pow(hi / b, a));
      c0 = (T)1 / a;
      c1 = b;
      kind = kTruncWeibullKind;
      break;
    }
    case GR_GAMMA:
    case GR_BETA:
    case GR_STUDENT_T:
    case GR_CHI_SQUARED:
    case GR_FISHER_F:
    case GR_BERNOULLI:
      reject = true;
      return GR_OK;
    default:
      return fail(GR_ERR_UNSUPPORTED, "truncation of this distribution kind is not implemented");
  }
  const T slope = top - bias;
  std::memset(&p, 0, sizeof p);
  p.kind = kind;
  p.dtype = d.dtype;
  p.fa = (float)slope;
  p.fb = (float)bias;
  p.fc = (float)c0;
  p.fd = (float)c1;
  p.da = (double)slope;
  p.db = (double)bias;
  p.dc = (double)c0;
  p.dd = (double)c1;
  return GR_OK;
}

// Advances every stream of the engine by npackets raw packets without writing
// them: k_direct's raw mode with no output, in jump-ahead segments like a
// long call.
gr_status advance_engine(gr_engine* e, uint64_t npackets, cudaStream_t s) {
  if (npackets == 0) return GR_OK;
  DistParams dp{};
  dp.kind = kRawKind;
  dp.dtype = GR_U64;
  Plan p{};
  p.eng = e->st;
  p.K = e->K;
  p.gran = 4;
  p.gran_per_k = (int64_t)npackets;
  p.gran_rem = 0;
  p.out = nullptr;
  int S;
  int64_t J;
  plan_segments(e, (int64_t)npackets, 1, S, J);
  gr_status st = prepare_segments(e, p, S, J, 0, s);
  if (st != GR_OK) return st;
  const cudaError_t err = launch_direct(p, dp, e->snap, s);
  if (err != cudaSuccess) return cuda_fail(err, "engine advance");
  return GR_OK;
}

// Engine packets per base output packet when the base's consumption is
// fixed (direct and staged kinds: GammaGen with integer alpha, StudentTGen,
// BernoulliGen), else 0 (rejection and walk kinds).
int64_t fixed_packets_per_packet(const DistParams& dp) {
  const Family fam = family_of(dp);
  if (fam == Family::Direct) return kind_packets_per_unit(dp.kind, dp.dtype);
  if (fam == Family::Staged && dp.dtype != GR_I32) return dp.kind == GR_STUDENT_T ? 2 : dp.ib;
  return 0;
}

// TruncGen<Base>::generate for the rejection form on a single-stream engine.
// The base packets are drawn in chunks into HBM and filtered (gr_trunc.cu);
// the host reads how many outputs each chunk gave.  When a chunk holds the
// last wanted output at base packet k*, the engine goes back to its state at
// the chunk start and moves to just after base packet k*: by a raw advance of
// (k* + 1) * U packets when the base consumes a fixed U packets per packet,
// else by drawing the k* + 1 base packets again (with the base's caches
// restored too).  Chunk sizes come from the acceptance seen so far (a first
// call draws a pilot chunk): a fixed-consumption base draws its expected need
// plus four standard deviations, so one chunk almost always suffices; any
// other base draws four standard deviations short, so the redrawn last chunk
// is small.  Synchronises the stream once per chunk.
gr_status run_trunc(gr_engine* e, gr_gen* g, void* out, size_t n, cudaStream_t s) {
  const int dt = g->dp.dtype;
  const int64_t P = dt == GR_F32 ? 8 : 4;
  const size_t lb = dt == GR_F32 ? 4 : 8;
  if (n % (size_t)P)
    return fail(GR_ERR_INVALID, "size must be a multiple of " + std::to_string(P) + " (the reference packet width)");
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  if (e->K != 1) return fail(GR_ERR_UNSUPPORTED, "TruncGen rejection needs a single-stream engine");
  gr_gen* b = g->trunc_base;
  gr_status st = ensure_gen_state(b, 1, s);
  if (st != GR_OK) return st;
  if (!g->trunc_carry) {
    GR_CUDA(cudaMalloc(&g->trunc_carry, sizeof(GenSlot)));
    GR_CUDA(cudaMemsetAsync(g->trunc_carry, 0, sizeof(GenSlot), s));
  }
  const int64_t upk = fixed_packets_per_packet(b->dp);
  const int64_t need = (int64_t)(n / (size_t)P);
  const int64_t mcap = kTruncChunkMax - 1;
  // scratch, grown when a chunk needs more: candidates, FIFO, CTA sums,
  // group slots, results, saved engine and base states
  char* buf = nullptr;
  int64_t have_m = 0;
  auto layout = [&](int64_t m, size_t off[7]) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t r = o;
      o += (bytes + 255) / 256 * 256;
      return r;
    };
    off[0] = take((size_t)m * P * lb);
    off[1] = take((size_t)(m + 1) * P * lb);
    off[2] = take(sizeof(int64_t) * 2 * (size_t)((m + 255) / 256));
    off[3] = take(sizeof(int64_t) * (size_t)(m + 1));
    off[4] = take(sizeof(int64_t) * 8);
    off[5] = take(sizeof(EngState));
    off[6] = take(sizeof(GenState));
    return o;
  };
  auto bail = [&](gr_status r) {
    if (buf) cudaFreeAsync(buf, s);
    return r;
  };
  size_t off[7];
  int64_t done = 0, drawn = 0;
  int64_t res[6];
  while (done < need) {
    const int64_t rem = need - done;
    const double q = g->trunc_lanes > 0 ? (double)g->trunc_acc / (double)g->trunc_lanes : 0.0;
    int64_t M;
    if (q <= 0) {
      M = std::min<int64_t>(rem, 4096);
    } else {
      // packets for rem * P accepted lanes, and the spread of that count
      const double lanes = (double)rem * (double)P, E = lanes / (q * (double)P);
      const double sd = std::sqrt(lanes * std::max(1.0 - q, 0.0)) / (q * (double)P);
      if (upk == 0 && E > 32768) M = (int64_t)(E - 4 * sd) - 16;
      else M = (int64_t)std::ceil(E + 4 * sd) + 16;
    }
    M = std::max<int64_t>(1, std::min(M, mcap));
    drawn += M;
    if (drawn > ((int64_t)1 << 40))
      return bail(fail(GR_ERR_REJECT_LIMIT, "TruncGen: the support holds almost none of the base distribution"));
    if (M > have_m) {
      if (buf) cudaFreeAsync(buf, s);
      buf = nullptr;
      const int64_t m = std::min(mcap, std::max(M, have_m * 2));
      const cudaError_t err = cudaMallocAsync(&buf, layout(m, off), s);
      if (err != cudaSuccess) return cuda_fail(err, "TruncGen scratch");
      have_m = m;
    }
    layout(have_m, off);
    void* cand = buf + off[0];
    int64_t* dres = reinterpret_cast<int64_t*>(buf + off[4]);
    EngState* saved_e = reinterpret_cast<EngState*>(buf + off[5]);
    GenState* saved_g = reinterpret_cast<GenState*>(buf + off[6]);
    cudaError_t err = cudaMemcpyAsync(saved_e, e->st, sizeof(EngState), cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess) err = cudaMemcpyAsync(saved_g, b->gst, sizeof(GenState), cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "TruncGen state copy"));
    st = run_call(e, b, b->dp, cand, (size_t)(M * P), s);
    if (st != GR_OK) return bail(st);
    TruncFilterArgs a{};
    a.cand = cand;
    a.M = M;
    a.lower = g->trunc_lo;
    a.upper = g->trunc_hi;
    a.carry = g->trunc_carry;
    a.out = static_cast<char*>(out) + (size_t)done * P * lb;
    a.cap = rem;
    a.queue = buf + off[1];
    a.blk = reinterpret_cast<int64_t*>(buf + off[2]);
    a.grp = reinterpret_cast<int64_t*>(buf + off[3]);
    a.res = dres;
    err = launch_trunc_filter(dt, a, s);
    if (err == cudaSuccess) err = cudaMemcpyAsync(res, dres, sizeof res, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "TruncGen filter"));
    g->trunc_lanes += M * P;
    g->trunc_acc += res[2] * P + res[3];
    if (res[1] < 0) {
      done += res[0];
      continue;
    }
    if (res[1] + 1 < M) {
      // back to the chunk start, then just past base packet k*
      err = cudaMemcpyAsync(e->st, saved_e, sizeof(EngState), cudaMemcpyDeviceToDevice, s);
      if (err == cudaSuccess) err = cudaMemcpyAsync(b->gst, saved_g, sizeof(GenState), cudaMemcpyDeviceToDevice, s);
      if (err != cudaSuccess) return bail(cuda_fail(err, "TruncGen state copy"));
      st = upk ? advance_engine(e, (uint64_t)((res[1] + 1) * upk), s)
               : run_call(e, b, b->dp, cand, (size_t)((res[1] + 1) * P), s);
      if (st != GR_OK) return bail(st);
    }
    done = need;
  }
  return bail(GR_OK);
}

// TruncGen<Base>{base, Support(lower, upper)}: fills g (inverse-CDF forms in
// g->dp; the rejection form with a base generator and carried lanes).
gr_status make_truncated(gr_gen* g, const gr_dist_desc& base, double lower, double upper) {
  if (base.dtype != GR_F32 && base.dtype != GR_F64)
    return fail(GR_ERR_INVALID, "truncation needs a float or double generator");
  bool reject = false;
  gr_status st = base.dtype == GR_F32 ? trunc_setup<float>(base, (float)lower, (float)upper, g->dp, reject)
                                      : trunc_setup<double>(base, lower, upper, g->dp, reject);
  if (st != GR_OK || !reject) return st;
  st = gr_gen_create(&g->trunc_base, &base);
  if (st != GR_OK) return st;
  g->dp = g->trunc_base->dp;
  g->trunc_lo = base.dtype == GR_F32 ? (double)(float)lower : lower;
  g->trunc_hi = base.dtype == GR_F32 ? (double)(float)upper : upper;
  return GR_OK;
}

// binomial(urng, trials, p) with int32 trials and float p arrays, or one of
// them a scalar (Discrete.h:1822-1898): BinomialVGen<int32_t> on packets of 4.
gr_status run_binom_v(gr_engine* e, const gr_dist_desc& d, const void* dev_a, const void* dev_b, void* out, size_t n,
                      cudaStream_t s) {
  if (d.dtype != GR_I32) return fail(GR_ERR_UNSUPPORTED, "per-element binomial: BinomialVGen<int32_t> only");
  if (n % 4) return fail(GR_ERR_INVALID, "size must be a multiple of 4 (the reference packet width for this type)");
  if (n == 0) return GR_OK;
  Plan p{};
  p.eng = e->st;
  p.K = e->K;
  p.gran = 4;
  p.gran_per_k = (int64_t)(n / 4) / e->K;
  p.gran_rem = (int64_t)(n / 4) % e->K;
  p.out = out;
  BinomVArgs a{};
  a.trials = static_cast<const int32_t*>(dev_a);
  a.p = static_cast<const float*>(dev_b);
  a.trials0 = d.trials;
  a.p0 = (float)d.a;
  // half packets per output packet: the Poisson loop (mean < 1) draws about
  // its largest count + 1, the tan rejection two per round until every lane
  // has accepted
  const int64_t npk = p.gran_per_k + (p.gran_rem ? 1 : 0);
  a.max_blocks = (npk * 128) / (2 * kN) + 64;
  const cudaError_t err = launch_binom_v(p, a, s);
  if (err != cudaSuccess) return cuda_fail(err, "per-element binomial kernel");
  return GR_OK;
}

}  // namespace

extern "C" {

gr_status gr_raw_u64(gr_engine* e, uint64_t* dev_out, size_t n, gr_stream_t stream) {
  if (!e) return fail(GR_ERR_INVALID, "engine is NULL");
  DistParams dp{};
  dp.kind = kRawKind;
  dp.dtype = GR_U64;
  return run_call(e, nullptr, dp, dev_out, n, (cudaStream_t)stream);
}

gr_status gr_engine_discard(gr_engine* e, uint64_t npackets, gr_stream_t stream) {
  if (!e) return fail(GR_ERR_INVALID, "engine is NULL");
  return advance_engine(e, npackets, (cudaStream_t)stream);
}

gr_status gr_gen_create(gr_gen** out, const gr_dist_desc* desc) {
  if (!out || !desc) return fail(GR_ERR_INVALID, "NULL argument");
  gr_gen* g = new gr_gen;
  g->desc = *desc;
  gr_status st = GR_OK;
  if (desc->kind == GR_DISCRETE) {
    if (!desc->weights || desc->nweights <= 0) {
      delete g;
      return fail(GR_ERR_INVALID, "discrete needs weights");
    }
    g->weights.assign(desc->weights, desc->weights + desc->nweights);
    g->desc.weights = nullptr;
    std::vector<int32_t> prob, alias;
    int ncdf = 0;
    uint32_t mask = 0;
    st = build_discrete(g->weights, prob, alias, ncdf, mask);
    if (st == GR_OK) {
      const size_t np = prob.size(), na = alias.size();
      if (cudaMalloc(&g->table, sizeof(int32_t) * (np + na + 1)) != cudaSuccess) st = fail(GR_ERR_NOMEM, "table");
      if (st == GR_OK) {
        cudaMemcpy(g->table, prob.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice);
        if (na) cudaMemcpy(g->table + np, alias.data(), sizeof(int32_t) * na, cudaMemcpyHostToDevice);
      }
      std::memset(&g->dp, 0, sizeof g->dp);
      g->dp.kind = GR_DISCRETE;
      g->dp.dtype = GR_I32;
      g->dp.ncdf = ncdf;
      g->dp.bitmask = mask;
      g->dp.prob = g->table;
      g->dp.alias = g->table + np;
    }
  } else {
    st = make_params(g->desc, g->dp);
  }
  if (st != GR_OK) {
    cudaFree(g->table);
    delete g;
    return st;
  }
  *out = g;
  return GR_OK;
}

gr_status gr_gen_destroy(gr_gen* g) {
  if (!g) return GR_OK;
  cudaFree(g->table);
  cudaFree(g->gst);
  cudaFree(g->trunc_carry);
  gr_gen_destroy(g->trunc_base);
  delete g;
  return GR_OK;
}

gr_status gr_gen_create_truncated(gr_gen** out, const gr_dist_desc* base, double lower, double upper) {
  if (!out || !base) return fail(GR_ERR_INVALID, "NULL argument");
  gr_gen* g = new gr_gen;
  g->desc = *base;
  g->desc.weights = nullptr;
  const gr_status st = make_truncated(g, *base, lower, upper);
  if (st != GR_OK) {
    gr_gen_destroy(g);
    return st;
  }
  *out = g;
  return GR_OK;
}

gr_status gr_sample_truncated(gr_engine* e, const gr_dist_desc* base, double lower, double upper, void* dev_out,
                              size_t n, gr_stream_t stream) {
  if (!e || !base) return fail(GR_ERR_INVALID, "NULL argument");
  gr_gen tmp;
  tmp.desc = *base;
  gr_status st = make_truncated(&tmp, *base, lower, upper);
  if (st == GR_OK) {
    // the inverse-CDF forms keep no cache; the rejection form is synchronous
    st = tmp.trunc_base ? gr_generate(&tmp, e, dev_out, n, stream)
                        : run_call(e, nullptr, tmp.dp, dev_out, n, (cudaStream_t)stream);
  }
  cudaFree(tmp.trunc_carry);
  gr_gen_destroy(tmp.trunc_base);
  tmp.trunc_carry = nullptr;
  tmp.trunc_base = nullptr;
  return st;
}

gr_status gr_generate(gr_gen* g, gr_engine* e, void* dev_out, size_t n, gr_stream_t stream) {
  if (!g || !e) return fail(GR_ERR_INVALID, "NULL generator or engine");
  if (n && ((uintptr_t)dev_out % 16)) return fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  if (g->trunc_base) {
    if (need_four_lanes(e, "truncated rejection") != GR_OK) return GR_ERR_UNSUPPORTED;
    return run_trunc(e, g, dev_out, n, (cudaStream_t)stream);
  }
  gr_status st = ensure_gen_state(g, e->K, (cudaStream_t)stream);
  if (st != GR_OK) return st;
  return run_call(e, g, g->dp, dev_out, n, (cudaStream_t)stream);
}

// ---- batched sets + autotuner ------------------------------------------------
// Candidates: CTA width 160 (the 156-thread twist plus 4) or 320 (twice the
// threads for trial evaluation, half the CTAs per SM).  The first call for a
// (kind, log2 nsets) class times each candidate on the call's own sets with
// CUDA events (the results are deterministic, so the timed runs just rewrite
// the same outputs) and caches the fastest.
namespace {
std::mutex g_tune_mu;
std::map<std::pair<int, int>, int> g_tuned;
}  // namespace

static int tuned_threads(int kind, int64_t nsets) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int b = 0;
  while (((int64_t)1 << b) < nsets) ++b;
  auto it = g_tuned.find({kind, b});
  return it == g_tuned.end() ? 0 : it->second;
}

gr_status gr_sample_batched(gr_engine* e, const gr_batch_desc* bd, gr_stream_t stream) {
  if (!e || !bd) return fail(GR_ERR_INVALID, "NULL argument");
  if (bd->kind != GR_GAMMA && bd->kind != GR_BINOMIAL_V)
    return fail(GR_ERR_UNSUPPORTED, "batched sets support GR_GAMMA and GR_BINOMIAL_V");
  if (bd->nsets <= 0) return GR_OK;
  if (!bd->a || !bd->counts || !bd->offsets || !bd->out || (bd->kind == GR_GAMMA && !bd->b) ||
      (bd->kind == GR_BINOMIAL_V && !bd->trials))
    return fail(GR_ERR_INVALID, "missing device array in gr_batch_desc");
  if ((uintptr_t)bd->out % 16) return fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  VopArgs va{};
  va.nsets = bd->nsets;
  va.perm = nullptr;
  va.seed = bd->seed;
  va.a = bd->a;
  va.b = bd->b;
  va.trials = bd->trials;
  va.counts = bd->counts;
  va.offsets = bd->offsets;
  va.out = bd->out;
  va.status = &e->st[0].status;
  int b = 0;
  while (((int64_t)1 << b) < bd->nsets) ++b;
  int threads = tuned_threads(bd->kind, bd->nsets);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cap);
  if (threads == 0 && cap == cudaStreamCaptureStatusNone) {
    const int cand[2] = {160, 320};
    float best = 1e30f;
    int best_t = 160;
    cudaEvent_t e0, e1;
    GR_CUDA(cudaEventCreate(&e0));
    GR_CUDA(cudaEventCreate(&e1));
    for (int c : cand) {
      GR_CUDA(launch_vop(bd->kind, c, va, s));  // warm
      GR_CUDA(cudaEventRecord(e0, s));
      GR_CUDA(launch_vop(bd->kind, c, va, s));
      GR_CUDA(cudaEventRecord(e1, s));
      GR_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      GR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        best_t = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[{bd->kind, b}] = best_t;
    threads = best_t;
    // the timed runs already wrote the outputs; one more launch keeps the
    // call's own semantics simple (identical values)
  }
  if (threads == 0) threads = 160;
  GR_CUDA(launch_vop(bd->kind, threads, va, s));
  return GR_OK;
}

gr_status gr_sample(gr_engine* e, const gr_dist_desc* desc, void* dev_out, size_t n, gr_stream_t stream) {
  if (!e || !desc) return fail(GR_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  // A temporary *Gen: its caches start empty and die with the call.  They
  // live in engine-owned scratch that is cleared in stream order, so the
  // call stays asynchronous.
  if (!e->scratch_gen) GR_CUDA(cudaMalloc(&e->scratch_gen, sizeof(GenState) * (size_t)e->K));
  GR_CUDA(cudaMemsetAsync(e->scratch_gen, 0, sizeof(GenState) * (size_t)e->K, s));
  gr_gen tmp;
  tmp.desc = *desc;
  gr_status st = GR_OK;
  if (desc->kind == GR_DISCRETE) {
    if (!desc->weights || desc->nweights <= 0) return fail(GR_ERR_INVALID, "discrete needs weights");
    std::vector<double> w(desc->weights, desc->weights + desc->nweights);
    std::vector<int32_t> prob, alias;
    int ncdf = 0;
    uint32_t mask = 0;
    st = build_discrete(w, prob, alias, ncdf, mask);
    if (st != GR_OK) return st;
    const size_t np = prob.size(), na = alias.size();
    std::vector<int32_t> both(prob);
    both.insert(both.end(), alias.begin(), alias.end());
    GR_CUDA(cudaMallocAsync(&tmp.table, sizeof(int32_t) * (np + na + 1), s));
    GR_CUDA(cudaMemcpyAsync(tmp.table, both.data(), sizeof(int32_t) * (np + na), cudaMemcpyHostToDevice, s));
    std::memset(&tmp.dp, 0, sizeof tmp.dp);
    tmp.dp.kind = GR_DISCRETE;
    tmp.dp.dtype = GR_I32;
    tmp.dp.ncdf = ncdf;
    tmp.dp.bitmask = mask;
    tmp.dp.prob = tmp.table;
    tmp.dp.alias = tmp.table + np;
    tmp.gst = e->scratch_gen;
    tmp.gst_K = e->K;
    // pageable source: the table is staged before cudaMemcpyAsync returns
    st = run_call(e, &tmp, tmp.dp, dev_out, n, s);
    cudaFreeAsync(tmp.table, s);
    tmp.table = nullptr;
    tmp.gst = nullptr;
    return st;
  }
  st = make_params(tmp.desc, tmp.dp);
  if (st != GR_OK) return st;
  tmp.gst = e->scratch_gen;
  tmp.gst_K = e->K;
  st = run_call(e, &tmp, tmp.dp, dev_out, n, s);
  tmp.gst = nullptr;
  return st;
}

gr_status gr_sample_v(gr_engine* e, const gr_dist_desc* desc, const void* dev_a, void* dev_out, size_t n,
                      gr_stream_t stream) {
  return gr_sample_v2(e, desc, dev_a, nullptr, dev_out, n, stream);
}

gr_status gr_sample_v2(gr_engine* e, const gr_dist_desc* desc, const void* dev_a, const void* dev_b, void* dev_out,
                       size_t n, gr_stream_t stream) {
  if (!e || !desc) return fail(GR_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  // a fresh *VGen: its StdNormalGen cache (normal, lognormal) starts empty
  if (!e->scratch_gen) GR_CUDA(cudaMalloc(&e->scratch_gen, sizeof(GenState) * (size_t)e->K));
  GR_CUDA(cudaMemsetAsync(e->scratch_gen, 0, sizeof(GenState) * (size_t)e->K, s));
  gr_gen tmp;
  tmp.desc = *desc;
  tmp.gst = e->scratch_gen;
  tmp.gst_K = e->K;
  const gr_status st = gr_generate_v(&tmp, e, dev_a, dev_b, dev_out, n, stream);
  tmp.gst = nullptr;
  return st;
}

gr_status gr_generate_v(gr_gen* g, gr_engine* e, const void* dev_a, const void* dev_b, void* dev_out, size_t n,
                        gr_stream_t stream) {
  if (!g || !e || (n && !dev_out)) return fail(GR_ERR_INVALID, "NULL argument");
  if (need_four_lanes(e, "per-element parameters") != GR_OK) return GR_ERR_UNSUPPORTED;
  const gr_dist_desc& d = g->desc;
  if (((uintptr_t)dev_a | (uintptr_t)dev_b | (uintptr_t)dev_out) % 16)
    return fail(GR_ERR_INVALID, "parameter and output arrays must be 16-byte aligned");
  DistParams dp{};
  if (d.kind == GR_BERNOULLI && d.dtype == GR_F32 && dev_a && !dev_b) {
    dp.kind = kBernoulliVKind;
    dp.dtype = GR_F32;
    dp.vparam = dev_a;
    return run_call(e, nullptr, dp, dev_out, n, (cudaStream_t)stream);
  }
  if (d.kind == GR_BERNOULLI)
    return fail(GR_ERR_UNSUPPORTED,
                "per-element bernoulli: BernoulliVGen<float> only (the double form goes through a cast the "
                "reference leaves to Eigen's generic pcast)");
  if (d.kind == GR_BINOMIAL) return run_binom_v(e, d, dev_a, dev_b, dev_out, n, (cudaStream_t)stream);
  if (d.dtype != GR_F32 && d.dtype != GR_F64) return fail(GR_ERR_UNSUPPORTED, "per-element forms are float/double");
  gr_status st = GR_OK;
  switch (d.kind) {
    case GR_UNIFORM_REAL2:
    case GR_BALANCED2:
    case GR_NORMAL:
    case GR_LOGNORMAL:
    case GR_WEIBULL:
    case GR_EXTREME_VALUE:
    case GR_CAUCHY:
      break;
    case GR_EXPONENTIAL:
    case GR_STUDENT_T:
      if (dev_b) return fail(GR_ERR_INVALID, "this per-element form takes one parameter array");
      break;
    default:
      return fail(GR_ERR_UNSUPPORTED, "no per-element form for this distribution kind");
  }
  st = make_params(d, dp);
  if (st != GR_OK) return st;
  dp.flags = (dev_a ? kParamVecA : 0) | (dev_b ? kParamVecB : 0);
  dp.vparam = dev_a;
  dp.vparam2 = dev_b;
  if (d.kind != GR_STUDENT_T) {
    // direct kernels: kind kVecBase + K, scalar operands in fe/ff, de/df
    dp.kind = kVecBase + d.kind;
    dp.fe = (float)d.a;
    dp.ff = (float)d.b;
    dp.de = d.a;
    dp.df = d.b;
  }
  st = ensure_gen_state(g, e->K, (cudaStream_t)stream);
  if (st != GR_OK) return st;
  return run_call(e, g, dp, dev_out, n, (cudaStream_t)stream);
}

}  // extern "C"

// ---- multinomial draws on an engine (k_multinomial, gr_mv.cu) ---------------
namespace gr {

gr_status build_discrete_table(const std::vector<double>& w, std::vector<int32_t>& prob, std::vector<int32_t>& alias,
                               int& ncdf, uint32_t& bitmask) {
  return build_discrete(w, prob, alias, ncdf, bitmask);
}

gr_status run_multinomial(gr_engine* e, GenState* gst, const MnArgs& a0, int64_t samples, cudaStream_t stream) {
  if (samples <= 0) return GR_OK;
  MnArgs a = a0;
  // words per state period do not depend on the state the call starts in
  const MnLayout L0 = mn_layout(a.trials, 0);
  if (L0.W0 > kMnMaxSampleWords || L0.W1 > kMnMaxSampleWords)
    return fail(GR_ERR_UNSUPPORTED, "multinomial draws per sample above the kernel's ring size");
  const int64_t Wu = L0.spu == 2 ? L0.W0 + L0.W1 : L0.W0;
  Plan p{};
  p.eng = e->st;
  p.gen = gst;
  p.K = e->K;
  p.gran = 1;
  p.gran_per_k = samples / e->K;
  p.gran_rem = samples % e->K;
  p.out = a.out;
  const int64_t ns_max = p.gran_per_k + (p.gran_rem ? 1 : 0);
  const int64_t units = (ns_max + L0.spu - 1) / L0.spu;
  const int64_t packets_max = units * Wu / 8;
  int S = 1;
  int64_t Us = std::max<int64_t>(units, 1), J = std::max<int64_t>(packets_max, 2);
  if (e->K < 16 && packets_max >= ((int64_t)1 << 17)) {
    const int64_t target = std::max<int64_t>(1, 128 / e->K);
    int64_t us = 2;
    while (us * target < units || us * Wu / 8 < ((int64_t)1 << 14)) us <<= 1;
    Us = us;
    J = us * Wu / 8;
    S = (int)((units + us - 1) / us);
  }
  a.Us = Us;
  gr_status st = prepare_segments(e, p, S, J, 0, stream);
  if (st != GR_OK) return st;
  cudaError_t err = launch_multinomial(p, a, e->snap, stream);
  if (err != cudaSuccess) return cuda_fail(err, "multinomial kernel");
  return GR_OK;
}

}  // namespace gr

// ---- engine scratch reservation (serving loop) -------------------------------
namespace gr {

// Allocates the scratch a segmented call may need (prefix, call snapshot,
// windows for up to max_segments segments, the temporary-generator caches), so
// that later calls on this engine allocate nothing.
gr_status engine_reserve(gr_engine* e, int max_segments) {
  if (!e->prefix) {
    GR_CUDA(cudaMalloc(&e->prefix, sizeof(uint64_t) * (size_t)kPrefixLen * kLanes * (size_t)e->K));
    GR_CUDA(cudaMalloc(&e->snap, sizeof(CallSnap) * (size_t)e->K));
  }
  const size_t need = (size_t)e->K * (size_t)std::max(max_segments - 1, 1) * kLanes * kN;
  if (e->segwin_words < need) {
    cudaFree(e->segwin);
    e->segwin = nullptr;
    GR_CUDA(cudaMalloc(&e->segwin, sizeof(uint64_t) * need));
    e->segwin_words = need;
  }
  if (!e->scratch_gen) GR_CUDA(cudaMalloc(&e->scratch_gen, sizeof(GenState) * (size_t)e->K));
  return GR_OK;
}

}  // namespace gr

namespace gr {

gr_status draw_first_words(gr_engine* e, uint64_t* out, int64_t per_sample, int64_t samples, cudaStream_t s) {
  if (per_sample <= 0 || samples <= 0) return GR_OK;
  if (need_four_lanes(e, "scalar draws") != GR_OK) return GR_ERR_UNSUPPORTED;
  DistParams dp{};
  dp.kind = kRawLane0Kind;
  dp.dtype = GR_U64;
  Plan p{};
  p.eng = e->st;
  p.K = e->K;
  p.gran = (int32_t)(4 * per_sample);  // four (virtual) outputs per packet
  p.gran_per_k = samples / e->K;
  p.gran_rem = samples % e->K;
  p.out = out;
  const int64_t packets_max = (p.gran_per_k + (p.gran_rem ? 1 : 0)) * per_sample;
  int S;
  int64_t J;
  plan_segments(e, packets_max, 1, S, J);
  gr_status st = prepare_segments(e, p, S, J, 0, s);
  if (st != GR_OK) return st;
  const cudaError_t err = launch_direct(p, dp, e->snap, s);
  if (err != cudaSuccess) return cuda_fail(err, "scalar draws");
  return GR_OK;
}

}  // namespace gr

// ---- scalar engines ------------------------------------------------------------
namespace {

__global__ void k_p8_words(const uint64_t* pbuf, int cnt, int64_t from_buf, const uint64_t* fresh, int64_t R,
                           uint64_t* out, int64_t W) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W) return;
  if (i < from_buf) {
    out[i] = pbuf[cnt + i];
    return;
  }
  const int64_t q = i - from_buf, r = q / 8, j = q % 8;
  out[i] = j < 4 ? fresh[4 * r + j] : fresh[4 * R + 4 * r + (j - 4)];
}

__global__ void k_p8_keep(uint64_t* pbuf, const uint64_t* fresh, int64_t R) {
  const int j = threadIdx.x;
  if (j < 8) pbuf[j] = j < 4 ? fresh[4 * (R - 1) + j] : fresh[4 * R + 4 * (R - 1) + (j - 4)];
}

// The next W 64-bit draws of the scalar engine into out (device).
gr_status sengine_words(gr_sengine* se, uint64_t* out, int64_t W, cudaStream_t s) {
  if (W <= 0) return GR_OK;
  if (se->kind == GR_SCALAR_MT19937_64) {
    for (int64_t done = 0; done < W;) {  // a call's granule counts outputs in int32
      const int64_t c = std::min<int64_t>(W - done, (int64_t)1 << 28);
      const gr_status st = draw_first_words(se->eng, out + done, c, 1, s);
      if (st != GR_OK) return st;
      done += c;
    }
    return GR_OK;
  }
  const int64_t from_buf = std::min<int64_t>(W, 8 - se->cnt), rest = W - from_buf;
  const int64_t R = (rest + 7) / 8;  // new packets from each of the two engines
  uint64_t* fresh = nullptr;
  if (R > 0) {
    GR_CUDA(cudaMallocAsync(&fresh, sizeof(uint64_t) * 8 * (size_t)R, s));
    DistParams dp{};
    dp.kind = kRawKind;
    dp.dtype = GR_U64;
    // two streams: stream 0's 4R words, then stream 1's
    const gr_status st = run_call(se->eng, nullptr, dp, fresh, (size_t)(8 * R), s);
    if (st != GR_OK) {
      cudaFreeAsync(fresh, s);
      return st;
    }
  }
  k_p8_words<<<(unsigned)((W + 255) / 256), 256, 0, s>>>(se->pbuf, se->cnt, from_buf, fresh, R, out, W);
  cudaError_t err = cudaGetLastError();
  if (R > 0) {
    if (err == cudaSuccess) {
      k_p8_keep<<<1, 32, 0, s>>>(se->pbuf, fresh, R);
      err = cudaGetLastError();
    }
    cudaFreeAsync(fresh, s);
    se->cnt = (int)(rest - 8 * (R - 1));
  } else {
    se->cnt += (int)W;
  }
  if (err != cudaSuccess) return cuda_fail(err, "scalar engine words");
  return GR_OK;
}

// A one-chain sampler on a scalar engine: chunks of the engine's words are
// drawn into HBM from a saved engine state, one warp runs the sampler over
// them until they run out (launch(w, W, done, res) for the packets from
// `done` on, res = {packets completed, words they used}), and the engine is
// put back and advanced by exactly the words used.  wpp: words per packet
// expected, for the first chunk's size.
template <class Launch>
gr_status sengine_chain(gr_sengine* se, int64_t npk, int64_t wpp, Launch&& launch, cudaStream_t s) {
  gr_engine* e = se->eng;
  constexpr int64_t kMaxWords = (int64_t)1 << 24;
  EngState* saved = nullptr;
  uint64_t *w = nullptr, *pb = nullptr;
  int64_t* res = nullptr;
  auto bail = [&](gr_status st) {
    cudaFreeAsync(saved, s);
    cudaFreeAsync(w, s);
    cudaFreeAsync(pb, s);
    cudaFreeAsync(res, s);
    return st;
  };
  int64_t W = std::min<int64_t>(kMaxWords, std::max<int64_t>(4096, wpp * npk + 64));
  cudaError_t err = cudaMallocAsync(&saved, sizeof(EngState) * (size_t)e->K, s);
  if (err == cudaSuccess) err = cudaMallocAsync(&pb, sizeof(uint64_t) * 8, s);
  if (err == cudaSuccess) err = cudaMallocAsync(&res, sizeof(int64_t) * 2, s);
  if (err == cudaSuccess) err = cudaMallocAsync(&w, sizeof(uint64_t) * (size_t)W, s);
  if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine chain scratch"));
  for (int64_t done = 0; done < npk;) {
    err = cudaMemcpyAsync(saved, e->st, sizeof(EngState) * (size_t)e->K, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && se->pbuf)
      err = cudaMemcpyAsync(pb, se->pbuf, sizeof(uint64_t) * 8, cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine state copy"));
    const int cnt0 = se->cnt;
    gr_status st = sengine_words(se, w, W, s);
    if (st != GR_OK) return bail(st);
    err = launch(w, W, done, res);
    int64_t hres[2] = {0, 0};
    if (err == cudaSuccess) err = cudaMemcpyAsync(hres, res, sizeof hres, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "sampling on a scalar engine"));
    // back to the saved state, then forward by the words the packets used
    err = cudaMemcpyAsync(e->st, saved, sizeof(EngState) * (size_t)e->K, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && se->pbuf)
      err = cudaMemcpyAsync(se->pbuf, pb, sizeof(uint64_t) * 8, cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine state copy"));
    se->cnt = cnt0;
    if (hres[0] == 0) {  // one packet needs more words than the chunk: a larger chunk
      if (W == kMaxWords) return bail(fail(GR_ERR_REJECT_LIMIT, "a packet drew more than 2^24 words"));
      W = std::min<int64_t>(kMaxWords, 2 * W);
      cudaFreeAsync(w, s);
      w = nullptr;
      err = cudaMallocAsync(&w, sizeof(uint64_t) * (size_t)W, s);
      if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine chain scratch"));
      continue;
    }
    st = sengine_words(se, w, hres[1], s);
    if (st != GR_OK) return bail(st);
    done += hres[0];
  }
  return bail(GR_OK);
}

// binomial(urng, trials, p) on a scalar engine (BinomialVGen<int32_t>)
gr_status sengine_binom_v(gr_sengine* se, const gr_dist_desc& d, const void* dev_a, const void* dev_b, void* out,
                          size_t n, cudaStream_t s) {
  if (d.dtype != GR_I32) return fail(GR_ERR_UNSUPPORTED, "per-element binomial: BinomialVGen<int32_t> only");
  if (n % 4) return fail(GR_ERR_INVALID, "size must be a multiple of 4 (the reference packet width for this type)");
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  const int64_t npk = (int64_t)(n / 4);
  BinomVArgs a{};
  a.trials0 = d.trials;
  a.p0 = (float)d.a;
  // about 10 half packets (20 words) per packet in common parameter ranges
  return sengine_chain(
      se, npk, 24,
      [&](const uint64_t* w, int64_t W, int64_t done, int64_t* res) {
        a.trials = dev_a ? static_cast<const int32_t*>(dev_a) + 4 * done : nullptr;
        a.p = dev_b ? static_cast<const float*>(dev_b) + 4 * done : nullptr;
        return launch_binom_v_words(w, W, a, static_cast<int32_t*>(out) + 4 * done, npk - done, res, s);
      },
      s);
}

// GammaGen's rejection branches (GS for alpha < 1, the tan proposal) on a
// scalar engine, a fresh generator (the free functions): chunks of trials are
// drawn into HBM, every trial's candidate lanes evaluated at once (rejected
// lanes NaN), and TruncGen's CompressMask filter, with an unbounded support,
// emits the outputs in the reference's order.  A chunk that runs out leaves
// the engine exactly past its words; the chunk that completes the call puts
// the engine back and advances it past the trial that emitted the last
// output.
gr_status sengine_reject(gr_sengine* se, const DistParams& dp, int rk, void* out, size_t n, cudaStream_t s) {
  const int dt = dp.dtype;
  const int64_t P = dt == GR_F32 ? 8 : 4;
  const size_t lb = dt == GR_F32 ? 4 : 8;
  if (n % (size_t)P)
    return fail(GR_ERR_INVALID, "size must be a multiple of " + std::to_string(P) + " (the reference packet width)");
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  gr_engine* e = se->eng;
  // words per trial: packets per trial (GS 3, tan 2) of 3 (float) or 4 (double) draws
  const int64_t wpt = (rk == 0 ? 3 : 2) * (dt == GR_F32 ? 3 : 4);
  const int64_t need = (int64_t)(n / (size_t)P);
  const int64_t mcap = kTruncChunkMax - 1;
  const double q = reject_yield(rk, dp);
  char* buf = nullptr;
  int64_t have_m = 0;
  auto layout = [&](int64_t m, size_t off[8]) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t r = o;
      o += (bytes + 255) / 256 * 256;
      return r;
    };
    off[0] = take((size_t)m * P * lb);                                  // candidates
    off[1] = take((size_t)(m + 1) * P * lb);                            // FIFO
    off[2] = take(sizeof(int64_t) * 2 * (size_t)((m + 255) / 256));     // CTA sums
    off[3] = take(sizeof(int64_t) * (size_t)(m + 1));                   // group slots
    off[4] = take(sizeof(int64_t) * 8);                                 // results
    off[5] = take(sizeof(EngState) * (size_t)e->K + sizeof(uint64_t) * 8);  // saved engine
    off[6] = take(sizeof(GenSlot));                                     // carried lanes
    off[7] = take(sizeof(uint64_t) * (size_t)m * wpt);                  // words
    return o;
  };
  auto bail = [&](gr_status r) {
    if (buf) cudaFreeAsync(buf, s);
    return r;
  };
  size_t off[8];
  int64_t done = 0, drawn = 0;
  int64_t res[6];
  bool carry_clear = false;
  while (done < need) {
    const int64_t rem = need - done;
    // trials for rem output packets: q P accepted lanes per trial, plus spread
    const double E = (double)rem / q, sd = std::sqrt((double)rem * P * std::max(1.0 - q, 0.0)) / (q * P);
    int64_t M = (int64_t)std::ceil(E + 4 * sd) + 16;
    M = std::max<int64_t>(1, std::min(M, mcap));
    drawn += M;
    if (drawn > ((int64_t)1 << 40)) return bail(fail(GR_ERR_REJECT_LIMIT, "rejection: almost no trial accepts"));
    if (M > have_m) {
      // grow the scratch; the carried lanes move to the new buffer
      char* nb = nullptr;
      const int64_t m = std::min(mcap, std::max(M, have_m * 2));
      size_t noff[8];
      cudaError_t err = cudaMallocAsync(&nb, layout(m, noff), s);
      if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine rejection scratch"));
      if (buf && carry_clear)
        err = cudaMemcpyAsync(nb + noff[6], buf + off[6], sizeof(GenSlot), cudaMemcpyDeviceToDevice, s);
      else
        err = cudaMemsetAsync(nb + noff[6], 0, sizeof(GenSlot), s);
      if (buf) cudaFreeAsync(buf, s);
      buf = nb;
      carry_clear = true;
      if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine rejection scratch"));
      have_m = m;
    }
    layout(have_m, off);
    void* cand = buf + off[0];
    int64_t* dres = reinterpret_cast<int64_t*>(buf + off[4]);
    EngState* saved = reinterpret_cast<EngState*>(buf + off[5]);
    uint64_t* pb = reinterpret_cast<uint64_t*>(buf + off[5] + sizeof(EngState) * (size_t)e->K);
    uint64_t* w = reinterpret_cast<uint64_t*>(buf + off[7]);
    cudaError_t err = cudaMemcpyAsync(saved, e->st, sizeof(EngState) * (size_t)e->K, cudaMemcpyDeviceToDevice, s);
    if (err == cudaSuccess && se->pbuf)
      err = cudaMemcpyAsync(pb, se->pbuf, sizeof(uint64_t) * 8, cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine state copy"));
    const int cnt0 = se->cnt;
    gr_status st = sengine_words(se, w, M * wpt, s);
    if (st != GR_OK) return bail(st);
    err = launch_sx_cand(rk, dt, w, M, dp, cand, s);
    TruncFilterArgs a{};
    a.cand = cand;
    a.M = M;
    a.lower = -INFINITY;
    a.upper = INFINITY;
    a.carry = reinterpret_cast<GenSlot*>(buf + off[6]);
    a.out = static_cast<char*>(out) + (size_t)done * P * lb;
    a.cap = rem;
    a.queue = buf + off[1];
    a.blk = reinterpret_cast<int64_t*>(buf + off[2]);
    a.grp = reinterpret_cast<int64_t*>(buf + off[3]);
    a.res = dres;
    if (err == cudaSuccess) err = launch_trunc_filter(dt, a, s);
    if (err == cudaSuccess) err = cudaMemcpyAsync(res, dres, sizeof res, cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine rejection"));
    if (res[1] < 0) {
      done += res[0];
      continue;
    }
    if (res[1] + 1 < M) {
      // back to the chunk start, then just past trial res[1]
      err = cudaMemcpyAsync(e->st, saved, sizeof(EngState) * (size_t)e->K, cudaMemcpyDeviceToDevice, s);
      if (err == cudaSuccess && se->pbuf)
        err = cudaMemcpyAsync(se->pbuf, pb, sizeof(uint64_t) * 8, cudaMemcpyDeviceToDevice, s);
      if (err != cudaSuccess) return bail(cuda_fail(err, "scalar engine state copy"));
      se->cnt = cnt0;
      st = sengine_words(se, w, (res[1] + 1) * wpt, s);
      if (st != GR_OK) return bail(st);
    }
    done = need;
  }
  return bail(GR_OK);
}

// BetaGen / FisherFGen on a scalar engine, a fresh generator (the free
// functions): the chain of k_sx_beta over chunks of the engine's words, the
// carried lanes of GammaGen(a), GammaGen(b) and the beta's own loop starting
// empty and dropped after the call
gr_status sengine_beta(gr_sengine* se, const DistParams& dp, void* out, size_t n, cudaStream_t s) {
  const int64_t P = dp.dtype == GR_F32 ? 8 : 4;
  if (n % (size_t)P)
    return fail(GR_ERR_INVALID, "size must be a multiple of " + std::to_string(P) + " (the reference packet width)");
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  const int64_t npk = (int64_t)(n / (size_t)P);
  const size_t es = dp.dtype == GR_F32 ? 4 : 8;
  SxBetaArgs a{};
  a.beta = dp;
  if (!dp.ic) {  // GammaGen(a), GammaGen(b) with the parameters in the scalar type (NormalExp.h:914-917)
    for (int c = 0; c < 2; ++c) {
      gr_dist_desc gd{};
      gd.kind = GR_GAMMA;
      gd.dtype = dp.dtype;
      gd.a = dp.dtype == GR_F32 ? (double)(c == 0 ? dp.fa : dp.fb) : (c == 0 ? dp.da : dp.db);
      gd.b = 1.0;
      const gr_status st = make_params(gd, a.g[c]);
      if (st != GR_OK) return st;
    }
  }
  char* buf = nullptr;
  const size_t carry_bytes = sizeof(uint64_t) * 3 * 2 * (size_t)P;
  GR_CUDA(cudaMallocAsync(&buf, carry_bytes + 64, s));
  a.carry = reinterpret_cast<uint64_t*>(buf);
  a.cnt = reinterpret_cast<int32_t*>(buf + carry_bytes);
  a.res = reinterpret_cast<int64_t*>(buf + carry_bytes + 32);
  cudaError_t err = cudaMemsetAsync(buf, 0, carry_bytes + 64, s);
  if (err != cudaSuccess) {
    cudaFreeAsync(buf, s);
    return cuda_fail(err, "scalar engine carry");
  }
  // words per output packet: about two uniform packets per gamma, or per
  // trial of the a, b < 1 loop, of 3 (float) or 4 (double) draws
  const gr_status st = sengine_chain(
      se, npk, dp.dtype == GR_F32 ? 24 : 32,
      [&](const uint64_t* w, int64_t W, int64_t done, int64_t* res) {
        a.out = static_cast<char*>(out) + (size_t)done * P * es;
        a.npk = npk - done;
        a.res = res;
        return launch_sx_beta(w, W, a, dp.dtype, s);
      },
      s);
  cudaFreeAsync(buf, s);
  return st;
}

// PoissonGen / BinomialGen (int32) on a scalar engine: a fresh generator, so
// CompressMask's carried lanes start empty and are dropped after the call
gr_status sengine_int(gr_sengine* se, const DistParams& dp, void* out, size_t n, cudaStream_t s) {
  if (n % 4) return fail(GR_ERR_INVALID, "size must be a multiple of 4 (the reference packet width for this type)");
  if (n == 0) return GR_OK;
  if (!out) return fail(GR_ERR_INVALID, "output is NULL");
  const int64_t npk = (int64_t)(n / 4);
  uint32_t* carry = nullptr;
  GR_CUDA(cudaMallocAsync(&carry, sizeof(uint32_t) * 9, s));
  cudaError_t err = cudaMemsetAsync(carry, 0, sizeof(uint32_t) * 9, s);
  if (err != cudaSuccess) {
    cudaFreeAsync(carry, s);
    return cuda_fail(err, "scalar engine carry");
  }
  int64_t wpp = 24;
  if (dp.kind == GR_BINOMIAL && dp.ia < 25) wpp = 2 * std::max(dp.ia, 0) + 2;
  const gr_status st = sengine_chain(
      se, npk, wpp,
      [&](const uint64_t* w, int64_t W, int64_t done, int64_t* res) {
        return launch_int_words(w, W, dp, static_cast<int32_t*>(out) + 4 * done, npk - done, res, carry, s);
      },
      s);
  cudaFreeAsync(carry, s);
  return st;
}

}  // namespace

extern "C" {

gr_status gr_sengine_create(gr_sengine** out, int32_t kind, uint64_t seed) {
  if (!out) return fail(GR_ERR_INVALID, "NULL argument");
  if (kind != GR_SCALAR_MT19937_64 && kind != GR_SCALAR_P8_MT19937_64)
    return fail(GR_ERR_INVALID, "scalar engine kind: GR_SCALAR_MT19937_64 or GR_SCALAR_P8_MT19937_64");
  gr_sengine* se = new gr_sengine;
  se->kind = kind;
  gr_status st = gr_engine_create(&se->eng, seed, 4, kind == GR_SCALAR_P8_MT19937_64 ? 2 : 1);
  if (st == GR_OK && kind == GR_SCALAR_P8_MT19937_64 && cudaMalloc(&se->pbuf, sizeof(uint64_t) * 8) != cudaSuccess)
    st = fail(GR_ERR_NOMEM, "scalar engine buffer");
  if (st != GR_OK) {
    gr_sengine_destroy(se);
    return st;
  }
  *out = se;
  return GR_OK;
}

gr_status gr_sengine_destroy(gr_sengine* se) {
  if (!se) return GR_OK;
  cudaFree(se->pbuf);
  gr_engine_destroy(se->eng);
  delete se;
  return GR_OK;
}

gr_status gr_sengine_raw_u64(gr_sengine* se, uint64_t* dev_out, size_t n, gr_stream_t stream) {
  if (!se || (n && !dev_out)) return fail(GR_ERR_INVALID, "NULL argument");
  if (n && ((uintptr_t)dev_out % 16)) return fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  return sengine_words(se, dev_out, (int64_t)n, (cudaStream_t)stream);
}

gr_status gr_sengine_sample_v2(gr_sengine* se, const gr_dist_desc* desc, const void* dev_a, const void* dev_b,
                               void* dev_out, size_t n, gr_stream_t stream) {
  if (!se || !desc) return fail(GR_ERR_INVALID, "NULL argument");
  if (((uintptr_t)dev_a | (uintptr_t)dev_b | (uintptr_t)dev_out) % 16)
    return fail(GR_ERR_INVALID, "parameter and output arrays must be 16-byte aligned");
  if (desc->kind != GR_BINOMIAL)
    return fail(GR_ERR_UNSUPPORTED, "scalar engines: the per-element form is built for binomial only");
  return sengine_binom_v(se, *desc, dev_a, dev_b, dev_out, n, (cudaStream_t)stream);
}

gr_status gr_sengine_sample(gr_sengine* se, const gr_dist_desc* desc, void* dev_out, size_t n, gr_stream_t stream) {
  if (!se || !desc) return fail(GR_ERR_INVALID, "NULL argument");
  if (n && ((uintptr_t)dev_out % 16)) return fail(GR_ERR_INVALID, "output array must be 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  gr_status st = GR_OK;
  if (desc->kind == GR_DISCRETE) {
    // DiscreteGen<int32_t> (Discrete.h:443-480): one Packet8i of four draws
    // gives two output packets; an odd last packet still draws all four, its
    // upper half cached in the call's generator and dropped with it
    if (n % 4) return fail(GR_ERR_INVALID, "size must be a multiple of 4 (the reference packet width for this type)");
    if (n == 0) return GR_OK;
    if (!dev_out) return fail(GR_ERR_INVALID, "output is NULL");
    if (!desc->weights || desc->nweights <= 0) return fail(GR_ERR_INVALID, "discrete needs weights");
    std::vector<double> wts(desc->weights, desc->weights + desc->nweights);
    std::vector<int32_t> prob, alias;
    int ncdf = 0;
    uint32_t mask = 0;
    st = build_discrete(wts, prob, alias, ncdf, mask);
    if (st != GR_OK) return st;
    const size_t np = prob.size();
    std::vector<int32_t> both(prob);
    both.insert(both.end(), alias.begin(), alias.end());
    const int64_t npk = (int64_t)n / 4, W = 4 * ((npk + 1) / 2);
    int32_t* table = nullptr;
    uint64_t* w = nullptr;
    GR_CUDA(cudaMallocAsync(&table, sizeof(int32_t) * (both.size() + 1), s));
    cudaError_t err = cudaMemcpyAsync(table, both.data(), sizeof(int32_t) * both.size(), cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess) err = cudaMallocAsync(&w, sizeof(uint64_t) * (size_t)W, s);
    if (err != cudaSuccess) {
      cudaFreeAsync(table, s);
      return cuda_fail(err, "scalar engine discrete table");
    }
    // the pageable source is staged before the copy call returns
    DistParams dd{};
    dd.kind = GR_DISCRETE;
    dd.dtype = GR_I32;
    dd.ncdf = ncdf;
    dd.bitmask = mask;
    dd.prob = table;
    dd.alias = table + np;
    st = sengine_words(se, w, W, s);
    if (st == GR_OK) {
      err = launch_scalar_xform(w, dev_out, npk, dd, s);
      if (err != cudaSuccess) st = cuda_fail(err, "scalar-engine sampling kernel");
    }
    cudaFreeAsync(w, s);
    cudaFreeAsync(table, s);
    return st;
  }
  DistParams dp{};
  st = make_params(*desc, dp);
  if (st != GR_OK) return st;
  if (dp.dtype == GR_I32 && (dp.kind == GR_POISSON || dp.kind == GR_BINOMIAL || dp.kind == GR_UNIFORM_INT ||
                             dp.kind == GR_NEGATIVE_BINOMIAL))
    return sengine_int(se, dp, dev_out, n, s);
  if (dp.kind == GR_GAMMA && reject_code(dp) >= 0 && family_of(dp) == Family::Reject)
    return sengine_reject(se, dp, reject_code(dp), dev_out, n, s);
  if (dp.kind == GR_BETA && dp.dtype != GR_I32) return sengine_beta(se, dp, dev_out, n, s);
  if (dp.dtype != GR_I32 && family_of(dp) == Family::Staged && (dp.kind == GR_GAMMA || dp.kind == GR_STUDENT_T)) {
    // a fixed run of U uniform packets per output packet: all words at once
    const int U = dp.kind == GR_GAMMA ? dp.ib : 2;
    const int64_t P = dp.dtype == GR_F32 ? 8 : 4;
    if (n % (size_t)P) return fail(GR_ERR_INVALID, "size must be a multiple of the reference packet width");
    if (n == 0) return GR_OK;
    if (!dev_out) return fail(GR_ERR_INVALID, "output is NULL");
    const int64_t npk = (int64_t)n / P, W = npk * U * (dp.dtype == GR_F32 ? 3 : 4);
    uint64_t* w = nullptr;
    GR_CUDA(cudaMallocAsync(&w, sizeof(uint64_t) * (size_t)W, s));
    st = sengine_words(se, w, W, s);
    if (st == GR_OK) {
      const cudaError_t err = launch_sx_staged(w, dev_out, npk, dp, U, s);
      if (err != cudaSuccess) st = cuda_fail(err, "scalar-engine sampling kernel");
    }
    cudaFreeAsync(w, s);
    return st;
  }
  const int wpp = scalar_words_per_packet(dp.kind, dp.dtype);
  if (wpp == 0 || (dp.kind == GR_GAMMA && dp.ia != 1))
    return fail(GR_ERR_UNSUPPORTED, "scalar engines: the fixed-draw kinds only (uniformReal, balanced, normal, "
                                    "lognormal, exponential, cauchy, weibull, extremeValue, gamma(1), bernoulli, "
                                    "randBits), gamma, chiSquared, studentT, beta, fisherF, poisson, binomial, "
                                    "negativeBinomial, uniformInt, geometric and discrete");
  const int64_t P = kind_granule(dp.kind, dp.dtype);
  // a partial last packet: the scalar operator(), one draw per element (the
  // kinds whose scalar form is exact bit arithmetic)
  const int64_t r = (int64_t)(n % (size_t)P);
  if (r && !kind_has_exact_tail(dp.kind, dp.dtype))
    return fail(GR_ERR_INVALID, "size must be a multiple of the reference packet width; a partial last packet is "
                                "supported for uniformReal, balanced, bernoulli and randBits");
  if (n == 0) return GR_OK;
  if (!dev_out) return fail(GR_ERR_INVALID, "output is NULL");
  const int64_t npk = (int64_t)n / P;
  const bool unit2 = dp.kind == GR_NORMAL_STD || dp.kind == GR_NORMAL || dp.kind == GR_LOGNORMAL;
  const int64_t W = wpp * (unit2 ? 2 * ((npk + 1) / 2) : npk);  // a normal unit draws both packets
  uint64_t* w = nullptr;
  GR_CUDA(cudaMallocAsync(&w, sizeof(uint64_t) * (size_t)(W + r), s));
  st = sengine_words(se, w, W + r, s);
  if (st == GR_OK && npk) {
    const cudaError_t err = launch_scalar_xform(w, dev_out, npk, dp, s);
    if (err != cudaSuccess) st = cuda_fail(err, "scalar-engine sampling kernel");
  }
  if (st == GR_OK && r) {
    const size_t es = dp.dtype == GR_F64 ? 8 : 4;
    const cudaError_t err = launch_tail(w + W, static_cast<char*>(dev_out) + (size_t)npk * P * es, (int)r, dp, false, s);
    if (err != cudaSuccess) st = cuda_fail(err, "scalar-engine tail");
  }
  cudaFreeAsync(w, s);
  return st;
}

}  // extern "C"
