/*
 * gpurand.h — C ABI of the GB300 sampling library (libgpurand.so).
 *
 * The drop-in boundary for EigenRand's sampling path (bab2min/EigenRand
 * v0.6.0).  Every entry point takes plain pointers and sizes; device buffers
 * are owned by the caller, engine and generator state lives in HBM and is
 * owned by the library.  Calls are asynchronous on the given CUDA stream and
 * never block, throw or abort; errors come back as gr_status, device-side
 * error words are folded into the next gr_engine_sync().
 *
 * Engines and generators are externally synchronised: use one stream per
 * engine, as EigenRand requires one engine per thread.
 *
 * Every device output array must be 16-byte aligned (cudaMalloc and the
 * caching allocators of the usual frameworks return such pointers): the
 * kernels write whole packets with 16-byte stores.  A misaligned output
 * returns GR_ERR_INVALID before anything is launched.
 *
 * Stream semantics (bit-exact with the reference, AVX2 + Eigen 3.4 profile):
 *   - lane l of a Vmt19937_64 seeded s is std::mt19937_64(s + l), l < 4;
 *   - raw u64 stream R[4k + l] = lane_l[k]  (packet k = 4 lanes);
 *   - u32 word stream W[2i] = low32(R[i]), W[2i+1] = high32(R[i]);
 *   - float outputs use one packet (8 words) per 8 samples, double outputs
 *     one packet per 4 samples, int32 outputs half packets (4 words) per 4
 *     samples, exactly as the reference's packetOp code consumes them.
 * An engine created with streams = K > 1 holds K independent
 * Vmt19937_64(seed + 4k) engines; a call then splits its output into K
 * contiguous slices, slice k generated by engine k — identical to K host
 * threads each running EigenRand on its own engine and slice.
 */
#ifndef GPURAND_H
#define GPURAND_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gr_stream_t; /* == cudaStream_t; NULL = default stream */

typedef enum {
  GR_OK = 0,
  GR_ERR_INVALID = 1,      /* bad argument (size not a multiple of the packet width, NULL, ...) */
  GR_ERR_CUDA = 2,         /* a CUDA runtime call failed; see gr_last_error() */
  GR_ERR_UNSUPPORTED = 3,  /* parameter combination not implemented */
  GR_ERR_NOMEM = 4,        /* device allocation failed */
  GR_ERR_REJECT_LIMIT = 5, /* a rejection loop hit its iteration cap (device word) */
  GR_ERR_NOT_PD = 6,       /* covariance / scale matrix not positive definite */
  GR_ERR_NAN_WEIGHT = 7,   /* non-finite weight sum (AliasMethod, Discrete.h:88) */
  GR_ERR_CANCELLED = 8     /* a served request was cancelled (gr_server_cancel) */
} gr_status;

typedef enum { GR_F32 = 0, GR_F64 = 1, GR_I32 = 2, GR_U64 = 3 } gr_dtype;

/* Distribution kinds.  Parameter meaning follows the reference generator's
 * constructor (a, b in the order of the C++ arguments). */
typedef enum {
  GR_UNIFORM_REAL = 1,  /* StdUniformRealGen (a,b unused); Basic.h:525-591       */
  GR_UNIFORM_REAL2 = 2, /* UniformRealGen(min=a, max=b); Basic.h:598-646          */
  GR_BALANCED = 3,      /* BalancedGen; Basic.h:407-429                           */
  GR_BALANCED2 = 4,     /* Balanced2Gen(a, b); Basic.h:436-467                    */
  GR_NORMAL_STD = 5,    /* StdNormalGen; NormalExp.h:25-83                        */
  GR_NORMAL = 6,        /* NormalGen(mean=a, stdev=b); NormalExp.h:92-136          */
  GR_LOGNORMAL = 7,     /* LognormalGen(mean=a, stdev=b); NormalExp.h:170-210      */
  GR_EXPONENTIAL = 8,   /* ExponentialGen(lambda=a); NormalExp.h:356-399           */
  GR_CAUCHY = 9,        /* CauchyGen(a, b); NormalExp.h:809-856                   */
  GR_WEIBULL = 10,      /* WeibullGen(a, b); NormalExp.h:613-656                  */
  GR_EXTREME_VALUE = 11,/* ExtremeValueGen(a, b); NormalExp.h:689-733             */
  GR_GAMMA = 12,        /* GammaGen(alpha=a, beta=b); NormalExp.h:434-606          */
  GR_BETA = 13,         /* BetaGen(a, b); NormalExp.h:895-977                     */
  GR_STUDENT_T = 14,    /* StudentTGen(n=a); NormalExp.h:241-300                  */
  GR_CHI_SQUARED = 15,  /* ChiSquaredGen(n=a); NormalExp.h:767-802                */
  GR_POISSON = 16,      /* PoissonGen(mean=a); Discrete.h:788-904                 */
  GR_BINOMIAL = 17,     /* BinomialGen(trials, p=a); Discrete.h:911-1053          */
  GR_DISCRETE = 18,     /* DiscreteGen<int32_t,int32_t>(weights); Discrete.h:352-486 */
  GR_RANDBITS = 19,     /* RandbitsGen<int32_t>; Basic.h:378-400                  */
  GR_BINOMIAL_V = 20,   /* BinomialVGen<int32_t>, per-element (trials, p); Discrete.h:1061-1192 */
  GR_BERNOULLI = 21,    /* BernoulliGen(p=a), f32 / f64 / int32; Basic.h:669-708    */
  GR_GEOMETRIC = 22,    /* GeometricGen<int32_t>(p=a); Discrete.h:1338-1376         */
  GR_FISHER_F = 23,     /* FisherFGen(m=a, n=b); NormalExp.h:984-1023             */
  GR_UNIFORM_INT = 24,  /* UniformIntGen<int32_t>(min=a, max=b); Discrete.h:214-336 */
  GR_NEGATIVE_BINOMIAL = 25 /* NegativeBinomialGen<int32_t>(trials, p=a); GammaPoisson.h:28-98 */
} gr_dist_kind;

typedef struct {
  int32_t kind;           /* gr_dist_kind */
  int32_t dtype;          /* GR_F32 / GR_F64 for real kinds, GR_I32 for integer kinds */
  double a, b;            /* scalar parameters */
  int32_t trials;         /* binomial */
  int32_t nweights;       /* discrete */
  const double* weights;  /* discrete, host pointer, copied at gr_gen_create */
} gr_dist_desc;

typedef struct gr_engine gr_engine;
typedef struct gr_gen gr_gen;

/* ---- engines ------------------------------------------------------------
 * Replaces Eigen::Rand::Vmt19937_64 (PacketRandomEngine.h:585-599, the
 * MersenneTwister class :196-415).  lanes = 4: the AVX2 packet engine
 * (Pmt19937_64<Packet8i>).  lanes = 2: the SSE / NEON engine
 * (Pmt19937_64<Packet4i>, :585-588), lanes seed and seed + 1, a Packet4f or
 * Packet2d per packet; it serves the raw stream and the kinds whose packetOp
 * transforms each 32-bit word (float) or 64-bit lane (double) on its own
 * (uniformReal, exponential, cauchy, weibull, extremeValue, gamma with
 * alpha = 1; balanced and bernoulli in float), other calls return
 * GR_ERR_UNSUPPORTED.
 * streams = 1 gives one Vmt19937_64(seed); streams = K > 1 gives K engines
 * seeded seed + 4k (the reference's one-engine-per-thread usage). */
gr_status gr_engine_create(gr_engine** out, uint64_t seed, int32_t lanes, int32_t streams);
gr_status gr_engine_destroy(gr_engine* e);
/* MersenneTwister(x0) / seed(x0), PacketRandomEngine.h:230-265 */
gr_status gr_engine_seed(gr_engine* e, uint64_t seed, gr_stream_t stream);
/* Copy of the engine (AlignedArray deep copy, PacketRandomEngine.h:89-118).
 * Host buffer layout: see gr_engine_state_size(). */
size_t gr_engine_state_size(const gr_engine* e);
gr_status gr_engine_save(const gr_engine* e, void* host_buf, size_t size, gr_stream_t stream);
gr_status gr_engine_restore(gr_engine* e, const void* host_buf, size_t size, gr_stream_t stream);
/* MersenneTwister::discard(num) (:317-323) — num packets.  Long discards
 * jump ahead (x^num mod the characteristic polynomial applied to the lane
 * windows), so the cost does not grow with num. */
gr_status gr_engine_discard(gr_engine* e, uint64_t npackets, gr_stream_t stream);
/* Waits for the engine's stream work and folds device error words. */
gr_status gr_engine_sync(gr_engine* e, gr_stream_t stream);
int32_t gr_engine_streams(const gr_engine* e);

/* Raw stream: makeUniversalRng<uint64_t>(Vmt19937_64) operator()
 * (PacketRandomEngine.h:468-475, 577-583).  n must be a multiple of 4 (2 for
 * a 2-lane engine). */
gr_status gr_raw_u64(gr_engine* e, uint64_t* dev_out, size_t n, gr_stream_t stream);

/* ---- generators ---------------------------------------------------------
 * A generator object mirrors one *Gen instance, including the caches it
 * carries between calls (StdNormalGen::valid, GammaGen::cache_rest_cnt, ...).
 * Weights / parameters are copied at creation. */
gr_status gr_gen_create(gr_gen** out, const gr_dist_desc* desc);
gr_status gr_gen_destroy(gr_gen* g);
/* *Gen::generate(rows, cols, urng) with n = rows * cols, column-major.  A
 * size that is not a whole number of packets ends with the generator's scalar
 * operator(), one engine packet per remaining element, drawn from the last
 * stream (Eigen's linear vectorised assignment loop); served for
 * uniformReal, balanced, bernoulli and randBits, whose scalar forms are exact
 * (Basic.h:386-391, 416-420, 456-460, 533-540, 620-624, 689-693), else
 * GR_ERR_INVALID. */
gr_status gr_generate(gr_gen* g, gr_engine* e, void* dev_out, size_t n, gr_stream_t stream);
/* Free-function form (Eigen::Rand::normal(rows, cols, urng, ...)): a fresh
 * generator for one call. */
gr_status gr_sample(gr_engine* e, const gr_dist_desc* desc, void* dev_out, size_t n, gr_stream_t stream);

/* ---- vectorize-over-params, many parameter sets in one launch ----------
 * Set i (0 <= i < nsets) is drawn from a fresh Vmt19937_64(seed + 4 i) with a
 * fresh generator: exactly what seeding an engine and making one per-call
 * sample of the set would give.  counts[i] samples land at
 * out[offsets[i] .. offsets[i] + counts[i]); a set of c samples draws
 * ceil(c / P) packets and keeps the first c values.
 *   GR_GAMMA      : GammaGen<float>(a[i], b[i]) (NormalExp.h:434-606), float out
 *   GR_BINOMIAL_V : BinomialVGen<int32_t> with (trials[i], a[i] = p)
 *                   (Discrete.h:1124-1192; the reference's binomial(urng,
 *                   ArrayXi, ArrayXf) over a set's repeated parameters), int32 out
 * All arrays are device pointers.  Launch shape (threads per CTA) comes from
 * the library's autotuner, which times the candidates on the first call for
 * a (kind, size) class and caches the winner.  Device errors fold into the
 * engine's status (gr_engine_sync). */
typedef struct {
  int32_t kind;
  int64_t nsets;
  uint64_t seed;
  const float* a;
  const float* b;
  const int32_t* trials;
  const int32_t* counts;
  const int64_t* offsets;
  void* out;
} gr_batch_desc;
gr_status gr_sample_batched(gr_engine* e, const gr_batch_desc* batch, gr_stream_t stream);

/* ---- per-element parameters ---------------------------------------------
 * The reference's vectorized forms (*VGen, and the free functions that take
 * parameter arrays of the output's shape): out[i] is drawn with parameters
 * a[i], b[i].  dev_a / dev_b are device arrays of n elements of the output's
 * type, 16-byte aligned; NULL takes desc->a / desc->b for every element (the
 * overloads with one scalar operand).  The draws are the scalar generator's
 * packet stream, so for every i the value equals that generator built with
 * (a[i], b[i]) at the same stream position.
 *   GR_UNIFORM_REAL2 (min, max)  UniformRealVGen     Basic.h:638-666
 *   GR_BALANCED2 (a, b)          BalancedVGen        Basic.h:472-492
 *   GR_NORMAL (mean, stdev)      NormalVGen          NormalExp.h:139-163
 *   GR_LOGNORMAL (mean, stdev)   LognormalVGen       NormalExp.h:213-236
 *   GR_EXPONENTIAL (lambda)      ExponentialVGen     NormalExp.h:402-427
 *   GR_STUDENT_T (n)             StudentTVGen        NormalExp.h:305-343
 *   GR_WEIBULL (a, b)            WeibullVGen         NormalExp.h:659-686
 *   GR_EXTREME_VALUE (a, b)      ExtremeValueVGen    NormalExp.h:736-765
 *   GR_CAUCHY (a, b)             CauchyVGen          NormalExp.h:859-889
 *   GR_BERNOULLI, GR_F32 (p)     BernoulliVGen<float> Basic.h:711-747
 *   GR_BINOMIAL, GR_I32          BinomialVGen<int32_t> Discrete.h:1124-1192:
 *     dev_a int32 trials (NULL: desc->trials), dev_b float p (NULL: (float)desc->a);
 *     the binomial(urng, trials, p) overloads of Discrete.h:1822-1898
 * The double BernoulliVGen goes through a packet cast the reference leaves to
 * Eigen's generic pcast, which cannot be pinned here: GR_ERR_UNSUPPORTED.
 * gr_sample_v / gr_sample_v2 use a fresh generator (the free functions);
 * gr_generate_v keeps g's caches between calls (NormalVGen's StdNormalGen). */
gr_status gr_sample_v(gr_engine* e, const gr_dist_desc* desc, const void* dev_a, void* dev_out, size_t n,
                      gr_stream_t stream);
gr_status gr_sample_v2(gr_engine* e, const gr_dist_desc* desc, const void* dev_a, const void* dev_b, void* dev_out,
                       size_t n, gr_stream_t stream);
gr_status gr_generate_v(gr_gen* g, gr_engine* e, const void* dev_a, const void* dev_b, void* dev_out, size_t n,
                        gr_stream_t stream);

/* ---- scalar engines as the Urng ------------------------------------------
 * EigenRand also draws from scalar 64-bit engines (RandomEngineType::
 * scalar_fullbit): std::mt19937_64 and P8_mt19937_64 (PacketRandomEngine.h:
 * 430-516, 600-607; the engine of the reference's own tests).  Their packets
 * are built by RawbitsMaker<..., scalar_fullbit> (arch/AVX/RandUtils.h:59-144,
 * arch/SSE/RandUtils.h:22-65): 3 draws per float uniform packet (rawbits_34),
 * 4 per double packet, 2 per half packet, in the order GCC evaluates the
 * intrinsics' arguments (right to left).
 *   gr_sengine_raw_u64: rng() n times.
 *   gr_sengine_sample: a fresh generator (the free functions) of every
 *     univariate kind: uniformReal, balanced, normal, lognormal, exponential,
 *     cauchy, weibull, extremeValue, gamma, chiSquared, studentT, beta,
 *     fisherF, bernoulli; for int32 randBits, bernoulli, geometric,
 *     discrete, uniformInt, poisson, binomial and negativeBinomial.  The
 *     data-dependent kinds run their single chain over chunks of pre-drawn
 *     words and synchronise the stream once per chunk. */
typedef struct gr_sengine gr_sengine;
typedef enum { GR_SCALAR_MT19937_64 = 1, GR_SCALAR_P8_MT19937_64 = 2 } gr_scalar_engine_kind;
gr_status gr_sengine_create(gr_sengine** out, int32_t kind, uint64_t seed);
gr_status gr_sengine_destroy(gr_sengine* e);
gr_status gr_sengine_raw_u64(gr_sengine* e, uint64_t* dev_out, size_t n, gr_stream_t stream);
gr_status gr_sengine_sample(gr_sengine* e, const gr_dist_desc* desc, void* dev_out, size_t n, gr_stream_t stream);
/* binomial(urng, trials, p) with a scalar engine as the Urng (BinomialVGen<
 * int32_t>, Discrete.h:1124-1192,1822-1898): arguments as gr_sample_v2
 * (desc->kind GR_BINOMIAL, GR_I32).  Each uniform packet takes two 64-bit
 * draws (RawbitsMaker<Packet4i, Rng, uint64_t, scalar_fullbit>::rawbits_34,
 * arch/SSE/RandUtils.h:36-55).  The engine is one chain, so the call runs as
 * one warp over chunks of pre-drawn words and synchronises the stream once per
 * chunk; afterwards the engine stands exactly past the words used.  Other
 * kinds: GR_ERR_UNSUPPORTED. */
gr_status gr_sengine_sample_v2(gr_sengine* e, const gr_dist_desc* desc, const void* dev_a, const void* dev_b,
                               void* dev_out, size_t n, gr_stream_t stream);

/* ---- truncated distributions (EigenRand/Dists/Truncated.h) --------------
 * TruncGen<Base>{base, Support(lower, upper)} (Truncated.h:202-263 and the
 * specialisations :342-964); `base` describes the base generator as for
 * gr_gen_create (a fresh one: its caches start empty), lower / upper are the
 * support and are converted to the base's scalar type first (pass that type's
 * lowest() / max() for an open side, as the reference's default does).
 *   inverse CDF, no rejection: GR_NORMAL_STD, GR_NORMAL (TruncNormalGen,
 *     :276-332), GR_LOGNORMAL, GR_EXPONENTIAL, GR_CAUCHY, GR_EXTREME_VALUE,
 *     GR_WEIBULL, and the uniform family (GR_UNIFORM_REAL[2],
 *     GR_BALANCED[2]: a UniformRealGen over the intersected range);
 *   CompressMask rejection over the base's packets: GR_GAMMA, GR_BETA,
 *     GR_STUDENT_T, GR_CHI_SQUARED, GR_FISHER_F, GR_BERNOULLI (float/double).
 *     This form needs a single-stream engine and synchronises the stream
 *     (it reads back how far each chunk of base packets got).
 * Nesting (TruncGen<TruncGen<B>>, :391-426) is the intersection of the
 * supports over the same base.  lower >= upper (or a support that misses the
 * base's range) is GR_ERR_INVALID. */
gr_status gr_gen_create_truncated(gr_gen** out, const gr_dist_desc* base, double lower, double upper);
/* truncated(rows, cols, urng, base, support) / truncatedNormal(...)
 * (Truncated.h:984-1045): a fresh TruncGen for one call. */
gr_status gr_sample_truncated(gr_engine* e, const gr_dist_desc* base, double lower, double upper, void* dev_out,
                              size_t n, gr_stream_t stream);

/* ---- multivariate generators (EigenRand/MvDists) -------------------------
 * Each object mirrors one Mv*Gen instance: its parameters, the FP64 factor of
 * its covariance / scale matrix (computed on the GPU at creation), and the
 * member generators whose caches persist between calls (StdNormalGen,
 * ChiSquaredGen per diagonal, GammaGen per category, DiscreteGen).  Host
 * matrices are column-major dim x dim doubles; outputs are device buffers in
 * the reference's layout:  *_sample(..., samples) == generate(urng, samples).
 * The draws use the engine exactly as the reference's member generators do,
 * so the normal / chi-squared / gamma / discrete streams are the reference's;
 * the linear algebra after them is float (FP64 for GR_F64 objects).
 * Creation synchronises the device; the first call of a given size may
 * allocate scratch, so make it before any stream capture. */
typedef struct gr_mvnormal gr_mvnormal;
typedef struct gr_wishart gr_wishart;
typedef struct gr_dirichlet gr_dirichlet;
typedef struct gr_multinomial gr_multinomial;

/* matrix_form: how `matrix` is given (MvNormal.h:42-46 tags) */
typedef enum {
  GR_MATRIX_FULL = 0,  /* covariance / scale matrix: factored by get_lt (MvNormal.h:21-38):
                          Cholesky, or V sqrt(max(lambda, 0)) when it is not positive definite */
  GR_MATRIX_LOWER = 1  /* already the factor: lower_triangular (MvNormalGen, WishartGen) or
                          inv_lower_triangular (InvWishartGen: factor of the inverse scale) */
} gr_matrix_form;

/* MvNormalGen<float|double>(mean, matrix[, lower_triangular]) (MvNormal.h:56-116).
 * sample: dev_out = dim x samples column-major, X = L Z + mean with Z the
 * generator's StdNormalGen draws of dim * samples values (a multiple of the
 * packet width: 8 for float, 4 for double).  Float: L Z on the tensor cores
 * as 3xTF32 with FP32 accumulation; dim <= 2048 (float), <= 800 (double). */
gr_status gr_mvnormal_create(gr_mvnormal** out, int32_t dtype, int32_t dim, const double* mean, const double* matrix,
                             int32_t matrix_form);
gr_status gr_mvnormal_sample(gr_mvnormal* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream);
gr_status gr_mvnormal_destroy(gr_mvnormal* g);

/* WishartGen (inverse = 0, MvNormal.h:185-277) / InvWishartGen (inverse = 1,
 * :347-442) with df > dim - 1.  sample: dev_out = dim x (dim * samples)
 * column-major (draw j in columns j*dim ..).  samples and
 * samples * dim * (dim - 1) / 2 must be multiples of the packet width.
 * Float and dim <= 128: Bartlett products on the tensor cores (3xTF32). */
gr_status gr_wishart_create(gr_wishart** out, int32_t dtype, int32_t dim, int64_t df, const double* matrix,
                            int32_t matrix_form, int32_t inverse);
gr_status gr_wishart_sample(gr_wishart* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream);
gr_status gr_wishart_destroy(gr_wishart* g);

/* DirichletGen(alpha) (Multinomial.h:160-204), alpha[i] > 0.  sample:
 * dev_out = dim x samples column-major; samples a multiple of the packet width. */
gr_status gr_dirichlet_create(gr_dirichlet** out, int32_t dtype, int32_t dim, const double* alpha);
gr_status gr_dirichlet_sample(gr_dirichlet* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream);
gr_status gr_dirichlet_destroy(gr_dirichlet* g);

/* MultinomialGen<int32_t>(trials, weights) (Multinomial.h:25-118), weights
 * >= 0.  sample: dev_out = int32 dim x samples column-major, bit-exact with
 * the reference.  trials < max(30 (dim - 1), 100): the per-trial DiscreteGen
 * path (trials <= 2400); above: the conditional-binomial path
 * (BinomialVGen<float> row by row), which needs samples % 8 == 0. */
gr_status gr_multinomial_create(gr_multinomial** out, int32_t dim, int32_t trials, const double* weights);
gr_status gr_multinomial_sample(gr_multinomial* g, gr_engine* e, int32_t* dev_out, size_t samples,
                                gr_stream_t stream);
gr_status gr_multinomial_destroy(gr_multinomial* g);

/* TruncMvNormalGen<T>(mean, cov | lt, support(lower, upper), burn_in)
 * (MvDists/TruncMvNormal.h:31-209): Gibbs chains, one per sample, through the
 * precision matrix; burn_in sweeps (0 = 5 * dim).  The factor comes from
 * get_lt (GR_MATRIX_FULL) or is the given lower triangle (GR_MATRIX_LOWER);
 * the precision matrix is computed in FP64 and rounded to T.  dim <= 64,
 * lower[i] < upper[i].  sample: dev_out = dim x samples column-major; the
 * draws are the reference's scalar draws (one engine packet each).  Values
 * match the reference within the rounding of erfc and of the dot products
 * (tolerance stated in the tests), not bit for bit. */
typedef struct gr_truncmvn gr_truncmvn;
gr_status gr_truncmvn_create(gr_truncmvn** out, int32_t dtype, int32_t dim, const double* mean, const double* matrix,
                             int32_t matrix_form, const double* lower, const double* upper, int64_t burn_in);
gr_status gr_truncmvn_sample(gr_truncmvn* g, gr_engine* e, void* dev_out, size_t samples, gr_stream_t stream);
gr_status gr_truncmvn_destroy(gr_truncmvn* g);

/* ---- serving loop ----------------------------------------------------------
 * No counterpart in the reference (EigenRand is a library called in-process);
 * this is the request loop the sampling path is deployed behind.  Each client
 * owns a device-resident Vmt19937_64 (streams = 1) seeded by the caller.
 * Requests of mixed kinds and sizes queue in arrival order and are admitted
 * while stream slots are free and their output fits the device-memory budget;
 * admitted requests run concurrently on the GPU and complete out of order.  A
 * client's requests run one at a time, in submission order, so every result
 * equals that client's plain call sequence run alone: gr_sample (a fresh
 * generator per request, the free-function form) or, for GR_SERVE_MVNORMAL,
 * the client's own MvNormalGen.  Results stay in budgeted device memory until
 * gr_server_release().  Not thread-safe: drive a server from one thread. */
#define GR_SERVE_MVNORMAL 64 /* gr_request.kind: MvNormalGen set by gr_server_set_mvnormal */
typedef struct gr_server gr_server;
typedef struct {
  int32_t client;   /* 0 <= client < nclients */
  int32_t kind;     /* a univariate gr_dist_kind value except GR_DISCRETE and GR_BINOMIAL_V, or GR_SERVE_MVNORMAL */
  int32_t dtype;    /* GR_F32 / GR_F64 (GR_I32 for the integer kinds) */
  int32_t trials;   /* binomial */
  double a, b;      /* as gr_dist_desc */
  uint64_t count;   /* output scalars; rounded up to the packet width (MvNormal: to whole samples) */
  double arrival;   /* gr_server_now() time the request arrived; < 0 means now */
} gr_request;
typedef struct {
  uint64_t ticket;
  int32_t status;   /* gr_status of the request */
  int32_t client;
  void* dev_out;    /* the result in device memory, valid until gr_server_release */
  uint64_t count;   /* scalars written */
  size_t bytes;
  double arrival, admitted, completed; /* gr_server_now() seconds */
} gr_completion;
gr_status gr_server_create(gr_server** out, int32_t nclients, const uint64_t* seeds, size_t budget_bytes,
                           int32_t slots);
/* the MvNormalGen<float>(mean, cov) every client uses for GR_SERVE_MVNORMAL (one factorisation, a
 * StdNormalGen per client) */
gr_status gr_server_set_mvnormal(gr_server* s, int32_t dim, const double* mean, const double* cov);
/* queues a request; GR_ERR_NOMEM if its output can never fit the budget */
gr_status gr_server_submit(gr_server* s, const gr_request* r, uint64_t* ticket);
/* non-blocking: harvests finished requests, admits queued ones, reports up to cap completions */
gr_status gr_server_progress(gr_server* s, gr_completion* done, size_t cap, size_t* ndone);
/* copies a finished result to host memory (synchronous) */
gr_status gr_server_read(gr_server* s, uint64_t ticket, void* host_dst, size_t bytes);
/* ends a reported request (any status): gives its memory back to the budget */
gr_status gr_server_release(gr_server* s, uint64_t ticket);
/* Cancels a request that has not been reported yet.  Queued: it is dropped
 * and nothing runs, so the client's engine is not advanced (the client's
 * later results equal its call sequence without it).  Running: the GPU work
 * completes (its draws are consumed, as in the call sequence with it) and the
 * result is freed when it does.  Either way the request is then reported by
 * gr_server_progress with status GR_ERR_CANCELLED and no result, and is ended
 * by gr_server_release like any other.  GR_ERR_INVALID if the ticket is
 * unknown or its completion was already reported. */
gr_status gr_server_cancel(gr_server* s, uint64_t ticket);
/* gr_server_cancel for every unreported request of a client (a client that
 * went away); its finished, reported results still need gr_server_release */
gr_status gr_server_cancel_client(gr_server* s, int32_t client);
/* test hook: the next n result allocations fail as if the server's memory
 * pool were exhausted (those requests complete with GR_ERR_NOMEM, nothing
 * runs for them and the client's engine is not advanced) */
gr_status gr_server_fail_allocs(gr_server* s, int32_t n);
gr_status gr_server_pending(const gr_server* s, size_t* queued, size_t* running, size_t* bytes_held);
double gr_server_now(void);
gr_status gr_server_destroy(gr_server* s);

const char* gr_last_error(void);
const char* gr_version(void);

/* ---- allocation-free raw stream ------------------------------------------
 * No counterpart in the reference (EigenRand runs on the host and never
 * allocates device memory).  Same output and engine advance as gr_raw_u64,
 * for callers that must not allocate device memory on their sampling path —
 * for example a plugin whose host framework owns all device memory, or a
 * thread with a real-time budget.  The engine is created once at set-up
 * (streams = 1 only); the call then allocates nothing: its jump-ahead scratch
 * and the jump polynomials of every segment length it can use are a
 * file-scope __device__ array of about 1.9 MiB that every GPU loading the
 * library keeps until process exit.  n <= GR_NOALLOC_MAX_DRAWS, else
 * GR_ERR_INVALID; a call runs as at most 32 jump-ahead segments.  Calls share
 * that array, so calls that overlap on the GPU race and must be serialised by
 * the caller.  The first call on a device performs one-time set-up with that
 * device current (the array's address, the kernels' code, the jump
 * polynomials computed on the host and copied in synchronously); make it
 * before any stream capture. */
#define GR_NOALLOC_MAX_DRAWS 4294967296ull
gr_status gr_raw_u64_noalloc(gr_engine* e, uint64_t* dev_out, size_t n, gr_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
