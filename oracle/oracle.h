/*
 * CPU ORACLE — test infrastructure only.
 *
 * A plain-C restatement of EigenRand's sampling hot path (bab2min/EigenRand
 * v0.6.0), used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline as the checker.  Nothing in the shipped library links or calls it.
 *
 * Reference profile that is emulated: x86-64 AVX2 with Eigen 3.4, i.e.
 *   Vmt19937_64 = Pmt19937_64<Packet8i> (4 u64 lanes, lane l seeded seed+l),
 *   float packets of 8, double packets of 4, int32 packets of 4 (Eigen 3.4
 *   keeps integer packets on SSE when AVX2 is on).
 *
 * Transcendentals: log/exp are the library's own published-method
 * implementations (float: Cody-Waite reduction + fitted polynomial; double:
 * Tang's table-driven methods, tables in ormath_tables.h), restated
 * independently here; sin/cos are EigenRand's own psincos
 * (EigenRand/MorePacketMath.h:297-491) restated; sqrt and division are IEEE.
 * Every float operation is rounded individually (-ffp-contract=off).
 *
 * Pins: the MT19937-64 lane against libstdc++ std::mt19937_64 and the C++
 * standard's known answer (pin_mt.cpp).  Beyond the engine, parity with the
 * reference is unpinned: the reference needs Eigen (absent here) and ships
 * no golden vectors, so the transforms are checked as restatements of its
 * source (file:line at each function) and by distribution tests.
 */
#ifndef GR_ORACLE_H
#define GR_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- one MT19937-64 lane, literal restatement of MersenneTwister --------- */
typedef struct {
  uint64_t state[624]; /* double buffer, PacketRandomEngine.h:406 */
  int idx;             /* stateIdx */
} or_mt64;

void or_mt64_seed(or_mt64* s, uint64_t seed);
uint64_t or_mt64_next(or_mt64* s);

/* ---- packet engine (Vmt19937_64 / P8 raw stream) ------------------------- */
#define OR_MAXL 8
typedef struct {
  int L;
  or_mt64 lane[OR_MAXL];
  int half_valid;               /* MersenneTwister::half() cache, :325-336 */
  uint32_t half_cache[OR_MAXL]; /* upper half of the last split packet      */
} or_vmt;

or_vmt* or_vmt_new(uint64_t seed, int lanes);
void or_vmt_free(or_vmt* e);
void or_vmt_copy(or_vmt* dst, const or_vmt* src);
size_t or_vmt_sizeof(void);
void or_vmt_raw(or_vmt* e, uint64_t* out, size_t npackets);
void or_vmt_discard(or_vmt* e, uint64_t npackets);
/* raw words of the last 312 outputs of each lane (untempered), for engine
 * state comparison: out[l*312 + i] */
void or_vmt_window(const or_vmt* e, uint64_t* out);

/* ---- scalar engines as the Urng: std::mt19937_64, P8_mt19937_64 --------- */
enum { OR_SENG_MT19937_64 = 1, OR_SENG_P8_MT19937_64 = 2 };
typedef struct {
  int kind;
  or_mt64 mt;        /* std::mt19937_64 */
  or_vmt *a, *b;     /* P8: Vmt19937_64(seed), Vmt19937_64(seed + 4) */
  uint64_t buf[8];   /* P8: the current eight lanes */
  int cnt;           /* P8: lanes handed out of buf (8 = empty) */
} or_seng;
or_seng* or_seng_new(int kind, uint64_t seed);
void or_seng_free(or_seng* s);
void or_seng_raw(or_seng* s, uint64_t* out, size_t n);

/* ---- generator state (caches that EigenRand keeps inside *Gen objects) --- */
typedef struct {
  int valid;          /* StdNormalGen / DiscreteGen packet cache flag        */
  uint32_t cache[16]; /* cached packet (up to 64 bytes)                      */
  int rest_cnt;       /* CompressMask::compress_append carry count           */
  uint32_t rest[16];  /* carried accepted lanes                              */
} or_gen;
size_t or_gen_sizeof(void);

/* Distribution families.  n must be a multiple of the packet width
 * (8 float / 4 double / 4 int32).  Returns 0 on success, nonzero on error.
 * dtype: 0 = float32, 1 = float64. */
enum {
  OR_UNIFORM = 1,   /* a=min, b=max (UniformRealGen); std form when a=0,b=1 */
  OR_BALANCED = 2,  /* a, b (Balanced2Gen); a=-1,b=1 is BalancedGen          */
  OR_NORMAL = 3,    /* a=mean, b=stdev                                        */
  OR_LOGNORMAL = 4, /* a=mean, b=stdev                                        */
  OR_EXPONENTIAL = 5, /* a=lambda                                             */
  OR_CAUCHY = 6,    /* a, b                                                   */
  OR_WEIBULL = 7,   /* a=shape, b=scale                                       */
  OR_EXTREME = 8,   /* a=location, b=scale                                    */
  OR_GAMMA = 9,     /* a=alpha, b=beta                                        */
  OR_BETA = 10,     /* a, b                                                   */
  OR_STUDENT_T = 11,  /* a = n                                                */
  OR_CHI_SQUARED = 12, /* a = n                                              */
  OR_STDNORMAL = 13,  /* StdNormalGen: no mean/stdev scaling                  */
  OR_BERNOULLI = 14,  /* a = p; BernoulliGen<float/double>                    */
  OR_FISHER_F = 15    /* a = m, b = n; FisherFGen                             */
};
int or_gen_real(or_vmt* e, or_gen* g, int dist, int dtype, double a, double b,
                void* out, size_t n);
/* per-element forms (*VGen): parameters a[i] / b[i] (NULL: the scalars) */
int or_gen_real_v(or_vmt* e, or_gen* g, int dist, int dtype, const void* av, const void* bv, double sa, double sb,
                  void* out, size_t n);
/* or_gen_real / or_gen_randbits with a scalar engine as the Urng */
int or_sgen_real(or_seng* s, or_gen* g, int dist, int dtype, double a, double b, void* out, size_t n);
int or_sgen_binomial_v(or_seng* s, const int32_t* trials, const float* p, int32_t trials0, float p0, int32_t* out,
                       size_t n);
int or_sgen_int(or_seng* s, int kind, int32_t trials, double a, int32_t* out, size_t n);
int or_sgen_randbits(or_seng* s, int32_t* out, size_t n);
/* TruncGen<Base>{base, Support(lower, upper)} (Truncated.h); g: four slots */
int or_gen_trunc(or_vmt* e, or_gen* g, int dist, int dtype, double a, double b, double lower, double upper,
                 void* out, size_t n);

/* int32 distributions */
int or_gen_binomial(or_vmt* e, or_gen* g, int32_t trials, double p, int32_t* out, size_t n);
int or_gen_poisson(or_vmt* e, or_gen* g, double mean, int32_t* out, size_t n);
int or_gen_randbits(or_vmt* e, int32_t* out, size_t n);
int or_gen_bernoulli_i32(or_vmt* e, double p, int32_t* out, size_t n);
int or_gen_geometric(or_vmt* e, double p, int32_t* out, size_t n);
int or_gen_uniform_int(or_vmt* e, or_gen* g, int32_t mn, int32_t mx, int32_t* out, size_t n);
int or_gen_negative_binomial(or_vmt* e, or_gen* g, int32_t trials, double p, int32_t* out, size_t n);
int or_gen_bernoulli_v_f32(or_vmt* e, const float* pv, float* out, size_t n);

/* discrete with int32 precision (DiscreteGen<int32_t, int32_t>) */
typedef struct {
  int use_cdf;
  int n;             /* number of weights */
  uint32_t cdf[64];  /* used when n < 16 */
  int bitsize;       /* alias table: 2^bitsize entries */
  uint32_t bitmask;
  int32_t* prob;
  int32_t* alias;
} or_discrete;
or_discrete* or_discrete_new(const double* w, int n);
void or_discrete_free(or_discrete* d);
int or_discrete_table(const or_discrete* d, int32_t* prob, int32_t* alias, int cap);
int or_gen_discrete(or_vmt* e, or_gen* g, const or_discrete* d, int32_t* out, size_t n);
int or_sgen_discrete(or_seng* s, const or_discrete* d, int32_t* out, size_t n);
/* MultinomialGen<int32_t>(trials, w) per-trial path; out = dim x samples col-major */
int or_gen_multinomial(or_vmt* e, or_gen* g, const or_discrete* d, int32_t trials, int32_t dim, int32_t* out,
                       size_t samples);

/* vectorize-over-params */
int or_binomial_v_packet(or_vmt* e, const int32_t* trials, const float* p, int32_t* out);
int or_gen_binomial_v(or_vmt* e, const int32_t* trials, const float* p, int32_t trials0, float p0, int32_t* out,
                      size_t n);
/* TruncMvNormalGen Gibbs chains with the precision matrix H (FP64, column-major) */
int or_gen_truncmvn(or_vmt* e, int dtype, int dim, const double* H, const double* mean, const double* lower,
                    const double* upper, int64_t burn_in, void* out, size_t samples);
/* MultinomialGen, conditional-binomial path (trials >= max(30 (dim-1), 100)) */
double or_eigen_sum_avx(const double* v, int n);
int or_gen_multinomial_cond(or_vmt* e, const double* w, int32_t dim, int32_t trials, int32_t* out,
                            size_t samples);
int or_vop_set(uint64_t seed, int kind, double a, double b, int32_t trials, void* out, size_t count);

/* ---- math (library's own log/exp; EigenRand psincos restated) ---------- */
float or_logf(float x);
float or_expf(float x);
double or_log(double x);
double or_exp(double x);
/* CPU-baseline timing mode: or_log / or_exp become the C library's FP64
 * log / exp (never used for parity) */
void or_set_fp_math(int on);
void or_sincosf(float x, float* s, float* c);
void or_sincos(double x, double* s, double* c);
float or_lgamma_approxf(float x);
float or_erfinvf(float x);
double or_erfinv(double x);
double or_lgamma_approx(double x);
void or_vec_logf(const float* x, float* y, size_t n);
void or_vec_expf(const float* x, float* y, size_t n);
void or_vec_erfinvf(const float* x, float* y, size_t n);
void or_vec_erfinv(const double* x, double* y, size_t n);
void or_vec_log(const double* x, double* y, size_t n);
void or_vec_exp(const double* x, double* y, size_t n);
void or_vec_sincosf(const float* x, float* s, float* c, size_t n);
void or_vec_sincos(const double* x, double* s, double* c, size_t n);

#ifdef __cplusplus
}
#endif
#endif
