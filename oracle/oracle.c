/*
 * CPU ORACLE — engine and generators.  Test infrastructure only; see oracle.h.
 *
 * Restates, lane by lane, what EigenRand's packet code computes under the
 * AVX2 + Eigen 3.4 profile.  File:line citations are into bab2min/EigenRand.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint64_t d2u(double f) { uint64_t u; memcpy(&u, &f, 8); return u; }
static inline double u2d(uint64_t u) { double f; memcpy(&f, &u, 8); return f; }

#define PI_D 3.1415926535897932 /* Dists/Basic.h:23 */
#define E_D 2.7182818284590452  /* Dists/Basic.h:24 */

/* ======================================================================
 * MT19937-64 lane: PacketRandomEngine.h:256-265 (seed), :295-310 (temper),
 * :340-404 (refill_lower / refill_upper), constants :421-426.
 * ====================================================================== */
#define MT_N 312
#define MT_M 156
#define MT_A 0xb5026f5aa96619e9ull
#define MT_F 6364136223846793005ull
#define MT_HMASK (~0ull << 31)
#define MT_LMASK (~MT_HMASK)

static inline uint64_t mt_twist1(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t tmp = (a & MT_HMASK) | (b & MT_LMASK);
  return (tmp >> 1) ^ ((tmp & 1) ? MT_A : 0) ^ c;
}

void or_mt64_seed(or_mt64* s, uint64_t seed) {
  uint64_t prev = s->state[0] = seed;
  for (int i = 1; i < MT_N; ++i) {
    prev = s->state[i] = (prev ^ (prev >> 62)) * MT_F + (uint64_t)i;
  }
  for (int i = MT_N; i < 2 * MT_N; ++i) s->state[i] = 0;
  s->idx = MT_N;
}

static void mt_refill_upper(or_mt64* s) {
  for (int i = MT_N; i < 2 * MT_N; ++i)
    s->state[i] = mt_twist1(s->state[i - MT_N], s->state[i - MT_N + 1], s->state[i - MT_N + MT_M]);
}

static void mt_refill_lower(or_mt64* s) {
  int i;
  for (i = 0; i < MT_N - MT_M; ++i)
    s->state[i] = mt_twist1(s->state[i + MT_N], s->state[i + MT_N + 1], s->state[i + MT_N + MT_M]);
  for (; i < MT_N - 1; ++i)
    s->state[i] = mt_twist1(s->state[i + MT_N], s->state[i + MT_N + 1], s->state[i - MT_N + MT_M]);
  s->state[i] = mt_twist1(s->state[i + MT_N], s->state[0], s->state[MT_M - 1]);
  s->idx = 0;
}

uint64_t or_mt64_next(or_mt64* s) {
  if (s->idx == MT_N)
    mt_refill_upper(s);
  else if (2 * MT_N <= s->idx)
    mt_refill_lower(s);
  uint64_t r = s->state[s->idx++];
  r ^= (r >> 29) & 0x5555555555555555ull;
  r ^= (r << 17) & 0x71d67fffeda60000ull;
  r ^= (r << 37) & 0xfff7eee000000000ull;
  r ^= r >> 43;
  return r;
}

/* last 312 raw words produced (or the seed words before the first twist) */
static void mt_window(const or_mt64* s, uint64_t* out) {
  /* the 312 words preceding state[idx] in the cyclic double buffer */
  for (int i = 0; i < MT_N; ++i) {
    int j = s->idx - MT_N + i;
    if (j < 0) j += 2 * MT_N;
    out[i] = s->state[j];
  }
}

/* ======================================================================
 * Packet engine.  Lane l = MT19937-64 seeded seed+l (:230-239).
 * ====================================================================== */
or_vmt* or_vmt_new(uint64_t seed, int lanes) {
  if (lanes < 1 || lanes > OR_MAXL) return NULL;
  or_vmt* e = (or_vmt*)calloc(1, sizeof(or_vmt));
  e->L = lanes;
  for (int l = 0; l < lanes; ++l) or_mt64_seed(&e->lane[l], seed + (uint64_t)l);
  return e;
}
void or_vmt_free(or_vmt* e) { free(e); }
void or_vmt_copy(or_vmt* dst, const or_vmt* src) { memcpy(dst, src, sizeof(or_vmt)); }
size_t or_vmt_sizeof(void) { return sizeof(or_vmt); }
size_t or_gen_sizeof(void) { return sizeof(or_gen); }

static void vmt_packet(or_vmt* e, uint64_t* r) {
  for (int l = 0; l < e->L; ++l) r[l] = or_mt64_next(&e->lane[l]);
}

void or_vmt_raw(or_vmt* e, uint64_t* out, size_t npackets) {
  for (size_t k = 0; k < npackets; ++k) vmt_packet(e, out + k * (size_t)e->L);
}

void or_vmt_discard(or_vmt* e, uint64_t npackets) {
  uint64_t r[OR_MAXL];
  for (uint64_t k = 0; k < npackets; ++k) vmt_packet(e, r);
}

void or_vmt_window(const or_vmt* e, uint64_t* out) {
  for (int l = 0; l < e->L; ++l) mt_window(&e->lane[l], out + (size_t)l * MT_N);
}

/* ======================================================================
 * Scalar engines as the Urng (RandomEngineType::scalar_fullbit): a
 * std::mt19937_64, or P8_mt19937_64 = ParallelRandomEngineAdaptor over two
 * Vmt19937_64(seed), (seed + 4) whose operator() returns the eight lanes of
 * one packet of each in turn (PacketRandomEngine.h:430-516, 600-607).  While
 * g_src is set, the packet primitives below draw through
 * RawbitsMaker<Packet8i, Rng, uint64_t, scalar_fullbit> (arch/AVX/RandUtils.h:
 * 59-144) instead of the packet engine:
 *   rawbits      _mm256_set_epi64x(rng(), rng(), rng(), rng())
 *   rawbits_half _mm_set_epi64x(rng(), rng())
 *   rawbits_34   _mm256_setr_epi64x(rng(), rng(), rng(), 0), permuted
 * with GCC's right-to-left argument evaluation (pinned with g++ 13 -mavx2:
 * set_epi64x puts the k-th call in element k; setr_epi64x puts the first call
 * in element 2 and the third in element 0).
 * ====================================================================== */
static or_seng* g_src = NULL;

static uint64_t src_next(void) {
  or_seng* s = g_src;
  if (s->kind == OR_SENG_MT19937_64) return or_mt64_next(&s->mt);
  if (s->cnt >= 8) {
    vmt_packet(s->a, s->buf);
    vmt_packet(s->b, s->buf + 4);
    s->cnt = 0;
  }
  return s->buf[s->cnt++];
}

or_seng* or_seng_new(int kind, uint64_t seed) {
  or_seng* s = (or_seng*)calloc(1, sizeof(or_seng));
  s->kind = kind;
  if (kind == OR_SENG_MT19937_64) {
    or_mt64_seed(&s->mt, seed);
  } else {
    s->a = or_vmt_new(seed, 4);
    s->b = or_vmt_new(seed + 4, 4);
    s->cnt = 8;
  }
  return s;
}

void or_seng_free(or_seng* s) {
  if (!s) return;
  or_vmt_free(s->a);
  or_vmt_free(s->b);
  free(s);
}

void or_seng_raw(or_seng* s, uint64_t* out, size_t n) {
  or_seng* prev = g_src;
  g_src = s;
  for (size_t i = 0; i < n; ++i) out[i] = src_next();
  g_src = prev;
}

/* rawbits: four 64-bit draws, the k-th in element k */
static void raw4(or_vmt* e, uint64_t* r) {
  if (g_src) {
    for (int l = 0; l < 4; ++l) r[l] = src_next();
    return;
  }
  vmt_packet(e, r);
}

/* one engine packet viewed as 2L u32 words (Packet8i for L=4) */
static void draw_full(or_vmt* e, uint32_t* w) {
  uint64_t r[OR_MAXL];
  raw4(e, r);
  for (int l = 0; l < e->L; ++l) {
    w[2 * l] = (uint32_t)r[l];
    w[2 * l + 1] = (uint32_t)(r[l] >> 32);
  }
}

/* MersenneTwister::half(), PacketRandomEngine.h:325-336: split_two gives the
 * low 128 bits now and caches the high 128 bits. */
static void draw_half(or_vmt* e, uint32_t* w) {
  if (g_src) { /* rawbits_half: two draws, the first in element 0 */
    const uint64_t a = src_next(), b = src_next();
    w[0] = (uint32_t)a;
    w[1] = (uint32_t)(a >> 32);
    w[2] = (uint32_t)b;
    w[3] = (uint32_t)(b >> 32);
    return;
  }
  int hw = e->L; /* words in a half packet */
  if (e->half_valid) {
    e->half_valid = 0;
    memcpy(w, e->half_cache, sizeof(uint32_t) * (size_t)hw);
    return;
  }
  uint32_t full[2 * OR_MAXL];
  draw_full(e, full);
  memcpy(w, full, sizeof(uint32_t) * (size_t)hw);
  memcpy(e->half_cache, full + hw, sizeof(uint32_t) * (size_t)hw);
  e->half_valid = 1;
}

/* ======================================================================
 * Uniform building blocks (AVX2 profile)
 *   float  packet (P=8): rawbits_34 = rng()        arch/AVX/RandUtils.h:154-157
 *   float  packet (P=4): rawbits_34 = rng.half()   arch/AVX/RandUtils.h:28-31
 *   double packet (P=4): rawbits    = rng()        arch/AVX/RandUtils.h:149-152
 *   bit_to_ur_float/double                         MorePacketMath.h:205-227
 * ====================================================================== */
static inline float bit_ur_f(uint32_t x) { return u2f((x & 0x7fffffu) | (127u << 23)) - 1.0f; }
static inline double bit_ur_d(uint64_t x) {
  return u2d((x & 0xfffffffffffffull) | (1023ull << 52)) - 1.0;
}

/* rawbits_34 of a scalar engine: setr_epi64x(first, second, third) lands as
 * elements (third, second, first); permutevar8x32 (0,1,2,7,3,4,5,7) and
 * shuffle_epi8 (0..11, 3, 7, 11, 11) per 128-bit half give the words
 * (c.lo, c.hi, b.lo, t0, b.hi, a.lo, a.hi, t1), a/b/c the first/second/third
 * draw and t0 / t1 the top bytes of the half's three words (the third one
 * twice) -- 3 draws for 8 floats, whose low 23 bits are all that is used. */
static void draw_34(uint32_t* w) {
  const uint64_t a = src_next(), b = src_next(), c = src_next();
  const uint32_t v[6] = {(uint32_t)c, (uint32_t)(c >> 32), (uint32_t)b, (uint32_t)(b >> 32), (uint32_t)a,
                         (uint32_t)(a >> 32)};
  w[0] = v[0];
  w[1] = v[1];
  w[2] = v[2];
  w[3] = (v[0] >> 24) | ((v[1] >> 24) << 8) | ((v[2] >> 24) << 16) | ((v[2] >> 24) << 24);
  w[4] = v[3];
  w[5] = v[4];
  w[6] = v[5];
  w[7] = (v[3] >> 24) | ((v[4] >> 24) << 8) | ((v[5] >> 24) << 16) | ((v[5] >> 24) << 24);
}

static void ur_f8(or_vmt* e, float* u) {
  uint32_t w[8];
  if (g_src) draw_34(w); /* uniform_real<Packet8f> = bit_to_ur_float(rawbits_34) */
  else draw_full(e, w);
  for (int j = 0; j < 8; ++j) u[j] = bit_ur_f(w[j]);
}
static void ur_f4(or_vmt* e, float* u) {
  uint32_t w[4];
  draw_half(e, w);
  for (int j = 0; j < 4; ++j) u[j] = bit_ur_f(w[j]);
}
static void ur_d4(or_vmt* e, double* u) {
  uint64_t r[4];
  raw4(e, r);
  for (int j = 0; j < 4; ++j) u[j] = bit_ur_d(r[j]);
}

/* "packet of uniforms" for the generic real generators:
 * width P (8 float / 4 double), stored as double for convenience but the
 * float path keeps every operation in float below. */
typedef struct {
  int dbl;
  float f[8];
  double d[4];
} upk;

static int P_of(int dbl) { return dbl ? 4 : 8; }

static void ur_pk(or_vmt* e, int dbl, upk* p) {
  p->dbl = dbl;
  if (dbl) ur_d4(e, p->d); else ur_f8(e, p->f);
}

/* nonzero_uniform_real = ur + epsilon/8, RandUtils.h:46-51 */
static void nzur_pk(or_vmt* e, int dbl, upk* p) {
  ur_pk(e, dbl, p);
  if (dbl) for (int j = 0; j < 4; ++j) p->d[j] = p->d[j] + 2.220446049250313e-16 / 8;
  else for (int j = 0; j < 8; ++j) p->f[j] = p->f[j] + 1.1920928955078125e-07f / 8;
}

/* zero_to_one (balanced): float: rng() words, cvtepi32_ps / 2^31 (the float
 * constant 0x7FFFFFFF rounds to 2^31).  double: rng.half() words,
 * cvtepi32_pd / 2147483647.  arch/AVX/RandUtils.h:200-204, 215-219 */
static void z2o_pk(or_vmt* e, int dbl, upk* p) {
  p->dbl = dbl;
  if (dbl) {
    uint32_t w[4];
    draw_half(e, w);
    for (int j = 0; j < 4; ++j) p->d[j] = (double)(int32_t)(w[j] & 0x7fffffffu) / 2147483647.0;
  } else {
    uint32_t w[8];
    draw_full(e, w);
    for (int j = 0; j < 8; ++j) p->f[j] = (float)(int32_t)(w[j] & 0x7fffffffu) / (float)0x7FFFFFFF;
  }
}

/* ======================================================================
 * CompressMask::compress_append, arch/AVX/PacketFilter.h:147-184, generic P.
 * Fully accepted packets pass straight through; otherwise accepted lanes are
 * appended, in order, to the carried lanes and a packet is emitted once P
 * lanes are available.  `vals` are raw 32- or 64-bit lane bit patterns.
 * ====================================================================== */
static int compress_append(int P, int wide, void* value, const int* mask, void* rest, int rest_cnt,
                           int* full) {
  int m = 0;
  for (int j = 0; j < P; ++j) m += mask[j] ? 1 : 0;
  if (m == P) {
    *full = 1;
    return rest_cnt;
  }
  uint64_t acc[32];
  int n = 0;
  for (int j = 0; j < rest_cnt; ++j) acc[n++] = wide ? ((uint64_t*)rest)[j] : ((uint32_t*)rest)[j];
  for (int j = 0; j < P; ++j)
    if (mask[j]) acc[n++] = wide ? ((uint64_t*)value)[j] : ((uint32_t*)value)[j];
  if (n >= P) {
    for (int j = 0; j < P; ++j) {
      if (wide) ((uint64_t*)value)[j] = acc[j]; else ((uint32_t*)value)[j] = (uint32_t)acc[j];
    }
    for (int j = P; j < n; ++j) {
      if (wide) ((uint64_t*)rest)[j - P] = acc[j]; else ((uint32_t*)rest)[j - P] = (uint32_t)acc[j];
    }
    *full = 1;
    return n - P;
  }
  for (int j = 0; j < n; ++j) {
    if (wide) ((uint64_t*)rest)[j] = acc[j]; else ((uint32_t*)rest)[j] = (uint32_t)acc[j];
  }
  *full = 0;
  return n;
}

/* ======================================================================
 * Real-valued generators: one packet per call, as *Gen::packetOp does.
 * ====================================================================== */

/* StdNormalGen::packetOp, NormalExp.h:60-82 */
static void stdnormal_pk(or_vmt* e, or_gen* g, int dbl, upk* out) {
  int P = P_of(dbl);
  out->dbl = dbl;
  if (g->valid) {
    g->valid = 0;
    memcpy(dbl ? (void*)out->d : (void*)out->f, g->cache, (size_t)P * (dbl ? 8 : 4));
    return;
  }
  g->valid = 1;
  upk u1, u2;
  ur_pk(e, dbl, &u1);
  ur_pk(e, dbl, &u2);
  if (dbl) {
    double c[4];
    for (int j = 0; j < 4; ++j) {
      double a = 1.0 - u1.d[j];
      double radius = sqrt(-2.0 * or_log(a));
      double theta = (2 * PI_D) * u2.d[j];
      double s, cc;
      or_sincos(theta, &s, &cc);
      c[j] = radius * cc;
      out->d[j] = radius * s;
    }
    memcpy(g->cache, c, sizeof c);
  } else {
    float c[8];
    for (int j = 0; j < 8; ++j) {
      float a = 1.0f - u1.f[j];
      float radius = sqrtf((float)-2 * or_logf(a));
      float theta = (float)(2 * PI_D) * u2.f[j];
      float s, cc;
      or_sincosf(theta, &s, &cc);
      c[j] = radius * cc;
      out->f[j] = radius * s;
    }
    memcpy(g->cache, c, sizeof c);
  }
}

/* GammaGen::packetOp, NormalExp.h:527-605 */
static void gamma_pk(or_vmt* e, or_gen* g, int dbl, double alpha_in, double beta_in, upk* out) {
  int P = P_of(dbl);
  out->dbl = dbl;
  if (dbl) {
    double alpha = alpha_in, beta = beta_in;
    double px = (double)(E_D / (alpha + E_D));
    double sq = sqrt(2 * alpha - 1);
    if (alpha < 1) {
      for (;;) {
        upk ux, vx;
        ur_pk(e, 1, &ux);
        nzur_pk(e, 1, &vx);
        double cands[4];
        int mask[4];
        upk ux2;
        double xx[4], qx[4];
        for (int j = 0; j < 4; ++j) {
          double lv = or_log(vx.d[j]);
          double x1 = or_exp((1 / alpha) * lv);
          double q1 = or_exp(-x1);
          double x2 = 1.0 - lv;
          double q2 = or_exp(or_log(x2) * (alpha - 1));
          int c = ux.d[j] < px;
          xx[j] = c ? x1 : x2;
          qx[j] = c ? q1 : q2;
        }
        ur_pk(e, 1, &ux2);
        for (int j = 0; j < 4; ++j) {
          cands[j] = beta * xx[j];
          mask[j] = ux2.d[j] < qx[j];
        }
        int full = 0;
        g->rest_cnt = compress_append(4, 1, cands, mask, g->rest, g->rest_cnt, &full);
        if (full) {
          memcpy(out->d, cands, sizeof cands);
          return;
        }
      }
    }
    if (alpha == 1) {
      upk u;
      ur_pk(e, 1, &u);
      for (int j = 0; j < 4; ++j) out->d[j] = beta * (-(or_log(1.0 - u.d[j]) / 1.0));
      return;
    }
    int count = (int)alpha;
    if ((double)count == alpha && count < 20) {
      upk y, t;
      nzur_pk(e, 1, &y);
      while (--count) {
        nzur_pk(e, 1, &t);
        for (int j = 0; j < 4; ++j) y.d[j] = y.d[j] * t.d[j];
      }
      for (int j = 0; j < 4; ++j) out->d[j] = -(beta * or_log(y.d[j]));
      return;
    }
    for (;;) {
      double alpha_1 = alpha - 1;
      upk u, ux;
      ur_pk(e, 1, &u);
      double yx[4], xx[4];
      int c[4];
      for (int j = 0; j < 4; ++j) {
        double s, cc;
        or_sincos(PI_D * u.d[j], &s, &cc);
        yx[j] = s / cc;
        xx[j] = sq * yx[j] + alpha_1;
        c[j] = 0 < xx[j];
      }
      ur_pk(e, 1, &ux);
      double cands[4];
      int mask[4];
      for (int j = 0; j < 4; ++j) {
        double ub = (yx[j] * yx[j] + 1) * or_exp(alpha_1 * or_log(xx[j] / alpha_1) - yx[j] * sq);
        mask[j] = c[j] && (ux.d[j] <= ub);
        cands[j] = beta * xx[j];
      }
      int full = 0;
      g->rest_cnt = compress_append(4, 1, cands, mask, g->rest, g->rest_cnt, &full);
      if (full) {
        memcpy(out->d, cands, sizeof cands);
        return;
      }
    }
  } else {
    float alpha = (float)alpha_in, beta = (float)beta_in;
    float px = (float)(E_D / (alpha + E_D));
    float sq = sqrtf(2 * alpha - 1);
    (void)P;
    if (alpha < 1) {
      for (;;) {
        upk ux, vx, ux2;
        ur_pk(e, 0, &ux);
        nzur_pk(e, 0, &vx);
        float xx[8], qx[8];
        for (int j = 0; j < 8; ++j) {
          float lv = or_logf(vx.f[j]);
          float x1 = or_expf((1 / alpha) * lv);
          float q1 = or_expf(-x1);
          float x2 = 1.0f - lv;
          float q2 = or_expf(or_logf(x2) * (alpha - 1));
          int c = ux.f[j] < px;
          xx[j] = c ? x1 : x2;
          qx[j] = c ? q1 : q2;
        }
        ur_pk(e, 0, &ux2);
        float cands[8];
        int mask[8];
        for (int j = 0; j < 8; ++j) {
          cands[j] = beta * xx[j];
          mask[j] = ux2.f[j] < qx[j];
        }
        int full = 0;
        g->rest_cnt = compress_append(8, 0, cands, mask, g->rest, g->rest_cnt, &full);
        if (full) {
          memcpy(out->f, cands, sizeof cands);
          return;
        }
      }
    }
    if (alpha == 1) {
      upk u;
      ur_pk(e, 0, &u);
      for (int j = 0; j < 8; ++j) out->f[j] = beta * (-(or_logf(1.0f - u.f[j]) / 1.0f));
      return;
    }
    int count = (int)alpha;
    if ((float)count == alpha && count < 20) {
      upk y, t;
      nzur_pk(e, 0, &y);
      while (--count) {
        nzur_pk(e, 0, &t);
        for (int j = 0; j < 8; ++j) y.f[j] = y.f[j] * t.f[j];
      }
      for (int j = 0; j < 8; ++j) out->f[j] = -(beta * or_logf(y.f[j]));
      return;
    }
    for (;;) {
      float alpha_1 = alpha - 1;
      upk u, ux;
      ur_pk(e, 0, &u);
      float yx[8], xx[8];
      int c[8];
      for (int j = 0; j < 8; ++j) {
        float s, cc;
        or_sincosf((float)PI_D * u.f[j], &s, &cc);
        yx[j] = s / cc;
        xx[j] = sq * yx[j] + alpha_1;
        c[j] = 0 < xx[j];
      }
      ur_pk(e, 0, &ux);
      float cands[8];
      int mask[8];
      for (int j = 0; j < 8; ++j) {
        float ub = (yx[j] * yx[j] + 1) * or_expf(alpha_1 * or_logf(xx[j] / alpha_1) - yx[j] * sq);
        mask[j] = c[j] && (ux.f[j] <= ub);
        cands[j] = beta * xx[j];
      }
      int full = 0;
      g->rest_cnt = compress_append(8, 0, cands, mask, g->rest, g->rest_cnt, &full);
      if (full) {
        memcpy(out->f, cands, sizeof cands);
        return;
      }
    }
  }
}

/* BetaGen::packetOp, NormalExp.h:949-976 (g: its own cache for the a, b < 1
 * branch; g2, g3: the two GammaGens) */
static void beta_pk(or_vmt* e, or_gen* g, or_gen* g2, or_gen* g3, int dbl, double a, double b, upk* pp) {
  upk p;
  int both_small = dbl ? (a < 1 && b < 1) : ((float)a < 1 && (float)b < 1);
  if (both_small) {
    for (;;) {
      upk u1, u2;
      ur_pk(e, dbl, &u1);
      ur_pk(e, dbl, &u2);
      int mask[8];
      if (dbl) {
        double cands[4];
        for (int j = 0; j < 4; ++j) {
          double p1 = or_exp(or_log(u1.d[j]) * (1 / a));
          double p2 = or_exp(or_log(u2.d[j]) * (1 / b));
          double x = p1 + p2;
          cands[j] = p1 / x;
          mask[j] = x <= 1;
        }
        int full = 0;
        g->rest_cnt = compress_append(4, 1, cands, mask, g->rest, g->rest_cnt, &full);
        if (full) { memcpy(p.d, cands, sizeof cands); break; }
      } else {
        float cands[8];
        float fa = (float)a, fb = (float)b;
        for (int j = 0; j < 8; ++j) {
          float p1 = or_expf(or_logf(u1.f[j]) * (1 / fa));
          float p2 = or_expf(or_logf(u2.f[j]) * (1 / fb));
          float x = p1 + p2;
          cands[j] = p1 / x;
          mask[j] = x <= 1;
        }
        int full = 0;
        g->rest_cnt = compress_append(8, 0, cands, mask, g->rest, g->rest_cnt, &full);
        if (full) { memcpy(p.f, cands, sizeof cands); break; }
      }
    }
  } else {
    upk p1, p2;
    gamma_pk(e, g2, dbl, a, 1, &p1);
    gamma_pk(e, g3, dbl, b, 1, &p2);
    p.dbl = dbl;
    if (dbl) for (int j = 0; j < 4; ++j) p.d[j] = p1.d[j] / (p1.d[j] + p2.d[j]);
    else for (int j = 0; j < 8; ++j) p.f[j] = p1.f[j] / (p1.f[j] + p2.f[j]);
  }
  *pp = p;
}

/* The scalar operator() that fills the elements after the last whole packet
 * of a call (Eigen's linear vectorised assignment loop: packets, then scalars
 * for the remainder).  One draw per element: pfirst of the engine's packet,
 * or one draw of a scalar engine.  pfirst of a Packet8i is its first 32-bit
 * word; ExtractFirstUint<double> (Basic.h:345-371) stores the packet and takes
 * its first 64-bit element; pfirst of a scalar engine's uint64_t draw is the
 * draw.  dtype: 0 float, 1 double, 2 int32.
 *   randBits          pfirst(rng())                         Basic.h:386-391
 *   balanced          ((T)((int32)pfirst & 0x7FFFFFFF) / 0x7FFFFFFF) * 2 - 1   :416-420
 *   balanced(a, b)    ... * slope + bias                     :456-460
 *   uniformReal       to_ur(ExtractFirstUint<T>(rng()))     :533-540
 *   uniformReal(a, b) bias + to_ur(pfirst(rng())) * slope    :620-624
 *   bernoulli         ((uint32)pfirst & 0x7FFFFFFF) < p ? 1 : 0   :689-693 */
static void scalar_tail(or_vmt* e, int dist, int dtype, double a, double b, void* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    uint64_t r;
    int packet = 0;
    if (g_src) {
      r = src_next();
    } else {
      uint64_t pk[OR_MAXL];
      vmt_packet(e, pk);
      r = pk[0];
      packet = 1;
    }
    const uint32_t lo = (uint32_t)r;
    /* pfirst converted to uint64_t: a packet's first int32 word, sign-extended */
    const uint64_t first = packet ? (uint64_t)(int64_t)(int32_t)lo : r;
    if (dist == OR_UNIFORM) {
      const int std_form = a == 0 && b == 1;
      if (dtype == 1) {
        const double u = bit_ur_d(std_form ? r : first);
        ((double*)out)[i] = std_form ? u : a + u * (b - a);
      } else {
        const float fa = (float)a, fb = (float)b;
        const float u = bit_ur_f(lo);
        ((float*)out)[i] = std_form ? u : fa + u * (fb - fa);
      }
    } else if (dist == OR_BALANCED) {
      const int std_form = a == -1 && b == 1;
      const int32_t k = (int32_t)(lo & 0x7FFFFFFFu);
      if (dtype == 1) {
        const double z = (double)k / 2147483647.0;
        ((double*)out)[i] = std_form ? z * 2 - 1 : z * (b - a) + a;
      } else {
        const float fa = (float)a, fb = (float)b;
        const float z = (float)k / (float)0x7FFFFFFF;
        ((float*)out)[i] = std_form ? z * 2 - 1 : z * (fb - fa) + fa;
      }
    } else if (dist == OR_BERNOULLI) {
      const uint32_t pt = (uint32_t)(a * 2147483648.0);
      const int v = ((lo & 0x7FFFFFFFu) < pt) ? 1 : 0;
      if (dtype == 2) ((int32_t*)out)[i] = v;
      else if (dtype == 1) ((double*)out)[i] = v;
      else ((float*)out)[i] = (float)v;
    } else { /* randBits */
      ((int32_t*)out)[i] = (int32_t)lo;
    }
  }
}

/* The SSE / NEON profile: Vmt19937_64 = Pmt19937_64<Packet4i>, two lanes
 * (PacketRandomEngine.h:585-588); a Packet4f takes the engine packet's four
 * 32-bit words, a Packet2d its two 64-bit lanes.  The kinds whose packetOp
 * transforms each word (float) or lane (double) on its own: the same per-lane
 * arithmetic as the AVX2 profile (uniformReal Basic.h:584-590, 638-645;
 * balanced RandUtils.h:36-45 with arch/SSE's float zero_to_one; exponential
 * NormalExp.h:391-398; cauchy :844-855; weibull :648-655; extremeValue
 * :724-732; gamma with alpha = 1, its exponential branch; bernoulli
 * Basic.h:695-707).  Other kinds: 3. */
static int gen_real_sse(or_vmt* e, int dist, int dbl, double a, double b, void* out, size_t n) {
  const size_t P = dbl ? 2 : 4;
  if (n % P) return 2;
  const int supported = dist == OR_UNIFORM || dist == OR_EXPONENTIAL || dist == OR_CAUCHY || dist == OR_WEIBULL ||
                        dist == OR_EXTREME || (!dbl && (dist == OR_BALANCED || dist == OR_BERNOULLI));
  if (!supported) return 3;
  float* of = (float*)out;
  double* od = (double*)out;
  for (size_t k = 0; k < n / P; ++k) {
    uint64_t r[2];
    vmt_packet(e, r);
    for (size_t j = 0; j < P; ++j) {
      if (dbl) {
        const double u = bit_ur_d(r[j]);
        double v;
        switch (dist) {
          case OR_UNIFORM: v = (a == 0 && b == 1) ? u : u * (b - a) + a; break;
          case OR_EXPONENTIAL: v = -(or_log(1.0 - u) / a); break;
          case OR_CAUCHY: {
            double sn, cs;
            or_sincos(PI_D * (u - 0.5), &sn, &cs);
            v = a + b * (sn / cs);
            break;
          }
          case OR_WEIBULL: v = or_exp(or_log(-or_log(1.0 - u)) * (1 / a)) * b; break;
          default: v = a - or_log(-or_log(u + 2.220446049250313e-16 / 8)) * b; break; /* extreme value */
        }
        od[k * P + j] = v;
      } else {
        const uint32_t w = (j & 1) ? (uint32_t)(r[j >> 1] >> 32) : (uint32_t)r[j >> 1];
        const float u = bit_ur_f(w), fa = (float)a, fb = (float)b;
        float v;
        switch (dist) {
          case OR_UNIFORM: v = (a == 0 && b == 1) ? u : u * (fb - fa) + fa; break;
          case OR_BALANCED: {
            const float z = (float)(int32_t)(w & 0x7fffffffu) / (float)0x7FFFFFFF;
            v = (a == -1 && b == 1) ? z * 2.0f - 1.0f : z * (fb - fa) + fa;
            break;
          }
          case OR_EXPONENTIAL: v = -(or_logf(1.0f - u) / fa); break;
          case OR_CAUCHY: {
            float sn, cs;
            or_sincosf((float)PI_D * (u - 0.5f), &sn, &cs);
            v = fa + fb * (sn / cs);
            break;
          }
          case OR_WEIBULL: v = or_expf(or_logf(-or_logf(1.0f - u)) * (1 / fa)) * fb; break;
          case OR_BERNOULLI: v = ((int32_t)(w & 0x7fffffffu) < (int32_t)(uint32_t)(a * 2147483648.0)) ? 1.0f : 0.0f; break;
          default: v = fa - or_logf(-or_logf(u + 1.1920928955078125e-07f / 8)) * fb; break; /* extreme value */
        }
        of[k * P + j] = v;
      }
    }
  }
  return 0;
}

int or_gen_real(or_vmt* e, or_gen* g, int dist, int dtype, double a, double b, void* out, size_t n) {
  int dbl = dtype == 1;
  if (e->L == 2 && !g_src) {
    /* gamma with alpha = 1 is its exponential branch times beta */
    if (dist == OR_GAMMA && a == 1.0) {
      const int rc = gen_real_sse(e, OR_EXPONENTIAL, dbl, 1.0, 0.0, out, n);
      if (rc == 0 && b != 1.0)
        for (size_t i = 0; i < n; ++i) {
          if (dbl) ((double*)out)[i] = b * ((double*)out)[i];
          else ((float*)out)[i] = (float)b * ((float*)out)[i];
        }
      return rc;
    }
    return gen_real_sse(e, dist, dbl, a, b, out, n);
  }
  int P = P_of(dbl);
  /* a partial last packet: the scalar operator() (kinds whose scalar form is exact) */
  const size_t tail = n % (size_t)P;
  if (tail && dist != OR_UNIFORM && dist != OR_BALANCED && dist != OR_BERNOULLI) return 2;
  if (e->L != 4) return 3; /* AVX2 profile only */
  float* of = (float*)out;
  double* od = (double*)out;
  or_gen* g2 = g + 1; /* nested generators (beta: gd1, gd2) */
  or_gen* g3 = g + 2;
  for (size_t k = 0; k < n / (size_t)P; ++k) {
    upk p;
    switch (dist) {
      case OR_UNIFORM: { /* UniformRealGen, Basic.h:638-645; std form :584-590 */
        ur_pk(e, dbl, &p);
        if (dbl) {
          double slope = b - a, bias = a;
          for (int j = 0; j < 4; ++j) p.d[j] = (a == 0 && b == 1) ? p.d[j] : p.d[j] * slope + bias;
        } else {
          float fa = (float)a, fb = (float)b;
          float slope = fb - fa, bias = fa;
          for (int j = 0; j < 8; ++j) p.f[j] = (a == 0 && b == 1) ? p.f[j] : p.f[j] * slope + bias;
        }
        break;
      }
      case OR_BALANCED: { /* RandUtils::balanced, RandUtils.h:36-45 */
        z2o_pk(e, dbl, &p);
        if (dbl) {
          double slope = b - a, bias = a;
          for (int j = 0; j < 4; ++j)
            p.d[j] = (a == -1 && b == 1) ? p.d[j] * 2 - 1 : p.d[j] * slope + bias;
        } else {
          float fa = (float)a, fb = (float)b;
          float slope = fb - fa, bias = fa;
          for (int j = 0; j < 8; ++j)
            p.f[j] = (a == -1 && b == 1) ? p.f[j] * 2.0f - 1.0f : p.f[j] * slope + bias;
        }
        break;
      }
      case OR_STDNORMAL: /* StdNormalGen::packetOp, NormalExp.h:60-82 */
        stdnormal_pk(e, g, dbl, &p);
        break;
      case OR_NORMAL:    /* NormalGen::packetOp, NormalExp.h:127-135 */
      case OR_LOGNORMAL: /* LognormalGen::packetOp, :204-209 */
        stdnormal_pk(e, g, dbl, &p);
        if (dbl) {
          for (int j = 0; j < 4; ++j) {
            p.d[j] = p.d[j] * b + a;
            if (dist == OR_LOGNORMAL) p.d[j] = or_exp(p.d[j]);
          }
        } else {
          for (int j = 0; j < 8; ++j) {
            p.f[j] = p.f[j] * (float)b + (float)a;
            if (dist == OR_LOGNORMAL) p.f[j] = or_expf(p.f[j]);
          }
        }
        break;
      case OR_EXPONENTIAL: /* ExponentialGen::packetOp, NormalExp.h:391-398 */
        ur_pk(e, dbl, &p);
        if (dbl) for (int j = 0; j < 4; ++j) p.d[j] = -(or_log(1.0 - p.d[j]) / a);
        else for (int j = 0; j < 8; ++j) p.f[j] = -(or_logf(1.0f - p.f[j]) / (float)a);
        break;
      case OR_CAUCHY: /* CauchyGen::packetOp, NormalExp.h:844-855 */
        ur_pk(e, dbl, &p);
        if (dbl) {
          for (int j = 0; j < 4; ++j) {
            double s, c;
            or_sincos(PI_D * (p.d[j] - 0.5), &s, &c);
            p.d[j] = a + b * (s / c);
          }
        } else {
          for (int j = 0; j < 8; ++j) {
            float s, c;
            or_sincosf((float)PI_D * (p.f[j] - 0.5f), &s, &c);
            p.f[j] = (float)a + (float)b * (s / c);
          }
        }
        break;
      case OR_WEIBULL: /* WeibullGen::packetOp, NormalExp.h:648-655 */
        ur_pk(e, dbl, &p);
        if (dbl) {
          double ia = 1 / a;
          for (int j = 0; j < 4; ++j) p.d[j] = or_exp(or_log(-or_log(1.0 - p.d[j])) * ia) * b;
        } else {
          float ia = 1 / (float)a;
          for (int j = 0; j < 8; ++j) p.f[j] = or_expf(or_logf(-or_logf(1.0f - p.f[j])) * ia) * (float)b;
        }
        break;
      case OR_EXTREME: /* ExtremeValueGen::packetOp, NormalExp.h:724-732 */
        nzur_pk(e, dbl, &p);
        if (dbl) for (int j = 0; j < 4; ++j) p.d[j] = a - or_log(-or_log(p.d[j])) * b;
        else for (int j = 0; j < 8; ++j) p.f[j] = (float)a - or_logf(-or_logf(p.f[j])) * (float)b;
        break;
      case OR_GAMMA:
        gamma_pk(e, g, dbl, a, b, &p);
        break;
      case OR_BERNOULLI: { /* BernoulliGen::packetOp, Basic.h:695-707: Packet8i rawbits
                            * = rng() (arch/AVX/RandUtils.h:147-152), masked, compared
                            * signed with (int32)(uint32)(p * 2^31); for double the
                            * blend reads the sign of each 64-bit element, i.e. the
                            * compare of its high word (arch/AVX/MorePacketMath.h:583-586) */
        uint32_t w[8];
        draw_full(e, w);
        const int32_t pt = (int32_t)(uint32_t)(a * 2147483648.0);
        p.dbl = dbl;
        if (dbl) for (int j = 0; j < 4; ++j) p.d[j] = ((int32_t)(w[2 * j + 1] & 0x7fffffffu) < pt) ? 1.0 : 0.0;
        else for (int j = 0; j < 8; ++j) p.f[j] = ((int32_t)(w[j] & 0x7fffffffu) < pt) ? 1.0f : 0.0f;
        break;
      }
      case OR_CHI_SQUARED: /* ChiSquaredGen = GammaGen(n/2, 2), NormalExp.h:767-802 */
        gamma_pk(e, g, dbl, dbl ? a * 0.5 : (double)((float)a * 0.5f), 2, &p);
        break;
      case OR_BETA:
        beta_pk(e, g, g2, g3, dbl, a, b, &p);
        break;
      case OR_FISHER_F: { /* FisherFGen: BetaGen(m/2, n/2) in the scalar type, then
                           * (b/a) x / (1 - x), NormalExp.h:997-1021 */
        if (dbl) {
          const double ba = a * 0.5, bb = b * 0.5, c = bb / ba;
          beta_pk(e, g, g2, g3, dbl, ba, bb, &p);
          for (int j = 0; j < 4; ++j) p.d[j] = (c * p.d[j]) / (1.0 - p.d[j]);
        } else {
          const float ba = (float)a * 0.5f, bb = (float)b * 0.5f, c = bb / ba;
          beta_pk(e, g, g2, g3, dbl, ba, bb, &p);
          for (int j = 0; j < 8; ++j) p.f[j] = (c * p.f[j]) / (1.0f - p.f[j]);
        }
        break;
      }
      case OR_STUDENT_T: { /* StudentTGen::packetOp, NormalExp.h:283-299 (psin) */
        upk u1, u2;
        ur_pk(e, dbl, &u1);
        ur_pk(e, dbl, &u2);
        p.dbl = dbl;
        if (dbl) {
          for (int j = 0; j < 4; ++j) {
            double r = sqrt(a * (or_exp(or_log(1.0 - u1.d[j]) * (-2 / a)) - 1));
            double s, c;
            or_sincos((2 * PI_D) * u2.d[j], &s, &c);
            p.d[j] = r * s;
          }
        } else {
          float fa = (float)a;
          for (int j = 0; j < 8; ++j) {
            float r = sqrtf(fa * (or_expf(or_logf(1.0f - u1.f[j]) * (-2 / fa)) - 1));
            float s, c;
            or_sincosf((float)(2 * PI_D) * u2.f[j], &s, &c);
            p.f[j] = r * s;
          }
        }
        break;
      }
      default:
        return 1;
    }
    if (dbl) memcpy(od + k * 4, p.d, 32);
    else memcpy(of + k * 8, p.f, 32);
  }
  if (tail) {
    const size_t at = n - tail;
    scalar_tail(e, dist, dbl, a, b, dbl ? (void*)(od + at) : (void*)(of + at), tail);
  }
  return 0;
}

/* ======================================================================
 * Per-element forms (*VGen): the scalar generator's packet draws with the
 * lane's own parameters a[i], b[i] (NULL array: the scalar sa / sb).
 * UniformRealVGen Basic.h:660-665, BalancedVGen :486-491, NormalVGen
 * NormalExp.h:155-162, LognormalVGen :230-235, StudentTVGen :327-342,
 * ExponentialVGen :420-426, WeibullVGen :679-685, ExtremeValueVGen :757-764,
 * CauchyVGen :879-888.  g holds NormalVGen's StdNormalGen cache.
 * ====================================================================== */
int or_gen_real_v(or_vmt* e, or_gen* g, int dist, int dtype, const void* av, const void* bv, double sa, double sb,
                  void* out, size_t n) {
  const int dbl = dtype == 1, P = P_of(dbl);
  if (n % (size_t)P) return 2;
  if (e->L != 4) return 3;
  const float* af = (const float*)av;
  const float* bf = (const float*)bv;
  const double* ad = (const double*)av;
  const double* bd = (const double*)bv;
  for (size_t k = 0; k < n / (size_t)P; ++k) {
    upk p, p2;
    switch (dist) {
      case OR_UNIFORM:
      case OR_EXPONENTIAL:
      case OR_WEIBULL:
      case OR_CAUCHY:
        ur_pk(e, dbl, &p);
        break;
      case OR_BALANCED:
        z2o_pk(e, dbl, &p);
        break;
      case OR_NORMAL:
      case OR_LOGNORMAL:
        stdnormal_pk(e, g, dbl, &p);
        break;
      case OR_EXTREME:
        nzur_pk(e, dbl, &p);
        break;
      case OR_STUDENT_T:
        ur_pk(e, dbl, &p);
        ur_pk(e, dbl, &p2);
        break;
      default:
        return 1;
    }
    for (int j = 0; j < P; ++j) {
      const size_t i = k * (size_t)P + (size_t)j;
      if (dbl) {
        const double a = av ? ad[i] : sa, b = bv ? bd[i] : sb, u = p.d[j];
        double v;
        switch (dist) {
          case OR_UNIFORM:
          case OR_BALANCED: v = u * (b - a) + a; break;
          case OR_NORMAL: v = u * b + a; break;
          case OR_LOGNORMAL: v = or_exp(u * b + a); break;
          case OR_EXPONENTIAL: v = -(or_log(1.0 - u) / a); break;
          case OR_WEIBULL: v = or_exp(or_log(-or_log(1.0 - u)) * (1.0 / a)) * b; break;
          case OR_EXTREME: v = a - or_log(-or_log(u)) * b; break;
          case OR_CAUCHY: {
            double sn, cs;
            or_sincos(PI_D * (u - 0.5), &sn, &cs);
            v = a + b * (sn / cs);
            break;
          }
          default: { /* OR_STUDENT_T, n = a */
            const double r = sqrt(a * (or_exp(or_log(1.0 - u) * (-2.0 / a)) - 1));
            double sn, cs;
            or_sincos((2 * PI_D) * p2.d[j], &sn, &cs);
            v = r * sn;
            break;
          }
        }
        ((double*)out)[i] = v;
      } else {
        const float a = av ? af[i] : (float)sa, b = bv ? bf[i] : (float)sb, u = p.f[j];
        float v;
        switch (dist) {
          case OR_UNIFORM:
          case OR_BALANCED: v = u * (b - a) + a; break;
          case OR_NORMAL: v = u * b + a; break;
          case OR_LOGNORMAL: v = or_expf(u * b + a); break;
          case OR_EXPONENTIAL: v = -(or_logf(1.0f - u) / a); break;
          case OR_WEIBULL: v = or_expf(or_logf(-or_logf(1.0f - u)) * (1.0f / a)) * b; break;
          case OR_EXTREME: v = a - or_logf(-or_logf(u)) * b; break;
          case OR_CAUCHY: {
            float sn, cs;
            or_sincosf((float)PI_D * (u - 0.5f), &sn, &cs);
            v = a + b * (sn / cs);
            break;
          }
          default: {
            const float r = sqrtf(a * (or_expf(or_logf(1.0f - u) * (-2.0f / a)) - 1));
            float sn, cs;
            or_sincosf((float)(2 * PI_D) * p2.f[j], &sn, &cs);
            v = r * sn;
            break;
          }
        }
        ((float*)out)[i] = v;
      }
    }
  }
  return 0;
}

/* ======================================================================
 * Truncated family, Truncated.h.  A base with a closed-form CDF becomes
 * UniformRealGen(phi(lower), phi(upper)) pushed through its inverse CDF; the
 * constants are the constructors' own, in the scalar type, with the C
 * library's erfc / exp / atan / pow / log as std:: calls them.  Every other
 * base goes through TruncGen's CompressMask rejection over the base's own
 * packets (:247-262), its carried lanes in g[3].
 * ====================================================================== */
enum { TR_UNIFORM, TR_NORMAL, TR_LOGNORMAL, TR_EXPONENTIAL, TR_CAUCHY, TR_EXTREME, TR_WEIBULL, TR_REJECT };

typedef struct {
  int form;
  double bias, slope; /* UniformRealGen(phi_lower, phi_upper) */
  double c0, c1;      /* the inverse CDF's constants */
} or_trunc;

/* The constructors of Truncated.h:293-305 (TruncNormalGen), :448-458
 * (exponential), :507-515 (Cauchy), :565-575 (lognormal), :621-630 (extreme
 * value), :679-690 (Weibull), :741-751, :840-845, :888-893, :936-941
 * (uniform family), in float.  Returns 0, or 4 for an empty support. */
static int trunc_setup_f(int dist, float a, float b, float lo, float hi, or_trunc* t) {
  float bias = 0, top = 0, c0 = 0, c1 = 0;
  if (!(lo < hi)) return 4;
  switch (dist) {
    case OR_UNIFORM:
    case OR_BALANCED: {
      const float ob = a, os = b - a; /* the base's bias and slope */
      const float mn = lo > ob ? lo : ob, mx = hi < ob + os ? hi : ob + os;
      if (!(mn < mx)) return 4;
      t->form = TR_UNIFORM;
      bias = mn;
      top = mx;
      break;
    }
    case OR_STDNORMAL:
    case OR_NORMAL:
    case OR_LOGNORMAL: {
      const float mean = dist == OR_STDNORMAL ? 0.0f : a, sd = dist == OR_STDNORMAL ? 1.0f : b;
      if (!(sd > 0)) return 4;
      if (dist == OR_LOGNORMAL) {
        lo = lo <= 0 ? -3.40282347e+38f : logf(lo);
        hi = logf(hi);
        if (!(lo < hi)) return 4;
      }
      const float an = (lo - mean) / sd, bn = (hi - mean) / sd, k = (float)(1.0 / 1.4142135623730951);
      bias = 0.5f * erfcf(-an * k);
      top = 0.5f * erfcf(-bn * k);
      c0 = sd;
      c1 = mean;
      t->form = dist == OR_LOGNORMAL ? TR_LOGNORMAL : TR_NORMAL;
      break;
    }
    case OR_EXPONENTIAL: {
      const float el = lo < 0 ? 0.0f : lo;
      bias = 1.0f - expf(-a * el);
      top = 1.0f - expf(-a * hi);
      c0 = 1.0f / a;
      t->form = TR_EXPONENTIAL;
      break;
    }
    case OR_CAUCHY:
      bias = 0.5f + atanf((lo - a) / b) / (float)PI_D;
      top = 0.5f + atanf((hi - a) / b) / (float)PI_D;
      c0 = a;
      c1 = b;
      t->form = TR_CAUCHY;
      break;
    case OR_EXTREME:
      bias = expf(-expf(-(lo - a) / b));
      top = expf(-expf(-(hi - a) / b));
      c0 = a;
      c1 = b;
      t->form = TR_EXTREME;
      break;
    case OR_WEIBULL: {
      const float el = lo < 0 ? 0.0f : lo;
      bias = 1.0f - expf(-powf(el / b, a));
      top = 1.0f - expf(-powf(hi / b, a));
      c0 = 1.0f / a;
      c1 = b;
      t->form = TR_WEIBULL;
      break;
    }
    default:
      t->form = TR_REJECT;
      break;
  }
  t->bias = bias;
  t->slope = (float)(top - bias);
  t->c0 = c0;
  t->c1 = c1;
  return 0;
}

/* The same constructors in double. */
static int trunc_setup_d(int dist, double a, double b, double lo, double hi, or_trunc* t) {
  double bias = 0, top = 0, c0 = 0, c1 = 0;
  if (!(lo < hi)) return 4;
  switch (dist) {
    case OR_UNIFORM:
    case OR_BALANCED: {
      const double ob = a, os = b - a;
      const double mn = lo > ob ? lo : ob, mx = hi < ob + os ? hi : ob + os;
      if (!(mn < mx)) return 4;
      t->form = TR_UNIFORM;
      bias = mn;
      top = mx;
      break;
    }
    case OR_STDNORMAL:
    case OR_NORMAL:
    case OR_LOGNORMAL: {
      const double mean = dist == OR_STDNORMAL ? 0.0 : a, sd = dist == OR_STDNORMAL ? 1.0 : b;
      if (!(sd > 0)) return 4;
      if (dist == OR_LOGNORMAL) {
        lo = lo <= 0 ? -1.7976931348623157e+308 : log(lo);
        hi = log(hi);
        if (!(lo < hi)) return 4;
      }
      const double an = (lo - mean) / sd, bn = (hi - mean) / sd, k = 1.0 / 1.4142135623730951;
      bias = 0.5 * erfc(-an * k);
      top = 0.5 * erfc(-bn * k);
      c0 = sd;
      c1 = mean;
      t->form = dist == OR_LOGNORMAL ? TR_LOGNORMAL : TR_NORMAL;
      break;
    }
    case OR_EXPONENTIAL: {
      const double el = lo < 0 ? 0.0 : lo;
      bias = 1.0 - exp(-a * el);
      top = 1.0 - exp(-a * hi);
      c0 = 1.0 / a;
      t->form = TR_EXPONENTIAL;
      break;
    }
    case OR_CAUCHY:
      bias = 0.5 + atan((lo - a) / b) / PI_D;
      top = 0.5 + atan((hi - a) / b) / PI_D;
      c0 = a;
      c1 = b;
      t->form = TR_CAUCHY;
      break;
    case OR_EXTREME:
      bias = exp(-exp(-(lo - a) / b));
      top = exp(-exp(-(hi - a) / b));
      c0 = a;
      c1 = b;
      t->form = TR_EXTREME;
      break;
    case OR_WEIBULL: {
      const double el = lo < 0 ? 0.0 : lo;
      bias = 1.0 - exp(-pow(el / b, a));
      top = 1.0 - exp(-pow(hi / b, a));
      c0 = 1.0 / a;
      c1 = b;
      t->form = TR_WEIBULL;
      break;
    }
    default:
      t->form = TR_REJECT;
      break;
  }
  t->bias = bias;
  t->slope = top - bias;
  t->c0 = c0;
  t->c1 = c1;
  return 0;
}

/* One lane of an inverse-CDF form, u = UniformRealGen's value. */
static float trunc_lane_f(const or_trunc* t, float u) {
  const float c0 = (float)t->c0, c1 = (float)t->c1;
  switch (t->form) {
    case TR_NORMAL:
    case TR_LOGNORMAL: { /* TruncNormalGen::packetOp, Truncated.h:322-331 */
      const float z = (float)-1.4142135623730951 * or_erfinvf(1.0f - 2.0f * u);
      const float x = z * c0 + c1;
      return t->form == TR_LOGNORMAL ? or_expf(x) : x; /* :593-598 */
    }
    case TR_EXPONENTIAL: /* :477-484 */
      return -or_logf(1.0f - u) * c0;
    case TR_CAUCHY: { /* :534-543 */
      float s, c;
      or_sincosf((float)PI_D * (u - 0.5f), &s, &c);
      return c0 + c1 * (s / c);
    }
    case TR_EXTREME: /* :649-656 */
      return c0 - c1 * or_logf(-or_logf(u));
    case TR_WEIBULL: /* :709-718 */
      return c1 * or_expf(or_logf(-or_logf(1.0f - u)) * c0);
    default:
      return u;
  }
}

static double trunc_lane_d(const or_trunc* t, double u) {
  switch (t->form) {
    case TR_NORMAL:
    case TR_LOGNORMAL: {
      const double z = -1.4142135623730951 * or_erfinv(1.0 - 2.0 * u);
      const double x = z * t->c0 + t->c1;
      return t->form == TR_LOGNORMAL ? or_exp(x) : x;
    }
    case TR_EXPONENTIAL:
      return -or_log(1.0 - u) * t->c0;
    case TR_CAUCHY: {
      double s, c;
      or_sincos(PI_D * (u - 0.5), &s, &c);
      return t->c0 + t->c1 * (s / c);
    }
    case TR_EXTREME:
      return t->c0 - t->c1 * or_log(-or_log(u));
    case TR_WEIBULL:
      return t->c1 * or_exp(or_log(-or_log(1.0 - u)) * t->c0);
    default:
      return u;
  }
}

/* TruncGen<Base>{base, Support(lower, upper)}.generate: n samples.  `dist`,
 * `a`, `b` describe the base as in or_gen_real (OR_UNIFORM / OR_BALANCED with
 * the base's min and max).  g needs four slots: the base's caches in g[0..2]
 * and TruncGen's carried lanes in g[3].  Returns 0, or 4 for an empty
 * support / bad base parameter. */
int or_gen_trunc(or_vmt* e, or_gen* g, int dist, int dtype, double a, double b, double lower, double upper,
                 void* out, size_t n) {
  const int dbl = dtype == 1, P = P_of(dbl);
  if (n % (size_t)P) return 2;
  if (e->L != 4) return 3;
  or_trunc t;
  const int rc = dbl ? trunc_setup_d(dist, a, b, lower, upper, &t)
                     : trunc_setup_f(dist, (float)a, (float)b, (float)lower, (float)upper, &t);
  if (rc) return rc;
  float* of = (float*)out;
  double* od = (double*)out;
  or_gen* tg = g + 3;
  for (size_t k = 0; k < n / (size_t)P; ++k) {
    if (t.form == TR_REJECT) {
      /* TruncGen::packetOp, Truncated.h:247-262 */
      for (int it = 0;; ++it) {
        if (it > (1 << 24)) return 5;
        upk c;
        int mask[8], full = 0;
        const int r = or_gen_real(e, g, dist, dtype, a, b, dbl ? (void*)c.d : (void*)c.f, (size_t)P);
        if (r) return r;
        for (int j = 0; j < P; ++j) {
          if (dbl) mask[j] = lower <= c.d[j] && c.d[j] <= upper;
          else mask[j] = (float)lower <= c.f[j] && c.f[j] <= (float)upper;
        }
        tg->rest_cnt = compress_append(P, dbl, dbl ? (void*)c.d : (void*)c.f, mask, tg->rest, tg->rest_cnt, &full);
        if (full) {
          if (dbl) memcpy(od + k * 4, c.d, 32);
          else memcpy(of + k * 8, c.f, 32);
          break;
        }
      }
      continue;
    }
    /* UniformRealGen::packetOp (Basic.h:627-635), then the form's map */
    upk u;
    ur_pk(e, dbl, &u);
    if (dbl) {
      for (int j = 0; j < 4; ++j) od[k * 4 + j] = trunc_lane_d(&t, u.d[j] * t.slope + t.bias);
    } else {
      const float sl = (float)t.slope, bi = (float)t.bias;
      for (int j = 0; j < 8; ++j) of[k * 8 + j] = trunc_lane_f(&t, u.f[j] * sl + bi);
    }
  }
  return 0;
}

/* ======================================================================
 * Integer generators.  int32 packets are Packet4i; their float internals are
 * Packet4f drawn through rng.half() (arch/AVX/RandUtils.h:28-31).
 * ====================================================================== */

/* PoissonGen::packetOp, Discrete.h:854-903 */
static void poisson_pk(or_vmt* e, or_gen* g, double mean, int32_t* res) {
  if (mean < 12) {
    float pne = (float)exp(-mean);
    float val[4] = {1, 1, 1, 1};
    for (int j = 0; j < 4; ++j) res[j] = 0;
    for (;;) {
      float u[4];
      ur_f4(e, u);
      int any = 0;
      int c[4];
      for (int j = 0; j < 4; ++j) {
        val[j] = val[j] * u[j];
        c[j] = pne < val[j];
        any |= c[j];
      }
      if (!any) break;
      for (int j = 0; j < 4; ++j) res[j] += c[j];
    }
    return;
  }
  float ppi = (float)PI_D, psqrt_tmean = (float)sqrt(2 * mean), pmean = (float)mean;
  float plog_mean = (float)log(mean);
  float pg1 = (float)(mean * log(mean) - lgamma(mean + 1));
  for (;;) {
    float u[4], u2[4];
    ur_f4(e, u);
    float fres[4], p1[4];
    for (int j = 0; j < 4; ++j) {
      float s, c;
      or_sincosf(ppi * u[j], &s, &c);
      float yx = s / c;
      fres[j] = truncf(psqrt_tmean * yx + pmean);
      p1[j] = (yx * yx + 1.0f) * 0.9f;
    }
    ur_f4(e, u2);
    uint32_t cands[4];
    int mask[4];
    for (int j = 0; j < 4; ++j) {
      float p2 = or_expf((fres[j] * plog_mean - or_lgamma_approxf(fres[j] + 1.0f)) - pg1);
      mask[j] = (0.0f <= fres[j]) && (u2[j] <= p1[j] * p2);
      cands[j] = f2u(fres[j]);
    }
    int full = 0;
    g->rest_cnt = compress_append(4, 0, cands, mask, g->rest, g->rest_cnt, &full);
    if (full) {
      for (int j = 0; j < 4; ++j) res[j] = (int32_t)u2f(cands[j]);
      return;
    }
  }
}

int or_gen_poisson(or_vmt* e, or_gen* g, double mean, int32_t* out, size_t n) {
  if (n % 4 || e->L != 4) return 2;
  for (size_t k = 0; k < n / 4; ++k) poisson_pk(e, g, mean, out + 4 * k);
  return 0;
}

/* BinomialGen::packetOp, Discrete.h:990-1052 */
int or_gen_binomial(or_vmt* e, or_gen* g, int32_t trials, double p, int32_t* out, size_t n) {
  if (n % 4 || e->L != 4) return 2;
  double small_p = p < 1 - p ? p : 1 - p;
  double pmean_d = trials * small_p;
  double g1 = 0, sqrt_v = 0, lsp = 0, lsq = 0;
  if (!(trials < 25 || pmean_d < 1.0)) {
    g1 = lgamma(trials + 1);
    sqrt_v = sqrt(2 * pmean_d * (1 - small_p));
    lsp = log(small_p);
    lsq = log(1 - small_p);
  }
  for (size_t k = 0; k < n / 4; ++k) {
    int32_t res[4];
    if (trials < 25) {
      float pp = (float)p;
      for (int j = 0; j < 4; ++j) res[j] = trials;
      for (int i = 0; i < trials; ++i) {
        float u[4];
        ur_f4(e, u);
        for (int j = 0; j < 4; ++j) res[j] += (pp <= u[j]) ? -1 : 0;
      }
      memcpy(out + 4 * k, res, sizeof res);
      continue;
    } else if (pmean_d < 1.0) {
      poisson_pk(e, g, pmean_d, res);
    } else {
      float ppi = (float)PI_D, ptrials = (float)trials, psqrt_v = (float)sqrt_v, pmean = (float)pmean_d;
      float plsp = (float)lsp, plsq = (float)lsq, pg1 = (float)g1;
      for (;;) {
        float u[4], u2[4], fres[4], p1[4];
        ur_f4(e, u);
        for (int j = 0; j < 4; ++j) {
          float s, c;
          or_sincosf(ppi * u[j], &s, &c);
          float ys = s / c;
          fres[j] = truncf(psqrt_v * ys + pmean);
          p1[j] = ((float)1.2 * psqrt_v) * (1.0f + ys * ys);
        }
        ur_f4(e, u2);
        uint32_t cands[4];
        int mask[4];
        for (int j = 0; j < 4; ++j) {
          float t = (pg1 - or_lgamma_approxf(fres[j] + 1.0f)) - or_lgamma_approxf((ptrials + 1.0f) - fres[j]);
          t = t + fres[j] * plsp;
          t = t + (ptrials - fres[j]) * plsq;
          float p2 = or_expf(t);
          mask[j] = (0.0f <= fres[j]) && (fres[j] <= ptrials) && (u2[j] <= p1[j] * p2);
          cands[j] = f2u(fres[j]);
        }
        int full = 0;
        g->rest_cnt = compress_append(4, 0, cands, mask, g->rest, g->rest_cnt, &full);
        if (full) {
          for (int j = 0; j < 4; ++j) res[j] = (int32_t)u2f(cands[j]);
          break;
        }
      }
    }
    for (int j = 0; j < 4; ++j) out[4 * k + j] = (p == small_p) ? res[j] : trials - res[j];
  }
  return 0;
}

/* RandbitsGen::packetOp<Packet4i>: RawbitsMaker<Packet4i,..>::rawbits =
 * rng.half(), Basic.h:393-399, arch/AVX/RandUtils.h:23-26 */
int or_gen_randbits(or_vmt* e, int32_t* out, size_t n) {
  if (e->L != 4) return 2;
  for (size_t k = 0; k < n / 4; ++k) {
    uint32_t w[4];
    draw_half(e, w);
    memcpy(out + 4 * k, w, 16);
  }
  if (n % 4) scalar_tail(e, -1, 2, 0, 0, out + n / 4 * 4, n % 4);
  return 0;
}

/* BernoulliGen<int32_t>::packetOp<Packet4i>, Basic.h:695-707: rawbits of a
 * Packet4i = rng.half() (arch/AVX/RandUtils.h:23-26), (w & 0x7FFFFFFF)
 * compared signed with (int32)(uint32)(p * 2^31) (so p = 1 gives 0) */
int or_gen_bernoulli_i32(or_vmt* e, double p, int32_t* out, size_t n) {
  if (e->L != 4) return 2;
  const int32_t pt = (int32_t)(uint32_t)(p * 2147483648.0);
  for (size_t k = 0; k < n / 4; ++k) {
    uint32_t w[4];
    draw_half(e, w);
    for (int j = 0; j < 4; ++j) out[4 * k + j] = ((int32_t)(w[j] & 0x7fffffffu) < pt) ? 1 : 0;
  }
  if (n % 4) scalar_tail(e, OR_BERNOULLI, 2, p, 0, out + n / 4 * 4, n % 4);
  return 0;
}

/* _mm_cvttps_epi32 of one lane: truncation; NaN and out-of-range give
 * 0x80000000 */
static int32_t cvtt_f32(float x) {
  return (x >= -2147483648.0f && x < 2147483648.0f) ? (int32_t)x : INT32_MIN;
}

/* BernoulliVGen<float>::packetOp, Basic.h:735-745: one Packet8i rawbits
 * packet (rng()), p = pcast<Packet8f, Packet8i>(a * 2^31) (cvttps2dq),
 * compared signed with the masked words */
int or_gen_bernoulli_v_f32(or_vmt* e, const float* pv, float* out, size_t n) {
  if (n % 8 || e->L != 4) return 2;
  for (size_t k = 0; k < n / 8; ++k) {
    uint32_t w[8];
    draw_full(e, w);
    for (int j = 0; j < 8; ++j)
      out[8 * k + j] = ((int32_t)(w[j] & 0x7fffffffu) < cvtt_f32(pv[8 * k + j] * 2147483648.0f)) ? 1.0f : 0.0f;
  }
  return 0;
}

/* GeometricGen<int32_t>::packetOp<Packet4i>, Discrete.h:1355-1375:
 * rlog_q = 1 / log(1 - p) in double, set as a float packet; u from
 * StdUniformRealGen<float> over Packet4f (rng.half() words);
 * pcast(ptruncate(plog(1 - u) * rlog_q)) */
int or_gen_geometric(or_vmt* e, double p, int32_t* out, size_t n) {
  if (n % 4 || e->L != 4) return 2;
  const float rlq = (float)(1 / log(1 - p));
  for (size_t k = 0; k < n / 4; ++k) {
    float u[4];
    ur_f4(e, u);
    for (int j = 0; j < 4; ++j) out[4 * k + j] = cvtt_f32(truncf(or_logf(1.0f - u[j]) * rlq));
  }
  return 0;
}

/* UniformIntGen<int32_t>(min, max), Discrete.h:230-245 (constructor, size_t
 * arithmetic) and :287-331 (packetOp<Packet4i>): rx = randbits = rng.half();
 * a power-of-two range masks; otherwise bit slices of rx go through
 * compress_append until a packet is full, rx shifting by bitsize while
 * bitcnt + bitsize < 32 and redrawn after that. */
int or_gen_uniform_int(or_vmt* e, or_gen* g, int32_t mn, int32_t mx, int32_t* out, size_t n) {
  if (n % 4 || e->L != 4) return 2;
  const uint64_t pdiff = (uint64_t)(int64_t)(int32_t)((uint32_t)mx - (uint32_t)mn);
  uint64_t bitsize = 0, bitmask;
  if (pdiff == 0) bitsize = 0;
  else if (pdiff + 1 > pdiff) bitsize = (uint64_t)ceil(log2((double)(pdiff + 1)));
  else bitsize = (uint64_t)ceil(log2((double)pdiff));
  bitmask = bitsize == 0 ? ~0ull : (uint64_t)(int64_t)(int32_t)(uint32_t)(~0ull >> (64 - bitsize));
  const uint32_t pmask = (uint32_t)bitmask;
  const int32_t plen = (int32_t)(uint32_t)(pdiff + 1);
  for (size_t k = 0; k < n / 4; ++k) {
    if (pdiff == 0) {
      for (int j = 0; j < 4; ++j) out[4 * k + j] = mn;
      continue;
    }
    uint32_t rx[4];
    draw_half(e, rx);
    if (pdiff == bitmask) {
      for (int j = 0; j < 4; ++j) out[4 * k + j] = (int32_t)((rx[j] & pmask) + (uint32_t)mn);
      continue;
    }
    uint64_t bitcnt = bitsize;
    for (;;) {
      uint32_t cands[4];
      int mask[4], full = 0;
      for (int j = 0; j < 4; ++j) {
        cands[j] = rx[j] & pmask;
        mask[j] = (int32_t)cands[j] < plen;
      }
      g->rest_cnt = compress_append(4, 0, cands, mask, g->rest, g->rest_cnt, &full);
      if (full) {
        for (int j = 0; j < 4; ++j) out[4 * k + j] = (int32_t)(cands[j] + (uint32_t)mn);
        break;
      }
      if (bitcnt + bitsize < 32) {
        for (int j = 0; j < 4; ++j) rx[j] >>= bitsize;
        bitcnt += bitsize;
      } else {
        draw_half(e, rx);
        bitcnt = bitsize;
      }
    }
  }
  return 0;
}

/* NegativeBinomialGen<int32_t>(trials, p), GammaPoisson.h:42-98: a Packet4f
 * GammaGen<float>((float)trials, (float)((1 - p) / p)) draw (NormalExp.h:
 * 568-604 over rng.half() words), then a Poisson draw with those per-lane
 * means: the multiplicative loop when no lane's mean exceeds 12, else tan
 * rejection whose CompressMask carry is the GammaGen's own. */
int or_gen_negative_binomial(or_vmt* e, or_gen* g, int32_t trials, double p, int32_t* out, size_t n) {
  if (n % 4 || e->L != 4) return 2;
  const float alpha = (float)trials, beta = (float)((1 - p) / p);
  const float gsq = sqrtf(2 * alpha - 1);
  const int count0 = (int)alpha;
  const float eps8 = 1.1920928955078125e-07f / 8;
  for (size_t k = 0; k < n / 4; ++k) {
    float mean[4];
    if (alpha == 1) { /* beta * ExponentialGen(1) */
      float u[4];
      ur_f4(e, u);
      for (int j = 0; j < 4; ++j) mean[j] = beta * (-(or_logf(1.0f - u[j]) / 1.0f));
    } else if ((float)count0 == alpha && count0 < 20) { /* product of count uniforms */
      float y[4], u[4];
      ur_f4(e, u);
      for (int j = 0; j < 4; ++j) y[j] = u[j] + eps8;
      for (int c = 1; c < count0; ++c) {
        ur_f4(e, u);
        for (int j = 0; j < 4; ++j) y[j] = y[j] * (u[j] + eps8);
      }
      for (int j = 0; j < 4; ++j) mean[j] = -(beta * or_logf(y[j]));
    } else { /* tan rejection, NormalExp.h:589-603 */
      const float a1 = alpha - 1;
      for (;;) {
        float u[4], ux[4];
        ur_f4(e, u);
        float xx[4], ys[4], yc[4];
        int mask[4];
        for (int j = 0; j < 4; ++j) or_sincosf((float)PI_D * u[j], &ys[j], &yc[j]);
        ur_f4(e, ux);
        float cands[4];
        for (int j = 0; j < 4; ++j) {
          const float yx = ys[j] / yc[j];
          xx[j] = gsq * yx + a1;
          const float ub = (yx * yx + 1.0f) * or_expf(a1 * or_logf(xx[j] / a1) - yx * gsq);
          mask[j] = (0.0f < xx[j]) && (ux[j] <= ub);
          cands[j] = beta * xx[j];
        }
        int full = 0;
        g->rest_cnt = compress_append(4, 0, cands, mask, g->rest, g->rest_cnt, &full);
        if (full) {
          memcpy(mean, cands, sizeof mean);
          break;
        }
      }
    }
    float pne[4];
    int big = 0;
    for (int j = 0; j < 4; ++j) {
      pne[j] = or_expf(-mean[j]);
      big |= 12.0f < mean[j];
    }
    if (!big) {
      float val[4] = {1, 1, 1, 1};
      int32_t res[4] = {0, 0, 0, 0};
      for (;;) {
        float u[4];
        ur_f4(e, u);
        int any = 0, c[4];
        for (int j = 0; j < 4; ++j) {
          val[j] = val[j] * u[j];
          c[j] = pne[j] < val[j];
          any |= c[j];
        }
        if (!any) break;
        for (int j = 0; j < 4; ++j) res[j] += c[j];
      }
      memcpy(out + 4 * k, res, sizeof res);
      continue;
    }
    float st[4], lm[4], g1[4];
    for (int j = 0; j < 4; ++j) {
      st[j] = sqrtf(2.0f * mean[j]);
      lm[j] = or_logf(mean[j]);
      g1[j] = mean[j] * lm[j] - or_lgamma_approxf(mean[j] + 1.0f);
    }
    for (;;) {
      float u[4], u2[4], fres[4], p1[4];
      ur_f4(e, u);
      for (int j = 0; j < 4; ++j) {
        float s, c;
        or_sincosf((float)PI_D * u[j], &s, &c);
        const float yx = s / c;
        fres[j] = truncf(st[j] * yx + mean[j]);
        p1[j] = (yx * yx + 1.0f) * 0.9f;
      }
      ur_f4(e, u2);
      int mask[4];
      for (int j = 0; j < 4; ++j) {
        const float p2 = or_expf((fres[j] * lm[j] - or_lgamma_approxf(fres[j] + 1.0f)) - g1[j]);
        mask[j] = (0.0f <= fres[j]) && (u2[j] <= p1[j] * p2);
      }
      int full = 0;
      g->rest_cnt = compress_append(4, 0, fres, mask, g->rest, g->rest_cnt, &full);
      if (full) {
        for (int j = 0; j < 4; ++j) out[4 * k + j] = cvtt_f32(fres[j]);
        break;
      }
    }
  }
  return 0;
}

/* ======================================================================
 * DiscreteGen<int32_t, int32_t>: CDF (<16 weights) or AliasMethod (>=16),
 * Discrete.h:23-207 (table build), :385-412 (constructor), :443-485 (AVX2
 * packetOp: 8 draws from one rng() packet, 4 returned and 4 cached).
 * ====================================================================== */
or_discrete* or_discrete_new(const double* w, int n) {
  if (n < 1) return NULL;
  or_discrete* d = (or_discrete*)calloc(1, sizeof(or_discrete));
  d->n = n;
  if (n < 16) {
    d->use_cdf = 1;
    double acc = 0, cdfd[64];
    for (int i = 0; i < n; ++i) cdfd[i] = (acc += w[i]);
    for (int i = 0; i < n; ++i) d->cdf[i] = (uint32_t)(cdfd[i] / cdfd[n - 1] * 0x80000000);
    return d;
  }
  double sum = 0;
  for (int i = 0; i < n; ++i) sum += w[i];
  if (!isfinite(sum)) { free(d); return NULL; }
  size_t nbsize = (size_t)ceil(log2((double)n));
  size_t psize = (size_t)1 << nbsize;
  d->bitsize = (int)nbsize;
  d->bitmask = (uint32_t)(((size_t)-1) >> (sizeof(size_t) * 8 - nbsize));
  d->prob = (int32_t*)calloc(psize, sizeof(int32_t));
  d->alias = (int32_t*)calloc(psize, sizeof(int32_t));
  sum /= (double)psize;
  double* f = (double*)calloc(psize, sizeof(double));
  for (int i = 0; i < n; ++i) f[i] = w[i] / sum;
  size_t over = 0, under = 0, mm;
  while (over < psize && f[over] < 1) ++over;
  while (under < psize && f[under] >= 1) ++under;
  mm = under + 1;
  while (over < psize && under < psize) {
    d->prob[under] = (int32_t)(f[under] * (2147483647 + 1.0));
    d->alias[under] = (int32_t)over;
    f[over] += f[under] - 1;
    if (f[over] >= 1 || mm <= over) {
      for (under = mm; under < psize && f[under] >= 1; ++under) {}
      mm = under + 1;
    } else {
      under = over;
    }
    while (over < psize && f[over] < 1) ++over;
  }
  for (; over < psize; ++over) {
    if (f[over] >= 1) {
      d->prob[over] = 2147483647;
      d->alias[over] = (int32_t)over;
    }
  }
  if (under < psize) {
    d->prob[under] = 2147483647;
    d->alias[under] = (int32_t)under;
    for (under = mm; under < (size_t)n; ++under) {
      if (f[under] < 1) {
        d->prob[under] = 2147483647;
        d->alias[under] = (int32_t)under;
      }
    }
  }
  free(f);
  return d;
}

void or_discrete_free(or_discrete* d) {
  if (!d) return;
  free(d->prob);
  free(d->alias);
  free(d);
}

int or_discrete_table(const or_discrete* d, int32_t* prob, int32_t* alias, int cap) {
  if (d->use_cdf) {
    for (int i = 0; i < d->n && i < cap; ++i) prob[i] = (int32_t)d->cdf[i];
    return -d->n;
  }
  int ps = 1 << d->bitsize;
  for (int i = 0; i < ps && i < cap; ++i) {
    prob[i] = d->prob[i];
    alias[i] = d->alias[i];
  }
  return ps;
}

int or_gen_discrete(or_vmt* e, or_gen* g, const or_discrete* d, int32_t* out, size_t n) {
  if (n % 4 || e->L != 4) return 2;
  for (size_t k = 0; k < n / 4; ++k) {
    if (g->valid) {
      g->valid = 0;
      memcpy(out + 4 * k, g->cache, 16);
      continue;
    }
    uint32_t rx[8];
    int32_t ret[8];
    draw_full(e, rx);
    if (d->use_cdf) {
      for (int j = 0; j < 8; ++j) {
        int32_t r = d->n - 1;
        int32_t x = (int32_t)(rx[j] & 0x7fffffffu);
        for (int i = 0; i < d->n - 1; ++i) r += (x < (int32_t)d->cdf[i]) ? -1 : 0;
        ret[j] = r;
      }
    } else {
      for (int j = 0; j < 8; ++j) {
        int32_t albit = (int32_t)(rx[j] & d->bitmask);
        int32_t sh = (int32_t)(rx[j] >> 1);
        ret[j] = (sh < d->prob[albit]) ? albit : d->alias[albit];
      }
    }
    g->valid = 1;
    memcpy(g->cache, ret + 4, 16);
    memcpy(out + 4 * k, ret, 16);
  }
  return 0;
}

/* ======================================================================
 * MultinomialGen<int32_t>::generate(urng, samples) on the per-trial path
 * (trials < max(30 (dim - 1), 100); Multinomial.h:62-71, 95-118).  Per
 * sample, the DiscreteGen member draws 16 categories at a time through its
 * packet operator (a Matrix<int32_t, 16, 1> assignment), then the trials % 16
 * tail: its whole packets of 4 first, then trials % 4 draws through the
 * scalar operator() (Discrete.h:420-441).  A scalar draw takes one full
 * rng() packet, uses its first 32-bit word and leaves the packet cache alone.
 * Counts go to out[s * dim + category].
 * ====================================================================== */
static int32_t discrete_scalar(or_vmt* e, const or_discrete* d) {
  uint32_t rx[8];
  draw_full(e, rx);
  const int32_t x = (int32_t)rx[0];
  if (d->use_cdf) { /* std::lower_bound over the uint32 cdf[0 .. n-2] */
    const uint32_t v = (uint32_t)(x & 0x7fffffff);
    int32_t r = 0;
    for (int i = 0; i < d->n - 1; ++i) r += (d->cdf[i] < v) ? 1 : 0;
    return r;
  }
  const int32_t albit = x & (int32_t)d->bitmask;
  const uint32_t alx = (uint32_t)(x >> 1); /* arithmetic shift of the signed draw */
  return alx < (uint32_t)d->prob[albit] ? albit : d->alias[albit];
}

int or_gen_multinomial(or_vmt* e, or_gen* g, const or_discrete* d, int32_t trials, int32_t dim, int32_t* out,
                       size_t samples) {
  if (e->L != 4 || trials < 0) return 2;
  int32_t buf[16];
  for (size_t s = 0; s < samples; ++s) {
    int32_t* h = out + s * (size_t)dim;
    memset(h, 0, sizeof(int32_t) * (size_t)dim);
    int32_t i = 0;
    for (; i + 16 <= trials; i += 16) {
      int rc = or_gen_discrete(e, g, d, buf, 16);
      if (rc) return rc;
      for (int j = 0; j < 16; ++j) h[buf[j]] += 1;
    }
    const int32_t r = trials - i, q = r / 4;
    if (q) {
      int rc = or_gen_discrete(e, g, d, buf, (size_t)(4 * q));
      if (rc) return rc;
      for (int j = 0; j < 4 * q; ++j) h[buf[j]] += 1;
    }
    for (int j = 4 * q; j < r; ++j) h[discrete_scalar(e, d)] += 1;
  }
  return 0;
}

/* ======================================================================
 * BinomialVGen<int32_t>::packetOp (Discrete.h:1124-1192), one packet of 4
 * lanes whose (trials, p) may differ per lane.  Lanes with mean < 1 run the
 * multiplicative Poisson loop; the others a tan-proposal rejection with a
 * per-lane accepted mask, iterating until every lane has a value.
 * ====================================================================== */
static void binomial_v_lanes(or_vmt* e, int P, const int32_t* trials, const float* p, int32_t* out) {
  float small_p[8], ptrials[8], mean[8], g1[8], sqrt_v[8], lsp[8], lsq[8], ne[8];
  int valid[8], any_valid = 0, all_valid = 1;
  float valid_res[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j < P; ++j) {
    small_p[j] = p[j] < 1.0f - p[j] ? p[j] : 1.0f - p[j]; /* pmin(p, 1 - p) */
    ptrials[j] = (float)trials[j];
    mean[j] = ptrials[j] * small_p[j];
    g1[j] = or_lgamma_approxf(ptrials[j] + 1.0f);
    sqrt_v[j] = sqrtf((2.0f * mean[j]) * (1.0f - small_p[j]));
    lsp[j] = or_logf(small_p[j]);
    lsq[j] = or_logf(1.0f - small_p[j]);
    ne[j] = or_expf(-mean[j]);
    valid[j] = mean[j] < 1.0f;
    any_valid |= valid[j];
    all_valid &= valid[j];
  }
  if (any_valid) {
    int32_t res[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float val[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    for (;;) {
      float u[8];
      if (P == 8) ur_f8(e, u); else ur_f4(e, u);
      int any = 0, c[8];
      for (int j = 0; j < P; ++j) {
        val[j] = val[j] * u[j];
        c[j] = (ne[j] < val[j]) && valid[j];
        any |= c[j];
      }
      if (!any) break;
      for (int j = 0; j < P; ++j) res[j] += c[j];
    }
    for (int j = 0; j < P; ++j) valid_res[j] = (float)res[j];
  }
  if (!all_valid) {
    for (;;) {
      float u[8], u2[8], fres[8], ys[8];
      if (P == 8) ur_f8(e, u); else ur_f4(e, u);
      for (int j = 0; j < P; ++j) {
        float s, c;
        or_sincosf((float)PI_D * u[j], &s, &c);
        ys[j] = s / c;
        fres[j] = truncf(sqrt_v[j] * ys[j] + mean[j]);
      }
      if (P == 8) ur_f8(e, u2); else ur_f4(e, u2);
      int all = 1;
      for (int j = 0; j < P; ++j) {
        float p1 = ((float)1.2 * sqrt_v[j]) * (1.0f + ys[j] * ys[j]);
        float t = (g1[j] - or_lgamma_approxf(fres[j] + 1.0f)) - or_lgamma_approxf((ptrials[j] + 1.0f) - fres[j]);
        t = t + fres[j] * lsp[j];
        t = t + (ptrials[j] - fres[j]) * lsq[j];
        float p2 = or_expf(t);
        int fvalid = (0.0f <= fres[j]) && (fres[j] <= ptrials[j]) && (u2[j] <= p1 * p2);
        if (fvalid && !valid[j]) valid_res[j] = fres[j];
        valid[j] |= fvalid;
        all &= valid[j];
      }
      if (all) break;
    }
  }
  for (int j = 0; j < P; ++j) out[j] = (p[j] == small_p[j]) ? (int32_t)valid_res[j] : trials[j] - (int32_t)valid_res[j];
}

int or_binomial_v_packet(or_vmt* e, const int32_t* trials, const float* p, int32_t* out) {
  binomial_v_lanes(e, 4, trials, p, out);
  return 0;
}

/* binomial(urng, trials, p) (Discrete.h:1822-1898): BinomialVGen<int32_t>
 * over n outputs (a multiple of 4) in packets of 4; a NULL array takes the
 * scalar operand for every element. */
int or_gen_binomial_v(or_vmt* e, const int32_t* trials, const float* p, int32_t trials0, float p0, int32_t* out,
                      size_t n) {
  if (n % 4) return 1;
  for (size_t i = 0; i < n; i += 4) {
    int32_t tr[4];
    float pp[4];
    for (int j = 0; j < 4; ++j) {
      tr[j] = trials ? trials[i + j] : trials0;
      pp[j] = p ? p[i + j] : p0;
    }
    binomial_v_lanes(e, 4, tr, pp, out + i);
  }
  return 0;
}

/* Eigen 3.4's sum() of a dynamic double vector with AVX packets of 4 (the
 * LinearVectorizedTraversal redux of Redux.h): two packet accumulators over
 * pairs of packets, their sum, one more packet if the aligned part has an odd
 * count, the packet reduced as (a0 + a2) + (a1 + a3), then the tail in order;
 * below one packet, a plain left-to-right sum.  The vector's storage is
 * 32-byte aligned, so the aligned part starts at 0. */
double or_eigen_sum_avx(const double* v, int n) {
  const int ps = 4, as2 = (n / (2 * ps)) * (2 * ps), as = (n / ps) * ps;
  if (!as) {
    double r = v[0];
    for (int i = 1; i < n; ++i) r += v[i];
    return r;
  }
  double p0[4], p1[4];
  for (int j = 0; j < 4; ++j) p0[j] = v[j];
  if (as > ps) {
    for (int j = 0; j < 4; ++j) p1[j] = v[ps + j];
    for (int i = 2 * ps; i < as2; i += 2 * ps)
      for (int j = 0; j < 4; ++j) {
        p0[j] = p0[j] + v[i + j];
        p1[j] = p1[j] + v[i + ps + j];
      }
    for (int j = 0; j < 4; ++j) p0[j] = p0[j] + p1[j];
    if (as > as2)
      for (int j = 0; j < 4; ++j) p0[j] = p0[j] + v[as2 + j];
  }
  double r = (p0[0] + p0[2]) + (p0[1] + p0[3]);
  for (int i = as; i < n; ++i) r = r + v[i];
  return r;
}

/* MultinomialGen<int32_t>::generate(urng, samples) on its conditional-binomial
 * path, trials >= max(30 (dim - 1), 100) (Multinomial.h:62-87): probs =
 * weights / sum; row 0 is BinomialVGen<float> over every sample with p =
 * probs[0] and the remaining trials per lane, then rows 1 .. dim-2 with p =
 * probs[i] / rest_p (rest_p = 1 - probs[0] - ... in double, p converted to
 * float), each row one packet of 8 samples after another; the last row is
 * what remains.  out = dim x samples, column-major; samples % 8 == 0. */
int or_gen_multinomial_cond(or_vmt* e, const double* w, int32_t dim, int32_t trials, int32_t* out,
                            size_t samples) {
  if (e->L != 4 || dim < 1 || samples % 8) return 2;
  double* probs = (double*)malloc(sizeof(double) * (size_t)dim);
  int32_t* r = (int32_t*)malloc(sizeof(int32_t) * (samples ? samples : 1));
  const double sum = or_eigen_sum_avx(w, dim);
  for (int i = 0; i < dim; ++i) probs[i] = w[i] / sum;
  for (size_t q = 0; q < samples; ++q) r[q] = trials;
  double rest = 0;
  const int last = dim - 2 > 0 ? dim - 2 : 0;
  for (int i = 0; i <= last; ++i) {
    float pv = i == 0 ? (float)probs[0] : (float)(probs[i] / rest);
    float pp[8];
    for (int j = 0; j < 8; ++j) pp[j] = pv;
    for (size_t k = 0; k < samples / 8; ++k) {
      int32_t t[8];
      binomial_v_lanes(e, 8, r + 8 * k, pp, t);
      for (int j = 0; j < 8; ++j) {
        if (i < dim - 1) out[(8 * k + j) * (size_t)dim + i] = t[j];
        r[8 * k + j] -= t[j];
      }
    }
    rest = i == 0 ? 1 - probs[0] : rest - probs[i];
  }
  for (size_t q = 0; q < samples; ++q) out[q * (size_t)dim + dim - 1] = r[q];
  free(probs);
  free(r);
  return 0;
}

/* One vectorize-over-params set, as the batched API defines it: a fresh
 * Vmt19937_64(seed) and a fresh generator, count samples drawn with the
 * packet algorithm, the last packet truncated.  kind: 0 = GammaGen<float>
 * (a = alpha, b = beta), 1 = BinomialVGen<int32_t> with uniform (trials, p). */
int or_vop_set(uint64_t seed, int kind, double a, double b, int32_t trials, void* out, size_t count) {
  or_vmt* e = or_vmt_new(seed, 4);
  or_gen g[3];
  memset(g, 0, sizeof g);
  int rc = 0;
  if (kind == 0) {
    size_t n8 = (count + 7) / 8 * 8;
    float* tmp = (float*)malloc(sizeof(float) * (n8 ? n8 : 8));
    rc = n8 ? or_gen_real(e, g, OR_GAMMA, 0, a, b, tmp, n8) : 0;
    memcpy(out, tmp, sizeof(float) * count);
    free(tmp);
  } else {
    int32_t tr[4] = {trials, trials, trials, trials};
    float pp[4] = {(float)a, (float)a, (float)a, (float)a};
    int32_t* o = (int32_t*)out;
    for (size_t k = 0; k < count; k += 4) {
      int32_t r[4];
      or_binomial_v_packet(e, tr, pp, r);
      for (size_t j = 0; j < 4 && k + j < count; ++j) o[k + j] = r[j];
    }
  }
  or_vmt_free(e);
  return rc;
}

/* ======================================================================
 * TruncMvNormalGen::generate(urng, samples), TruncMvNormal.h:171-209, with
 * the precision matrix H given (column-major, FP64, rounded here to the
 * scalar type).  Draws are StdUniformRealGen's scalar draws: one packet each,
 * its first 32-bit word (float) or 64-bit lane (double) (Basic.h:533-540).
 * out = dim x samples, column-major.
 * ====================================================================== */
int or_gen_truncmvn(or_vmt* e, int dtype, int dim, const double* H, const double* mean, const double* lower,
                    const double* upper, int64_t burn_in, void* out, size_t samples) {
  if (e->L != 4 || dim < 1 || dim > 64) return 2;
  const int dbl = dtype == 1;
  const int64_t sweeps = burn_in == 0 ? 5 * (int64_t)dim : burn_in;
  const size_t n = (size_t)dim * samples;
  if (dbl) {
    double *x = (double*)out, *df = (double*)malloc(sizeof(double) * (n ? n : 1)), idg[64], csd[64];
    for (int i = 0; i < dim; ++i) {
      idg[i] = 1.0 / H[(size_t)i * dim + i];
      csd[i] = sqrt(idg[i]);
    }
    for (size_t q = 0; q < samples; ++q)
      for (int i = 0; i < dim; ++i) {
        const double m = mean[i], lo = lower[i], hi = upper[i];
        x[q * dim + i] = lo > (m < hi ? m : hi) ? lo : (m < hi ? m : hi);
        df[q * dim + i] = x[q * dim + i] - m;
      }
    for (int64_t sw = 0; sw < sweeps; ++sw)
      for (int i = 0; i < dim; ++i)
        for (size_t q = 0; q < samples; ++q) {
          double* xd = df + q * dim;
          double h = H[i] * xd[0];
          for (int j = 1; j < dim; ++j) h = h + H[(size_t)j * dim + i] * xd[j];
          const double cm = mean[i] - idg[i] * (h - H[(size_t)i * dim + i] * xd[i]);
          const double an = (lower[i] - cm) / csd[i], bn = (upper[i] - cm) / csd[i];
          const double pa = 0.5 * erfc(-an * (1.0 / 1.4142135623730951));
          const double pb = 0.5 * erfc(-bn * (1.0 / 1.4142135623730951));
          uint64_t r[4];
          vmt_packet(e, r);
          const double u = pa + (pb - pa) * bit_ur_d(r[0]);
          const double z = -1.4142135623730951 * or_erfinv(1.0 - 2.0 * u);
          const double nx = z * csd[i] + cm;
          xd[i] = nx - mean[i];
          x[q * dim + i] = nx;
        }
    free(df);
  } else {
    float *x = (float*)out, *df = (float*)malloc(sizeof(float) * (n ? n : 1)), Hf[64 * 64], mf[64], lf[64], hf[64],
          idg[64], csd[64];
    for (int i = 0; i < dim * dim; ++i) Hf[i] = (float)H[i];
    for (int i = 0; i < dim; ++i) {
      mf[i] = (float)mean[i];
      lf[i] = (float)lower[i];
      hf[i] = (float)upper[i];
      idg[i] = 1.0f / Hf[i * dim + i];
      csd[i] = sqrtf(idg[i]);
    }
    for (size_t q = 0; q < samples; ++q)
      for (int i = 0; i < dim; ++i) {
        const float c = mf[i] < hf[i] ? mf[i] : hf[i];
        x[q * dim + i] = lf[i] > c ? lf[i] : c;
        df[q * dim + i] = x[q * dim + i] - mf[i];
      }
    const float rs2 = (float)(1.0 / 1.4142135623730951);
    for (int64_t sw = 0; sw < sweeps; ++sw)
      for (int i = 0; i < dim; ++i)
        for (size_t q = 0; q < samples; ++q) {
          float* xd = df + q * dim;
          float h = Hf[i] * xd[0];
          for (int j = 1; j < dim; ++j) h = h + Hf[j * dim + i] * xd[j];
          const float cm = mf[i] - idg[i] * (h - Hf[i * dim + i] * xd[i]);
          const float an = (lf[i] - cm) / csd[i], bn = (hf[i] - cm) / csd[i];
          const float pa = 0.5f * erfcf(-an * rs2), pb = 0.5f * erfcf(-bn * rs2);
          uint64_t r[4];
          vmt_packet(e, r);
          const float u = pa + (pb - pa) * bit_ur_f((uint32_t)r[0]);
          const float z = (float)-1.4142135623730951 * or_erfinvf(1.0f - 2.0f * u);
          const float nx = z * csd[i] + cm;
          xd[i] = nx - mf[i];
          x[q * dim + i] = nx;
        }
    free(df);
  }
  return 0;
}

/* Any generator of or_gen_real drawn with a scalar engine as the Urng. */
int or_sgen_real(or_seng* s, or_gen* g, int dist, int dtype, double a, double b, void* out, size_t n) {
  or_vmt dummy;
  memset(&dummy, 0, sizeof dummy);
  dummy.L = 4;
  or_seng* prev = g_src;
  g_src = s;
  const int rc = or_gen_real(&dummy, g, dist, dtype, a, b, out, n);
  g_src = prev;
  return rc;
}

/* binomial(urng, trials, p) with a scalar engine as the Urng: BinomialVGen<
 * int32_t> whose uniform packets take two draws each (draw_half). */
int or_sgen_binomial_v(or_seng* s, const int32_t* trials, const float* p, int32_t trials0, float p0, int32_t* out,
                       size_t n) {
  or_vmt dummy;
  memset(&dummy, 0, sizeof dummy);
  dummy.L = 4;
  or_seng* prev = g_src;
  g_src = s;
  const int rc = or_gen_binomial_v(&dummy, trials, p, trials0, p0, out, n);
  g_src = prev;
  return rc;
}

/* PoissonGen (kind 0) / BinomialGen (kind 1) / UniformIntGen (kind 2, min a,
 * max trials) / BernoulliGen (kind 3) / GeometricGen (kind 4) /
 * NegativeBinomialGen (kind 5, trials, p = a) <int32_t> with
 * a scalar engine as the Urng, a fresh generator
 * (the free functions): every packet takes two draws (draw_half). */
int or_sgen_int(or_seng* s, int kind, int32_t trials, double a, int32_t* out, size_t n) {
  or_vmt dummy;
  memset(&dummy, 0, sizeof dummy);
  dummy.L = 4;
  or_gen g;
  memset(&g, 0, sizeof g);
  or_seng* prev = g_src;
  g_src = s;
  const int rc = kind == 0   ? or_gen_poisson(&dummy, &g, a, out, n)
                 : kind == 1 ? or_gen_binomial(&dummy, &g, trials, a, out, n)
                 : kind == 2 ? or_gen_uniform_int(&dummy, &g, (int32_t)a, trials, out, n)
                 : kind == 3 ? or_gen_bernoulli_i32(&dummy, a, out, n)
                 : kind == 4 ? or_gen_geometric(&dummy, a, out, n)
                             : or_gen_negative_binomial(&dummy, &g, trials, a, out, n);
  g_src = prev;
  return rc;
}

/* DiscreteGen<int32_t> with a scalar engine as the Urng, a fresh generator
 * (the free function discrete()): a Packet8i of four draws per two packets. */
int or_sgen_discrete(or_seng* s, const or_discrete* d, int32_t* out, size_t n) {
  or_vmt dummy;
  memset(&dummy, 0, sizeof dummy);
  dummy.L = 4;
  or_gen g;
  memset(&g, 0, sizeof g);
  or_seng* prev = g_src;
  g_src = s;
  const int rc = or_gen_discrete(&dummy, &g, d, out, n);
  g_src = prev;
  return rc;
}

int or_sgen_randbits(or_seng* s, int32_t* out, size_t n) {
  or_vmt dummy;
  memset(&dummy, 0, sizeof dummy);
  dummy.L = 4;
  or_seng* prev = g_src;
  g_src = s;
  const int rc = or_gen_randbits(&dummy, out, n);
  g_src = prev;
  return rc;
}
