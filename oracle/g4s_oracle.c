/*
 * g4s_oracle.c — CPU oracle for the GPU4SNN simulation step.  TEST INFRASTRUCTURE ONLY:
 * tests, the smoke check and bench.py's CPU-baseline leg load it as the checker; the
 * product never calls it.  See g4s_oracle.h for the reference lines each part restates.
 *
 * Build with -ffp-contract=off and without -ffast-math: every float operation below is
 * one IEEE-754 binary32 operation with round-to-nearest-even, written in the same order
 * as the CUDA kernels, so that the FP32 mode is bit-exact with the GPU.
 */
#include "g4s_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------------------
 * Philox4x64-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as
 * 1, 2, 3", SC'11).  Round: (hi0,lo0)=M0*c0, (hi1,lo1)=M1*c2,
 * c' = (hi1^c1^k0, lo1, hi0^c3^k1, lo0); the key is bumped by the Weyl constants
 * between rounds.  Pinned against numpy.random.Philox.
 * ------------------------------------------------------------------------------- */
#define PHILOX_M0 0xD2E7470EE14C6C93ull
#define PHILOX_M1 0xCA5A826395121157ull
#define PHILOX_W0 0x9E3779B97F4A7C15ull
#define PHILOX_W1 0xBB67AE8584CAA73Bull

static inline void mulhilo64(uint64_t a, uint64_t b, uint64_t *hi, uint64_t *lo) {
  unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
  *hi = (uint64_t)(p >> 64);
  *lo = (uint64_t)p;
}

void g4o_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]) {
  uint64_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint64_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += PHILOX_W0;
      k1 += PHILOX_W1;
    }
    uint64_t hi0, lo0, hi1, lo1;
    mulhilo64(PHILOX_M0, c0, &hi0, &lo0);
    mulhilo64(PHILOX_M1, c2, &hi1, &lo1);
    uint64_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* Philox4x32-10 (same paper): (hi0,lo0) = M0*c0, (hi1,lo1) = M1*c2 in 32x32->64,
 * c' = (hi1^c1^k0, lo1, hi0^c3^k1, lo0), key bumped by the 32-bit Weyl constants.
 * Pinned against the Philox4x32-10 host generator of the CUDA toolkit's cuRAND. */
void g4o_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

static inline void philox(uint64_t seed, uint64_t stream, uint64_t c0, uint64_t c1, uint64_t c2,
                          uint64_t out[4]) {
  const uint64_t ctr[4] = {c0, c1, c2, 0};
  const uint64_t key[2] = {seed, stream};
  g4o_philox4x64_10(ctr, key, out);
}

/* 24-bit uniform in [0,1): top 24 bits of a 64-bit word, scaled exactly. */
static inline float u24(uint64_t x) { return (float)(uint32_t)(x >> 40) * 0x1p-24f; }

/* ---------------------------------------------------------------------------------
 * Natural logarithm from basic operations (used by the normal transform).
 * x = m * 2^e with m in [sqrt(1/2), sqrt(2)]; log m = 2 atanh(f), f = (m-1)/(m+1),
 * |f| <= 0.1716, atanh by its Taylor series to f^11; e*ln2 split in a short high part
 * (exact product) and a low correction (Cody & Waite).  Valid for positive normal x.
 * ------------------------------------------------------------------------------- */
float g4o_logf(float x) {
  uint32_t bits;
  memcpy(&bits, &x, 4);
  int32_t e = (int32_t)(bits >> 23) - 127;
  uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) { /* m > sqrt(2): halve it */
    mb -= 0x00800000u;
    e += 1;
  }
  float m;
  memcpy(&m, &mb, 4);
  float num = m - 1.0f;
  float den = m + 1.0f;
  float f = num / den;
  float f2 = f * f;
  float p = 0.0909090936f; /* 1/11 */
  p = p * f2;
  p = p + 0.111111112f; /* 1/9 */
  p = p * f2;
  p = p + 0.142857149f; /* 1/7 */
  p = p * f2;
  p = p + 0.2f; /* 1/5 */
  p = p * f2;
  p = p + 0.333333343f; /* 1/3 */
  float t = f2 * p;
  float twof = f + f;
  float series = twof * t;
  series = series + twof;
  float ef = (float)e;
  float hi = ef * 0.693145751953125f;  /* ln2 high part, 16 significant bits */
  float lo = ef * 1.42860677e-06f;     /* ln2 - high part */
  float r = lo + series;
  return hi + r;
}

/* ---------------------------------------------------------------------------------
 * Standard normal for (neuron, step): Marsaglia's polar method.  One Philox4x32-10 call
 * with key (seed low, seed high) and counter (neuron, step, attempt, stream 4) gives two
 * (x, y) candidate pairs from the top 24 bits of words (0,1) and (2,3); x, y are odd
 * multiples of 2^-24 in (-1, 1) (exact in binary32).  Accept s = x^2 + y^2 < 1,
 * z = x * sqrt(-2 log(s) / s).  Up to 16 calls; if all 32 pairs are rejected
 * (p ~ 1e-21) z = 0.  Replaces curand_normal at gpu4snn.cu:358.
 * ------------------------------------------------------------------------------- */
static inline float pm1_from24(uint32_t k) { return (float)((int32_t)(2u * k + 1u) - 0x1000000) * 0x1p-24f; }

float g4o_normal(uint64_t seed, uint64_t neuron, uint64_t step) {
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (uint32_t attempt = 0; attempt < 16; ++attempt) {
    const uint32_t ctr[4] = {(uint32_t)neuron, (uint32_t)step, attempt, (uint32_t)G4O_STREAM_NOISE};
    uint32_t o[4];
    g4o_philox4x32_10(ctr, key, o);
    for (int p = 0; p < 2; ++p) {
      float x = pm1_from24(o[2 * p] >> 8);
      float y = pm1_from24(o[2 * p + 1] >> 8);
      float xx = x * x;
      float yy = y * y;
      float s = xx + yy;
      if (s < 1.0f) {
        float l = g4o_logf(s);
        float q = -2.0f * l;
        q = q / s;
        float r = sqrtf(q);
        return x * r;
      }
    }
  }
  return 0.0f;
}

float g4o_param_r(uint64_t seed, uint64_t neuron) {
  uint64_t o[4];
  philox(seed, G4O_STREAM_PARAM, neuron, 0, 0, o);
  return u24(o[0]);
}

/* Draw k of a row: draws come in blocks of 128; draw 128b + 32r + l is word r of the
 * Philox call with counter (row, 32b + l).  Uniform on [0,n) (self loops) or on
 * [0,n) \ {row}, by a 64x64->128 multiply (bias <= n / 2^64). */
int64_t g4o_conn_draw(uint64_t seed, int64_t n, int self_loops, int64_t row, int64_t k) {
  uint64_t b = (uint64_t)k >> 7, rem = (uint64_t)k & 127u;
  uint64_t o[4];
  philox(seed, G4O_STREAM_CONN, (uint64_t)row, 32u * b + (rem & 31u), 0, o);
  uint64_t x = o[rem >> 5];
  uint64_t range = self_loops ? (uint64_t)n : (uint64_t)(n - 1);
  uint64_t hi, lo;
  mulhilo64(x, range, &hi, &lo);
  int64_t t = (int64_t)hi;
  if (!self_loops && t >= row) t += 1;
  return t;
}

int64_t g4o_wfix(float w) {
  float s = w * 0x1p32f;
  return (int64_t)llrintf(s);
}

static inline int64_t n_exc_of(const g4o_desc *d) { return (d->n * (int64_t)d->exc_permille) / 1000; }

/* ---------------------------------------------------------------------------------
 * Connectivity, Philox law (the library's default).  Row i gets nsyn distinct targets
 * uniformly from [0,n) (minus i unless self loops), in draw order: draw k is accepted
 * iff its target was not accepted before.  Weight of slot j: (1000/nsyn)*0.5*U for
 * excitatory rows, (1000/nsyn)*(-1)*U for inhibitory ones, U = 24-bit uniform of word
 * j%4 of Philox(row, j/4) — the reference's law at gpu4snn.cu:887-898.
 * ------------------------------------------------------------------------------- */
/* One row of the Philox law into ri/rw; `mark` (n words) remembers the rows that took each
 * target, so it needs no clearing between rows. */
static void conn_philox_row(const g4o_desc *d, int64_t row, int64_t nexc, int64_t *mark, int32_t *ri, float *rw) {
  const int32_t nsyn = d->nsyn, stride = d->stride;
  const float wscale = 1000.0f / (float)nsyn;
  const float wexc = wscale * 0.5f, winh = wscale * -1.0f;
  const uint64_t range = d->self_loops ? (uint64_t)d->n : (uint64_t)(d->n - 1);
  int32_t acc = 0;
  for (uint64_t b = 0; acc < nsyn; ++b) {
    uint64_t blk[32][4];
    for (int l = 0; l < 32; ++l) philox(d->seed, G4O_STREAM_CONN, (uint64_t)row, 32u * b + (uint64_t)l, 0, blk[l]);
    for (int r = 0; r < 4 && acc < nsyn; ++r)
      for (int l = 0; l < 32 && acc < nsyn; ++l) {
        uint64_t hi, lo;
        mulhilo64(blk[l][r], range, &hi, &lo);
        int64_t t = (int64_t)hi;
        if (!d->self_loops && t >= row) t += 1;
        if (mark[t] != row) {
          mark[t] = row;
          ri[acc++] = (int32_t)t;
        }
      }
  }
  const float sc = row < nexc ? wexc : winh;
  for (int32_t j = 0; j < nsyn; j += 4) {
    uint64_t o[4];
    philox(d->seed, G4O_STREAM_WEIGHT, (uint64_t)row, (uint64_t)(j >> 2), 0, o);
    for (int q = 0; q < 4 && j + q < nsyn; ++q) rw[j + q] = sc * u24(o[q]);
  }
  for (int32_t j = nsyn; j < stride; ++j) {
    ri[j] = -1;
    rw[j] = 0.0f;
  }
}

int g4o_conn_philox(const g4o_desc *d, int64_t row0, int64_t nrows, int32_t *idx, float *w) {
  const int64_t n = d->n;
  const int32_t nsyn = d->nsyn, stride = d->stride;
  if (n < 2 || nsyn < 0 || stride < nsyn || nsyn > (d->self_loops ? n : n - 1)) return -1;
  const int64_t nexc = n_exc_of(d);
  int failed = 0;
  /* rows are independent: blocks of rows on all threads, each with its own mark array */
#pragma omp parallel if (nrows > 256)
  {
    int64_t *mark = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    if (!mark) {
#pragma omp atomic write
      failed = 1;
    } else {
      for (int64_t i = 0; i < n; ++i) mark[i] = -1;
#pragma omp for schedule(dynamic, 64)
      for (int64_t rr = 0; rr < nrows; ++rr)
        conn_philox_row(d, row0 + rr, nexc, mark, idx + rr * (int64_t)stride, w + rr * (int64_t)stride);
      free(mark);
    }
  }
  return failed ? -1 : 0;
}

/* Rows in the library's order: by target as unsigned (so unused slots, -1, come last),
 * equal targets by the weight's bits; a least-significant-digit radix sort of the 64-bit
 * keys (target << 32 | weight bits), rows on all threads. */
int g4o_sort_rows(int32_t *idx, float *w, int64_t nrows, int32_t stride) {
  int failed = 0;
#pragma omp parallel if (nrows > 64)
  {
    uint64_t *a = (uint64_t *)malloc((size_t)stride * 8), *b = (uint64_t *)malloc((size_t)stride * 8);
    if (!a || !b) {
#pragma omp atomic write
      failed = 1;
    } else {
#pragma omp for schedule(dynamic, 64)
      for (int64_t r = 0; r < nrows; ++r) {
        int32_t *ri = idx + r * (int64_t)stride;
        float *rw = w + r * (int64_t)stride;
        for (int32_t j = 0; j < stride; ++j) {
          uint32_t wb;
          memcpy(&wb, rw + j, 4);
          a[j] = ((uint64_t)(uint32_t)ri[j] << 32) | wb;
        }
        uint64_t *src = a, *dst = b;
        for (int pass = 0; pass < 8; ++pass) {
          const int sh = 8 * pass;
          uint32_t cnt[257] = {0};
          for (int32_t j = 0; j < stride; ++j) cnt[((src[j] >> sh) & 0xFF) + 1]++;
          if (cnt[((src[0] >> sh) & 0xFF) + 1] == (uint32_t)stride) continue; /* one digit value: order kept */
          for (int k = 0; k < 256; ++k) cnt[k + 1] += cnt[k];
          for (int32_t j = 0; j < stride; ++j) dst[cnt[(src[j] >> sh) & 0xFF]++] = src[j];
          uint64_t *t = src;
          src = dst;
          dst = t;
        }
        for (int32_t j = 0; j < stride; ++j) {
          ri[j] = (int32_t)(uint32_t)(src[j] >> 32);
          const uint32_t wb = (uint32_t)src[j];
          memcpy(rw + j, &wb, 4);
        }
      }
    }
    free(a);
    free(b);
  }
  return failed ? -1 : 0;
}

/* The reference's host generator (gpu4snn.cu:873-898): srand(seed); per row a fresh
 * list 0..n-1; per synapse idx = rand() % size, then one rand() for the weight, take
 * list[idx] and delete it.  Self loops allowed.  Pinned against the reference's own
 * tables. */
int g4o_conn_glibc(unsigned seed, int32_t n, int32_t nsyn, int32_t *idx, float *w) {
  if (n < 1 || nsyn < 0 || nsyn > n) return -1;
  int32_t *post = (int32_t *)malloc((size_t)n * sizeof(int32_t));
  if (!post) return -1;
  const int32_t nexc = (int32_t)(((int64_t)n * 4) / 5);
  srand(seed);
  for (int32_t i = 0; i < n; ++i) {
    size_t size = (size_t)n;
    for (int32_t j = 0; j < n; ++j) post[j] = j;
    for (int32_t j = 0; j < nsyn; ++j) {
      int32_t k = (int32_t)((size_t)rand() % size);
      float x;
      if (i < nexc) {
        x = (1000.0f / (float)nsyn) * 0.5f;
        x = x * (float)rand();
        x = x / (float)RAND_MAX;
      } else {
        x = (1000.0f / (float)nsyn) * -1.0f;
        x = x * (float)rand();
        x = x / (float)RAND_MAX;
      }
      w[(int64_t)i * nsyn + j] = x;
      idx[(int64_t)i * nsyn + j] = post[k];
      memmove(post + k, post + k + 1, (size - (size_t)k - 1) * sizeof(int32_t));
      size--;
    }
  }
  free(post);
  return 0;
}

/* ---------------------------------------------------------------------------------
 * Simulation.
 * ------------------------------------------------------------------------------- */
struct g4o_sim {
  g4o_desc d;
  int mode;
  int64_t nexc;
  const int32_t *idx;
  const float *w;
  float ge, gi;
  /* FP32 state */
  float *v, *u, *ilast;
  int64_t *acc;
  /* FP64 state */
  double *v64, *u64;
  __int128 *acc64; /* FP64 mode: exact Q64.64 sums of the weights */
  float *a, *b, *c, *dd;
  int32_t *nospks, *last;
  int64_t *nisi, *sisi, *sisi2;
  int64_t t;
  /* raster */
  int32_t *rt, *rid;
  int64_t rn, rcap;
  int32_t *counts;
  int64_t ccap;
  int32_t *list;
};

static void *xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

g4o_sim *g4o_sim_create(const g4o_desc *d, const int32_t *idx, const float *w, int mode) {
  if (!d || d->n < 1 || d->stride < d->nsyn) return NULL;
  g4o_sim *s = (g4o_sim *)xcalloc(1, sizeof *s);
  if (!s) return NULL;
  s->d = *d;
  s->mode = mode;
  s->nexc = n_exc_of(d);
  s->idx = idx;
  s->w = w;
  s->ge = 5.0f * d->drive_scale;
  s->gi = 2.0f * d->drive_scale;
  const size_t n = (size_t)d->n;
  s->v = xcalloc(n, 4);
  s->u = xcalloc(n, 4);
  s->ilast = xcalloc(n, 4);
  s->acc = xcalloc(n, 8);
  s->v64 = xcalloc(n, 8);
  s->u64 = xcalloc(n, 8);
  s->acc64 = xcalloc(n, sizeof(__int128));
  s->a = xcalloc(n, 4);
  s->b = xcalloc(n, 4);
  s->c = xcalloc(n, 4);
  s->dd = xcalloc(n, 4);
  s->nospks = xcalloc(n, 4);
  s->last = xcalloc(n, 4);
  s->nisi = xcalloc(n, 8);
  s->sisi = xcalloc(n, 8);
  s->sisi2 = xcalloc(n, 8);
  s->list = xcalloc(n, 4);
  if (!s->v || !s->u || !s->ilast || !s->acc || !s->v64 || !s->u64 || !s->acc64 || !s->a || !s->b ||
      !s->c || !s->dd || !s->nospks || !s->last || !s->nisi || !s->sisi || !s->sisi2 || !s->list) {
    g4o_sim_destroy(s);
    return NULL;
  }
  /* initNeuron, gpu4snn.cu:286-320 (powf(r,2) written as r*r) */
  for (int64_t i = 0; i < d->n; ++i) {
    float r = g4o_param_r(d->seed, (uint64_t)i);
    if (i < s->nexc) {
      float r2 = r * r;
      float t15 = 15.0f * r2, t6 = 6.0f * r2;
      s->a[i] = 0.02f;
      s->b[i] = 0.2f;
      s->c[i] = -65.0f + t15;
      s->dd[i] = 8.0f - t6;
    } else {
      float t8 = 0.08f * r, t5 = 0.05f * r;
      s->a[i] = 0.02f + t8;
      s->b[i] = 0.25f - t5;
      s->c[i] = -65.0f;
      s->dd[i] = 2.0f;
    }
    s->v[i] = -65.0f;
    s->u[i] = s->b[i] * s->v[i];
    s->v64[i] = (double)s->v[i];
    s->u64[i] = (double)s->b[i] * s->v64[i];
    s->last[i] = -1;
  }
  return s;
}

void g4o_sim_destroy(g4o_sim *s) {
  if (!s) return;
  free(s->v); free(s->u); free(s->ilast); free(s->acc); free(s->v64); free(s->u64);
  free(s->acc64); free(s->a); free(s->b); free(s->c); free(s->dd); free(s->nospks);
  free(s->last); free(s->nisi); free(s->sisi); free(s->sisi2); free(s->rt); free(s->rid);
  free(s->counts); free(s->list);
  free(s);
}

static int grow(g4o_sim *s, int64_t need) {
  if (need <= s->rcap) return 0;
  int64_t cap = s->rcap ? s->rcap : 1024;
  while (cap < need) cap *= 2;
  int32_t *a = realloc(s->rt, (size_t)cap * 4), *b;
  if (!a) return -1;
  s->rt = a;
  b = realloc(s->rid, (size_t)cap * 4);
  if (!b) return -1;
  s->rid = b;
  s->rcap = cap;
  return 0;
}

/* One neuron, FP32 mirror of stateupdate (gpu4snn.cu:356-405).  Returns 1 on a spike. */
static inline int update32(g4o_sim *s, int64_t i, int32_t t) {
  float z = g4o_normal(s->d.seed, (uint64_t)i, (uint64_t)t);
  float g = i < s->nexc ? s->ge : s->gi;
  float I = g * z;
  float isyn = (float)s->acc[i] * 0x1p-32f;
  I = I + isyn;
  s->acc[i] = 0;
  float v = s->v[i], u = s->u[i];
  for (int h = 0; h < 2; ++h) {
    float t1 = 0.04f * v;
    t1 = t1 * v;
    float t2 = 5.0f * v;
    t1 = t1 + t2;
    t1 = t1 + 140.0f;
    t1 = t1 - u;
    t1 = t1 + I;
    t1 = 0.5f * t1;
    v = v + t1;
  }
  float t3 = s->b[i] * v;
  t3 = t3 - u;
  t3 = s->a[i] * t3;
  u = u + t3;
  s->ilast[i] = I;
  int spk = (v >= 30.0f) || !isfinite(v);
  if (spk) {
    v = s->c[i];
    u = u + s->dd[i];
  }
  s->v[i] = v;
  s->u[i] = u;
  return spk;
}

/* FP64 currents: each weight as an exact Q64.64 integer (every float weight of magnitude
 * >= 2^-41 is exact; smaller ones round to nearest even), summed without rounding, and
 * converted to double once, correctly rounded, when the neuron consumes them.  The sum
 * therefore does not depend on the order of the additions. */
static inline __int128 wq64(float w) { return (__int128)rint(ldexp((double)w, 64)); }
static inline double q64_to_double(__int128 q) { return (double)q * 0x1p-64; }

/* The same step in double with the same random draws. */
static inline int update64(g4o_sim *s, int64_t i, int32_t t) {
  float z = g4o_normal(s->d.seed, (uint64_t)i, (uint64_t)t);
  double g = i < s->nexc ? (double)s->ge : (double)s->gi;
  double I = g * (double)z + q64_to_double(s->acc64[i]);
  s->acc64[i] = 0;
  double v = s->v64[i], u = s->u64[i];
  v += 0.5 * (0.04 * v * v + 5.0 * v + 140.0 - u + I);
  v += 0.5 * (0.04 * v * v + 5.0 * v + 140.0 - u + I);
  u += (double)s->a[i] * ((double)s->b[i] * v - u);
  s->ilast[i] = (float)I;
  int spk = (v >= 30.0) || !isfinite(v);
  if (spk) {
    v = (double)s->c[i];
    u += (double)s->dd[i];
  }
  s->v64[i] = v;
  s->u64[i] = u;
  s->v[i] = (float)v;
  s->u[i] = (float)u;
  return spk;
}

static inline void on_spike(g4o_sim *s, int64_t i, int32_t t) {
  s->nospks[i] += 1;
  if (s->last[i] >= 0) {
    int64_t isi = (int64_t)t - s->last[i];
    s->nisi[i] += 1;
    s->sisi[i] += isi;
    s->sisi2[i] += isi * isi;
  }
  s->last[i] = t;
}

int g4o_sim_run(g4o_sim *s, int32_t steps, int32_t threads) {
  if (!s || steps < 0) return -1;
  const int64_t n = s->d.n, stride = s->d.stride;
  if (s->ccap < s->t + steps) {
    int64_t cap = s->ccap ? s->ccap : 256;
    while (cap < s->t + steps) cap *= 2;
    int32_t *c = realloc(s->counts, (size_t)cap * 4);
    if (!c) return -1;
    s->counts = c;
    s->ccap = cap;
  }
  int nth = threads < 1 ? 1 : threads;
  if (s->mode == G4O_FP64) nth = 1; /* the FP64 mode runs on one thread */
  for (int32_t st = 0; st < steps; ++st) {
    const int32_t t = (int32_t)s->t;
    int64_t k = 0;
    if (nth == 1) {
      for (int64_t i = 0; i < n; ++i) {
        int spk = s->mode == G4O_FP64 ? update64(s, i, t) : update32(s, i, t);
        if (spk) {
          on_spike(s, i, t);
          s->list[k++] = (int32_t)i;
        }
      }
    } else {
#ifdef _OPENMP
      /* static chunks in thread order keep the merged list sorted by neuron id */
      int64_t *cnt = (int64_t *)calloc((size_t)nth + 1, sizeof(int64_t));
      if (!cnt) return -1;
#pragma omp parallel num_threads(nth)
      {
        int tid = omp_get_thread_num(), nt = omp_get_num_threads();
        int64_t lo = n * tid / nt, hi = n * (tid + 1) / nt, c = 0;
        for (int64_t i = lo; i < hi; ++i)
          if (update32(s, i, t)) {
            on_spike(s, i, t);
            s->list[lo + c++] = (int32_t)i;
          }
        cnt[tid + 1] = c;
#pragma omp barrier
#pragma omp single
        {
          for (int q = 0; q < nt; ++q) {
            int64_t qlo = n * q / nt;
            memmove(s->list + k, s->list + qlo, (size_t)cnt[q + 1] * 4);
            k += cnt[q + 1];
          }
        }
        /* delivery: spike rows in parallel, exact integer atomics */
#pragma omp for schedule(dynamic, 8)
        for (int64_t q = 0; q < k; ++q) {
          const int64_t row = s->list[q];
          const int32_t *ri = s->idx + row * stride;
          const float *rw = s->w + row * stride;
          for (int64_t j = 0; j < stride; ++j) {
            int32_t tg = ri[j];
            if (tg >= 0) __atomic_fetch_add(&s->acc[tg], g4o_wfix(rw[j]), __ATOMIC_RELAXED);
          }
        }
      }
      free(cnt);
#else
      return -1;
#endif
    }
    if (grow(s, s->rn + k)) return -1;
    for (int64_t q = 0; q < k; ++q) {
      s->rt[s->rn + q] = t;
      s->rid[s->rn + q] = s->list[q];
    }
    s->rn += k;
    s->counts[t] = (int32_t)k;
    if (nth == 1) {
      /* spike delivery (gpu4snn.cu:446-467 restated over the spike list) */
      for (int64_t q = 0; q < k; ++q) {
        const int64_t row = s->list[q];
        const int32_t *ri = s->idx + row * stride;
        const float *rw = s->w + row * stride;
        if (s->mode == G4O_FP64) {
          for (int64_t j = 0; j < stride; ++j)
            if (ri[j] >= 0) s->acc64[ri[j]] += wq64(rw[j]);
        } else {
          for (int64_t j = 0; j < stride; ++j)
            if (ri[j] >= 0) s->acc[ri[j]] += g4o_wfix(rw[j]);
        }
      }
    }
    s->t += 1;
  }
  return 0;
}

int64_t g4o_sim_step_index(const g4o_sim *s) { return s->t; }
int64_t g4o_sim_raster_size(const g4o_sim *s) { return s->rn; }

int64_t g4o_sim_raster(const g4o_sim *s, int32_t *t, int32_t *id, int64_t cap) {
  int64_t n = s->rn < cap ? s->rn : cap;
  memcpy(t, s->rt, (size_t)n * 4);
  memcpy(id, s->rid, (size_t)n * 4);
  return n;
}

int64_t g4o_sim_counts(const g4o_sim *s, int32_t *counts, int64_t cap) {
  int64_t n = s->t < cap ? s->t : cap;
  memcpy(counts, s->counts, (size_t)n * 4);
  return n;
}

void g4o_sim_state(const g4o_sim *s, float *v, float *u, float *i_last, float *a, float *b, float *c,
                   float *dd, int32_t *nospks) {
  const size_t n = (size_t)s->d.n;
  if (v) memcpy(v, s->v, n * 4);
  if (u) memcpy(u, s->u, n * 4);
  if (i_last) memcpy(i_last, s->ilast, n * 4);
  if (a) memcpy(a, s->a, n * 4);
  if (b) memcpy(b, s->b, n * 4);
  if (c) memcpy(c, s->c, n * 4);
  if (dd) memcpy(dd, s->dd, n * 4);
  if (nospks) memcpy(nospks, s->nospks, n * 4);
}

void g4o_sim_state64(const g4o_sim *s, double *v, double *u) {
  const size_t n = (size_t)s->d.n;
  if (v) memcpy(v, s->v64, n * 8);
  if (u) memcpy(u, s->u64, n * 8);
}

void g4o_sim_acc(const g4o_sim *s, int64_t *acc) { memcpy(acc, s->acc, (size_t)s->d.n * 8); }

void g4o_sim_stats(const g4o_sim *s, double *rate_hz, double *isi_cv, int64_t *total_spikes) {
  int64_t tot = s->rn;
  double cvsum = 0.0;
  int64_t ncv = 0;
  for (int64_t i = 0; i < s->d.n; ++i) {
    int64_t m = s->nisi[i];
    if (m >= 2) {
      double mean = (double)s->sisi[i] / (double)m;
      double var = (double)(m * s->sisi2[i] - s->sisi[i] * s->sisi[i]) / ((double)m * (double)m);
      cvsum += sqrt(var) / mean;
      ncv++;
    }
  }
  if (total_spikes) *total_spikes = tot;
  if (rate_hz) *rate_hz = s->t ? (double)tot * 1000.0 / ((double)s->d.n * (double)s->t) : 0.0;
  if (isi_cv) *isi_cv = ncv ? cvsum / (double)ncv : 0.0;
}
