/*
 * bw_oracle.c -- TEST INFRASTRUCTURE ONLY (see bw_oracle.h).
 *
 * Restates, in plain C, the reference semantics that the GPU path must match
 * bit for bit.  Every function cites the reference file:line it follows.
 * Nothing in the product links this file.
 */
#include "bw_oracle.h"

#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
typedef __int128 i128;

/* ================================================================ SHA-256
 * FIPS 180-4 section 6.2.  The round constants are the first 32 bits of the
 * fractional parts of the cube roots of the first 64 primes and the initial hash
 * the same for the square roots of the first 8 primes (FIPS 180-4 4.2.2, 5.3.3);
 * they are derived here with exact integer roots instead of being tabulated. */
static uint32_t sha_k[64], sha_h0[8];
static int sha_ready = 0;

static uint64_t iroot(u128 x, int n) {   /* floor(x^(1/n)) for n in {2,3} */
  uint64_t lo = 0, hi = (uint64_t)1 << 40;
  while (lo < hi) {
    uint64_t mid = lo + (hi - lo + 1) / 2;
    u128 p = (u128)mid * mid;
    if (n == 3) p *= mid;
    if (p <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

static void sha_init_constants(void) {
  uint32_t primes[64];
  int np = 0;
  for (uint32_t c = 2; np < 64; ++c) {
    int is_p = 1;
    for (int i = 0; i < np && primes[i] * primes[i] <= c; ++i)
      if (c % primes[i] == 0) { is_p = 0; break; }
    if (is_p) primes[np++] = c;
  }
  for (int i = 0; i < 64; ++i) sha_k[i] = (uint32_t)iroot((u128)primes[i] << 96, 3);
  for (int i = 0; i < 8; ++i) sha_h0[i] = (uint32_t)iroot((u128)primes[i] << 64, 2);
  sha_ready = 1;
}

static inline uint32_t rotr32(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static void sha_block(uint32_t h[8], const uint8_t* p) {
  uint32_t w[64];
  for (int i = 0; i < 16; ++i)
    w[i] = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) |
           ((uint32_t)p[4 * i + 2] << 8) | (uint32_t)p[4 * i + 3];
  for (int i = 16; i < 64; ++i) {
    uint32_t s0 = rotr32(w[i - 15], 7) ^ rotr32(w[i - 15], 18) ^ (w[i - 15] >> 3);
    uint32_t s1 = rotr32(w[i - 2], 17) ^ rotr32(w[i - 2], 19) ^ (w[i - 2] >> 10);
    w[i] = w[i - 16] + s0 + w[i - 7] + s1;
  }
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], k = h[7];
  for (int i = 0; i < 64; ++i) {
    uint32_t t1 = k + (rotr32(e, 6) ^ rotr32(e, 11) ^ rotr32(e, 25)) + ((e & f) ^ (~e & g)) +
                  sha_k[i] + w[i];
    uint32_t t2 = (rotr32(a, 2) ^ rotr32(a, 13) ^ rotr32(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
    k = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += k;
}

void bwo_sha256_hex(const void* data, size_t n, char out_hex[65]) {
  if (!sha_ready) sha_init_constants();
  uint32_t h[8];
  memcpy(h, sha_h0, sizeof(h));
  const uint8_t* p = (const uint8_t*)data;
  size_t full = n / 64;
  for (size_t i = 0; i < full; ++i) sha_block(h, p + 64 * i);
  uint8_t tail[128];
  size_t rem = n - full * 64;
  memset(tail, 0, sizeof(tail));
  if (rem) memcpy(tail, p + full * 64, rem);
  tail[rem] = 0x80;
  size_t tl = (rem < 56) ? 64 : 128;
  uint64_t bits = (uint64_t)n * 8u;
  for (int i = 0; i < 8; ++i) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
  sha_block(h, tail);
  if (tl == 128) sha_block(h, tail + 64);
  static const char* hx = "0123456789abcdef";
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) out_hex[8 * i + j] = hx[(h[i] >> (28 - 4 * j)) & 15];
  out_hex[64] = 0;
}

/* common.hpp:396-400 */
uint64_t bwo_fnv1a(const void* data, size_t n) {
  const uint8_t* p = (const uint8_t*)data;
  uint64_t h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ULL;
  return h;
}

/* ================================================================ RNG
 * SplitMix64 as common.hpp:40-54 (seed 0 is replaced by the golden gamma). */
#define GAMMA 0x9E3779B97F4A7C15ULL
uint64_t bwo_splitmix_next(uint64_t* s) {
  uint64_t z = (*s += GAMMA);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline uint64_t rng_seed(uint64_t s) { return s ? s : GAMMA; }
static inline uint32_t rng_bounded(uint64_t* s, uint32_t n) {
  return n ? (uint32_t)(bwo_splitmix_next(s) % n) : 0;
}
static inline int64_t rng_range(uint64_t* s, int64_t lo, int64_t hi) {
  if (hi <= lo) return lo;
  return lo + (int64_t)(bwo_splitmix_next(s) % (uint64_t)(hi - lo));
}

/* ================================================================ fixture */
static inline int64_t ld64(const uint8_t* p) { int64_t x; memcpy(&x, p, 8); return x; }
static inline int32_t ld32(const uint8_t* p) { int32_t x; memcpy(&x, p, 4); return x; }

int bwo_fixture_parse(const void* image, size_t len, bwo_fixture* f) {
  const uint8_t* b = (const uint8_t*)image;
  if (len < 64 || memcmp(b, "BWBASE02", 8) != 0) return 3;
  int64_t n = ld64(b + 8);
  int32_t G = ld32(b + 16);
  if (n <= 0 || G <= 0 || n > ((int64_t)1 << 40) || G > (1 << 20)) return 3;
  size_t off_rows = 64, off_fac = off_rows + (size_t)n * 24, off_lab = off_fac + (size_t)G * 8;
  if (off_lab + (size_t)G * 4 > len) return 3;
  f->n = n;
  f->groups = G;
  f->unit = ld32(b + 20);
  f->t_min = ld64(b + 40);
  f->t_max = ld64(b + 48);
  f->rows = b + off_rows;
  f->row_t = (const int64_t*)(b + off_rows);
  f->factor = (const int64_t*)(b + off_fac);
  f->labels = (const int32_t*)(b + off_lab);
  for (int32_t g = 0; g < G; ++g)
    if (ld64(b + off_fac + (size_t)g * 8) <= 0) return 3;
  return 0;
}
static inline int64_t row_t(const bwo_fixture* f, int64_t i) { return ld64(f->rows + 24 * i); }
static inline int64_t row_amt(const bwo_fixture* f, int64_t i) { return ld64(f->rows + 24 * i + 8); }
static inline int32_t row_g(const bwo_fixture* f, int64_t i) { return ld32(f->rows + 24 * i + 16); }
static inline int64_t fac0(const bwo_fixture* f, int32_t g) {
  return ld64((const uint8_t*)f->factor + 8 * (size_t)g);
}

/* ================================================================ workload */
/* version_parent, common.hpp:219-226 */
static int32_t version_parent(int32_t topology, int32_t v) {
  if (v <= 0) return -1;
  if (topology == 0) return v - 1;
  if (topology == 1) return (v - 1) / 2;
  return 0;
}

/* gen_nested, common.hpp:229-246 (only the first q levels are generated; level k
 * depends only on the first 2k draws, so the values equal the kMaxQ-level run). */
static void gen_nested(uint64_t* r, int64_t tmin, int64_t tmax, int32_t q, int64_t* lo_out,
                       int64_t* hi_out) {
  int64_t lo = tmin, hi = tmax + 1;
  const int64_t span0 = hi - lo;
  for (int32_t k = 0; k < q; ++k) {
    int64_t span = hi - lo;
    if (span <= 4096) {
      lo = tmin + span0 / 2;
      hi = lo + 2048;
      span = hi - lo;
    }
    int64_t a = span * (int64_t)(3 + rng_bounded(r, 16)) / 100;
    int64_t b = span * (int64_t)(3 + rng_bounded(r, 16)) / 100;
    lo += a;
    hi -= b;
    if (hi - lo < 1024) hi = lo + 1024;
    lo_out[k] = lo;
    hi_out[k] = hi;
  }
}

static int cmp_i64(const void* a, const void* b) {
  int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  return (x > y) - (x < y);
}

void bwo_workload_free(bwo_workload* w) {
  free(w->parent); free(w->op); free(w->eg); free(w->eid); free(w->eval); free(w->et);
  free(w->qlo); free(w->qhi); free(w->ins_t); free(w->ins_g); free(w->endpoints);
  memset(w, 0, sizeof(*w));
}

/* make_workload, common.hpp:279-374 */
int bwo_workload_make(const bwo_fixture* f, int32_t S, int32_t topology, int32_t seed,
                      int32_t fp, int32_t q, int32_t per_state, int32_t factor_pct,
                      bwo_workload* w) {
  memset(w, 0, sizeof(*w));
  if (S < 2 || q < 1 || topology < 0 || topology > 2) return 2;
  w->n_states = S; w->topology = topology; w->seed = seed; w->factor_period = fp; w->q = q;
  w->per_state = per_state; w->factor_pct = factor_pct;
  w->n_base = f->n; w->groups = f->groups; w->t_min = f->t_min; w->t_max = f->t_max;
  const int64_t N = f->n, tmin = f->t_min, tmax = f->t_max;
  const int32_t G = f->groups;
  w->parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)S);
  w->op = (uint8_t*)calloc((size_t)S, 1);
  w->eg = (int32_t*)calloc((size_t)S, 4);
  w->eid = (int64_t*)calloc((size_t)S, 8);
  w->eval = (int64_t*)calloc((size_t)S, 8);
  w->et = (int64_t*)calloc((size_t)S, 8);
  w->ins_t = (int64_t*)malloc(8 * (size_t)S);
  w->ins_g = (int32_t*)malloc(4 * (size_t)S);
  size_t nq = per_state ? (size_t)S * (size_t)q : (size_t)q;
  w->qlo = (int64_t*)calloc(nq, 8);
  w->qhi = (int64_t*)calloc(nq, 8);
  if (per_state) {
    for (int32_t v = 1; v < S; ++v) {
      uint64_t r = rng_seed((uint64_t)(int64_t)seed * 1000000007ULL + (uint64_t)(int64_t)topology * 65537ULL +
                            (uint64_t)(int64_t)fp * 131ULL + (uint64_t)v * 2654435761ULL + 17ULL);
      gen_nested(&r, tmin, tmax, q, w->qlo + (size_t)v * q, w->qhi + (size_t)v * q);
    }
  } else {
    uint64_t r = rng_seed((uint64_t)(int64_t)seed * 1000000007ULL + (uint64_t)(int64_t)topology * 65537ULL +
                          (uint64_t)(int64_t)fp * 131ULL + 17ULL);
    gen_nested(&r, tmin, tmax, q, w->qlo, w->qhi);
  }
  uint64_t rng = rng_seed((uint64_t)(int64_t)seed * 1000003ULL + (uint64_t)(int64_t)topology * 7919ULL +
                          (uint64_t)(int64_t)fp * 104729ULL + 20261025ULL);
  for (int32_t v = 0; v < S; ++v) w->parent[v] = version_parent(topology, v);
  int64_t* gfactor = (int64_t*)malloc(8 * (size_t)G);
  for (int32_t g = 0; g < G; ++g) gfactor[g] = 1000;
  int32_t next_group = 0, next_ins = 0;
  for (int32_t v = 1; v < S; ++v) {
    int factor_step;
    if (factor_pct >= 0) factor_step = rng_bounded(&rng, 100) < (uint32_t)factor_pct;
    else factor_step = (fp > 0) && (v % fp == 0);
    if (factor_step) {
      int32_t g = next_group++ % G;
      int64_t cur = gfactor[g];
      int64_t nf = (cur == 950) ? 1000 : (cur == 1000 ? 1050 : 950);
      gfactor[g] = nf;
      w->op[v] = BWO_OP_FACTOR; w->eg[v] = g; w->eval[v] = nf;
    } else {
      uint32_t roll = rng_bounded(&rng, 100);
      if (roll < 55) {
        w->op[v] = BWO_OP_REPLACE;
        w->eid[v] = rng_range(&rng, 0, N);
        w->eval[v] = row_amt(f, w->eid[v]) + rng_range(&rng, -100000, 100000);
      } else if (roll < 75) {
        w->op[v] = BWO_OP_INSERT;
        w->eid[v] = N + next_ins;
        w->et[v] = rng_range(&rng, tmin, tmax + 1);
        w->eg[v] = (int32_t)rng_bounded(&rng, (uint32_t)G);
        int64_t base_amt = row_amt(f, rng_bounded(&rng, (uint32_t)N));
        w->eval[v] = base_amt + rng_range(&rng, -100000, 100000);
        w->ins_t[next_ins] = w->et[v];
        w->ins_g[next_ins] = w->eg[v];
        ++next_ins;
      } else if (roll < 90) {
        w->op[v] = BWO_OP_DELETE;
        w->eid[v] = rng_range(&rng, 0, N);
      } else {
        w->op[v] = BWO_OP_MOVE;
        w->eid[v] = rng_range(&rng, 0, N);
        w->et[v] = rng_range(&rng, tmin, tmax + 1);
        w->eg[v] = (int32_t)rng_bounded(&rng, (uint32_t)G);
        w->eval[v] = row_amt(f, w->eid[v]) + rng_range(&rng, -100000, 100000);
      }
    }
  }
  free(gfactor);
  w->n_inserted = next_ins;
  /* declared endpoint domain: distinct endpoints of every state's first q ranges */
  size_t ne = (size_t)(S - 1) * (size_t)q * 2;
  w->endpoints = (int64_t*)malloc(8 * (ne ? ne : 1));
  size_t m = 0;
  for (int32_t v = 1; v < S; ++v)
    for (int32_t k = 0; k < q; ++k) {
      size_t qi = per_state ? (size_t)v * q + k : (size_t)k;
      w->endpoints[m++] = w->qlo[qi];
      w->endpoints[m++] = w->qhi[qi];
    }
  qsort(w->endpoints, m, 8, cmp_i64);
  size_t u = 0;
  for (size_t i = 0; i < m; ++i)
    if (u == 0 || w->endpoints[u - 1] != w->endpoints[i]) w->endpoints[u++] = w->endpoints[i];
  w->n_endpoints = (int64_t)u;
  return 0;
}

/* ================================================================ direct scan */
/* oracle.cpp:213-451: apply on entry, answer by one scan over all rows, revert on
 * exit.  Children are visited in ascending id order (oracle.cpp:268-276). */
int bwo_direct_scan(const bwo_fixture* f, const bwo_workload* w, int64_t* answers) {
  const int32_t S = w->n_states, q = w->q, G = w->groups;
  const int64_t N = w->n_base, M = w->n_base + w->n_inserted;
  int64_t* t = (int64_t*)malloc(8 * (size_t)M);
  int64_t* amt = (int64_t*)malloc(8 * (size_t)M);
  int32_t* g = (int32_t*)malloc(4 * (size_t)M);
  uint8_t* ex = (uint8_t*)malloc((size_t)M);
  int64_t* fac = (int64_t*)malloc(8 * (size_t)G);
  for (int64_t i = 0; i < N; ++i) { t[i] = row_t(f, i); amt[i] = row_amt(f, i); g[i] = row_g(f, i); ex[i] = 1; }
  for (int64_t k = 0; k < w->n_inserted; ++k) { t[N + k] = w->ins_t[k]; g[N + k] = w->ins_g[k]; amt[N + k] = 0; ex[N + k] = 0; }
  for (int32_t gg = 0; gg < G; ++gg) fac[gg] = fac0(f, gg);
  /* undo records */
  int64_t* u_amt = (int64_t*)malloc(8 * (size_t)S);
  int64_t* u_t = (int64_t*)malloc(8 * (size_t)S);
  int64_t* u_fac = (int64_t*)malloc(8 * (size_t)S);
  int32_t* u_g = (int32_t*)malloc(4 * (size_t)S);
  uint8_t* u_ex = (uint8_t*)malloc((size_t)S);
  /* children CSR, ascending */
  int32_t* cnt = (int32_t*)calloc((size_t)S + 1, 4);
  for (int32_t v = 1; v < S; ++v) {
    int32_t p = w->parent[v];
    if (p < 0 || p >= v) return 7;
    cnt[p + 1]++;
  }
  for (int32_t v = 0; v < S; ++v) cnt[v + 1] += cnt[v];
  int32_t* kids = (int32_t*)malloc(4 * (size_t)(S > 1 ? S - 1 : 1));
  int32_t* cur = (int32_t*)malloc(4 * (size_t)S);
  memcpy(cur, cnt, 4 * (size_t)S);
  for (int32_t v = 1; v < S; ++v) kids[cur[w->parent[v]]++] = v;
  int32_t* st_v = (int32_t*)malloc(4 * (size_t)S);
  int32_t* st_c = (int32_t*)malloc(4 * (size_t)S);
  i128* acc = (i128*)malloc(sizeof(i128) * (size_t)q);
  int rc = 0;
  int top = 0;
  st_v[0] = 0; st_c[0] = cnt[0];
  while (top >= 0) {
    int32_t v = st_v[top];
    if (st_c[top] < cnt[v + 1]) {
      int32_t c = kids[st_c[top]++];
      /* apply(c), oracle.cpp:280-330 */
      int64_t id = w->eid[c];
      switch (w->op[c]) {
        case BWO_OP_REPLACE: u_amt[c] = amt[id]; u_ex[c] = ex[id]; amt[id] = w->eval[c]; ex[id] = 1; break;
        case BWO_OP_INSERT:
        case BWO_OP_MOVE:
          u_amt[c] = amt[id]; u_t[c] = t[id]; u_g[c] = g[id]; u_ex[c] = ex[id];
          t[id] = w->et[c]; g[id] = w->eg[c]; amt[id] = w->eval[c]; ex[id] = 1; break;
        case BWO_OP_DELETE: u_ex[c] = ex[id]; ex[id] = 0; break;
        case BWO_OP_FACTOR: u_fac[c] = fac[w->eg[c]]; fac[w->eg[c]] = w->eval[c]; break;
        default: rc = 7; break;
      }
      /* answer_state(c), oracle.cpp:359-422 (general form; same values as the
       * nested bucket shortcut) */
      const int64_t* lo = w->per_state ? w->qlo + (size_t)c * q : w->qlo;
      const int64_t* hi = w->per_state ? w->qhi + (size_t)c * q : w->qhi;
      int nested = 1;
      for (int32_t k = 1; k < q; ++k)
        if (lo[k] < lo[k - 1] || hi[k] > hi[k - 1]) nested = 0;
      for (int32_t k = 0; k < q; ++k) acc[k] = 0;
      if (nested) {
        for (int64_t i = 0; i < M; ++i) {
          if (!ex[i]) continue;
          int32_t k = 0;
          while (k < q && t[i] >= lo[k] && t[i] < hi[k]) ++k;
          if (k) acc[k - 1] += (i128)amt[i] * (i128)fac[g[i]];
        }
        i128 run = 0;
        for (int32_t k = q - 1; k >= 0; --k) { run += acc[k]; acc[k] = run; }
      } else {
        for (int64_t i = 0; i < M; ++i) {
          if (!ex[i]) continue;
          i128 cv = (i128)amt[i] * (i128)fac[g[i]];
          for (int32_t k = 0; k < q; ++k)
            if (t[i] >= lo[k] && t[i] < hi[k]) acc[k] += cv;
        }
      }
      int64_t* out = answers + (size_t)(c - 1) * q;
      for (int32_t k = 0; k < q; ++k) {
        if (acc[k] < (i128)INT64_MIN || acc[k] > (i128)INT64_MAX) rc = rc ? rc : 6;
        out[k] = (int64_t)(uint64_t)(u128)acc[k];
      }
      ++top;
      st_v[top] = c; st_c[top] = cnt[c];
    } else {
      if (v > 0) {  /* revert(v), oracle.cpp:332-355 */
        int64_t id = w->eid[v];
        switch (w->op[v]) {
          case BWO_OP_REPLACE: amt[id] = u_amt[v]; ex[id] = u_ex[v]; break;
          case BWO_OP_INSERT:
          case BWO_OP_MOVE: t[id] = u_t[v]; g[id] = u_g[v]; amt[id] = u_amt[v]; ex[id] = u_ex[v]; break;
          case BWO_OP_DELETE: ex[id] = u_ex[v]; break;
          case BWO_OP_FACTOR: fac[w->eg[v]] = u_fac[v]; break;
          default: break;
        }
      }
      --top;
    }
  }
  free(t); free(amt); free(g); free(ex); free(fac); free(u_amt); free(u_t); free(u_fac);
  free(u_g); free(u_ex); free(cnt); free(kids); free(cur); free(st_v); free(st_c); free(acc);
  return rc;
}

/* ================================================================ event model */
/* CSR of item indices grouped by state, stable. */
static int32_t* group_by_state(int32_t S, int64_t n, const void* items, size_t stride,
                               int64_t** idx_out) {
  int32_t* off = (int32_t*)calloc((size_t)S + 1, 4);
  const uint8_t* b = (const uint8_t*)items;
  for (int64_t i = 0; i < n; ++i) {
    uint32_t s; memcpy(&s, b + (size_t)i * stride, 4);
    off[s + 1]++;
  }
  for (int32_t v = 0; v < S; ++v) off[v + 1] += off[v];
  int64_t* idx = (int64_t*)malloc(8 * (size_t)(n ? n : 1));
  int32_t* cur = (int32_t*)malloc(4 * (size_t)S);
  memcpy(cur, off, 4 * (size_t)S);
  for (int64_t i = 0; i < n; ++i) {
    uint32_t s; memcpy(&s, b + (size_t)i * stride, 4);
    idx[cur[s]++] = i;
  }
  free(cur);
  *idx_out = idx;
  return off;
}

static int validate_ev(int32_t S, const int32_t* parent, uint32_t C, int64_t E, const bwo_event* ev,
                       int64_t Q, const bwo_query* qs) {
  if (S < 1 || parent[0] != -1) return 2;
  for (int32_t v = 1; v < S; ++v)
    if (parent[v] < 0 || parent[v] >= v) return 2;
  for (int64_t i = 0; i < E; ++i)
    if (ev[i].state >= (uint32_t)S || (C && ev[i].key >= C)) return 2;
  for (int64_t i = 0; i < Q; ++i)
    if (qs[i].state >= (uint32_t)S || (C && (qs[i].lo > C || qs[i].hi > C))) return 2;
  return 0;
}

int bwo_ev_bruteforce(int32_t S, const int32_t* parent, int64_t E, const bwo_event* ev,
                      int64_t Q, const bwo_query* qs, int64_t* answers) {
  int rc = validate_ev(S, parent, 0, E, ev, Q, qs);
  if (rc) return rc;
  int64_t* eidx;
  int32_t* eoff = group_by_state(S, E, ev, sizeof(bwo_event), &eidx);
  for (int64_t j = 0; j < Q; ++j) {
    i128 acc = 0;
    const uint32_t lo = qs[j].lo, hi = qs[j].hi;
    if (hi > lo)
      for (int32_t s = (int32_t)qs[j].state; s >= 0; s = parent[s])
        for (int32_t a = eoff[s]; a < eoff[s + 1]; ++a) {
          const bwo_event* e = &ev[eidx[a]];
          if (e->key >= lo && e->key < hi) acc += e->delta;
        }
    if (acc < (i128)INT64_MIN || acc > (i128)INT64_MAX) rc = 6;
    answers[j] = (int64_t)(uint64_t)(u128)acc;
  }
  free(eidx); free(eoff);
  return rc;
}

/* Preorder apply/undo replay (batch_engine_v7.hpp:1021-1059): an event is added on
 * entry to its state and removed when the preorder leaves the state's subtree. */
static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int ev_sweep_impl(int32_t S, const int32_t* parent, uint32_t C, int64_t E,
                         const bwo_event* ev, int64_t Q, const bwo_query* qs, int64_t* answers,
                         int64_t limit_steps, int64_t* answered, double* seconds) {
  int rc = validate_ev(S, parent, C, E, ev, Q, qs);
  if (rc) return rc;
  int64_t *eidx, *qidx;
  int32_t* eoff = group_by_state(S, E, ev, sizeof(bwo_event), &eidx);
  int32_t* qoff = group_by_state(S, Q, qs, sizeof(bwo_query), &qidx);
  int32_t* cnt = (int32_t*)calloc((size_t)S + 1, 4);
  for (int32_t v = 1; v < S; ++v) cnt[parent[v] + 1]++;
  for (int32_t v = 0; v < S; ++v) cnt[v + 1] += cnt[v];
  int32_t* kids = (int32_t*)malloc(4 * (size_t)(S > 1 ? S - 1 : 1));
  int32_t* cur = (int32_t*)malloc(4 * (size_t)S);
  memcpy(cur, cnt, 4 * (size_t)S);
  for (int32_t v = 1; v < S; ++v) kids[cur[parent[v]]++] = v;
  uint64_t* fen = (uint64_t*)calloc((size_t)C + 1, 8);
  int32_t* st_v = (int32_t*)malloc(4 * (size_t)S);
  int32_t* st_c = (int32_t*)malloc(4 * (size_t)S);
  int64_t steps = 0, done = 0;
  int top = 0;
  st_v[0] = 0; st_c[0] = -1;  /* -1: not yet entered */
  const double t_start = now_s();
  while (top >= 0) {
    int32_t v = st_v[top];
    if (st_c[top] < 0) {
      if (limit_steps >= 0 && steps >= limit_steps) break;
      ++steps;
      for (int32_t a = eoff[v]; a < eoff[v + 1]; ++a) {
        const bwo_event* e = &ev[eidx[a]];
        for (uint32_t i = e->key + 1; i <= C; i += i & (0u - i)) fen[i] += (uint64_t)e->delta;
      }
      for (int32_t a = qoff[v]; a < qoff[v + 1]; ++a) {
        const bwo_query* qq = &qs[qidx[a]];
        uint64_t r = 0;
        if (qq->hi > qq->lo) {
          for (uint32_t i = qq->hi; i > 0; i -= i & (0u - i)) r += fen[i];
          for (uint32_t i = qq->lo; i > 0; i -= i & (0u - i)) r -= fen[i];
        }
        answers[qidx[a]] = (int64_t)r;
        ++done;
      }
      st_c[top] = cnt[v];
    } else if (st_c[top] < cnt[v + 1]) {
      int32_t c = kids[st_c[top]++];
      ++top;
      st_v[top] = c; st_c[top] = -1;
    } else {
      for (int32_t a = eoff[v]; a < eoff[v + 1]; ++a) {
        const bwo_event* e = &ev[eidx[a]];
        for (uint32_t i = e->key + 1; i <= C; i += i & (0u - i)) fen[i] -= (uint64_t)e->delta;
      }
      --top;
    }
  }
  if (seconds) *seconds = now_s() - t_start;
  if (answered) *answered = done;
  free(eidx); free(qidx); free(eoff); free(qoff); free(cnt); free(kids); free(cur); free(fen);
  free(st_v); free(st_c);
  return 0;
}

int bwo_ev_sweep(int32_t S, const int32_t* parent, uint32_t C, int64_t E, const bwo_event* ev,
                 int64_t Q, const bwo_query* qs, int64_t* answers) {
  return ev_sweep_impl(S, parent, C, E, ev, Q, qs, answers, -1, NULL, NULL);
}

int bwo_ev_sweep_prefix(int32_t S, const int32_t* parent, uint32_t C, int64_t E,
                        const bwo_event* ev, int64_t Q, const bwo_query* qs, int64_t* answers,
                        int64_t limit_steps, int64_t* answered, double* seconds) {
  return ev_sweep_impl(S, parent, C, E, ev, Q, qs, answers, limit_steps, answered, seconds);
}

int bwo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Block-parallel chain executor, batch_engine_v7.hpp:707-722 (equal state blocks)
 * and 832-968 (phase 1 local replay, phase 2 serial carry, phase 3 combine). */
int bwo_ev_blocks(int32_t S, const int32_t* parent, uint32_t C, int64_t E, const bwo_event* ev,
                  int64_t Q, const bwo_query* qs, int64_t* answers, int32_t B, int32_t threads) {
  int rc = validate_ev(S, parent, C, E, ev, Q, qs);
  if (rc) return rc;
  for (int32_t v = 1; v < S; ++v)
    if (parent[v] != v - 1) return 2;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  if (B <= 0) B = bwo_max_threads();
  if (B > S) B = S;
  int64_t *eidx, *qidx;
  int32_t* eoff = group_by_state(S, E, ev, sizeof(bwo_event), &eidx);
  int32_t* qoff = group_by_state(S, Q, qs, sizeof(bwo_query), &qidx);
  const size_t Cp = (size_t)C + 1;
  uint64_t* dV = (uint64_t*)calloc((size_t)B * Cp, 8);
  uint64_t* cp = (uint64_t*)malloc(8 * (size_t)B * Cp);
  uint64_t* lv = (uint64_t*)malloc(16 * (size_t)(Q ? Q : 1));
  int32_t* bidx = (int32_t*)malloc(4 * (size_t)S);
  /* phase 1 */
#pragma omp parallel
  {
    uint64_t* fen = (uint64_t*)malloc(8 * Cp);
#pragma omp for schedule(dynamic, 1)
    for (int32_t b = 0; b < B; ++b) {
      int32_t v0 = (int32_t)(((int64_t)S * b) / B), v1 = (int32_t)(((int64_t)S * (b + 1)) / B);
      memset(fen, 0, 8 * Cp);
      uint64_t* leaf = dV + (size_t)b * Cp;
      for (int32_t v = v0; v < v1; ++v) {
        bidx[v] = b;
        for (int32_t a = eoff[v]; a < eoff[v + 1]; ++a) {
          const bwo_event* e = &ev[eidx[a]];
          leaf[e->key + 1] += (uint64_t)e->delta;
          for (uint32_t i = e->key + 1; i <= C; i += i & (0u - i)) fen[i] += (uint64_t)e->delta;
        }
        for (int32_t a = qoff[v]; a < qoff[v + 1]; ++a) {
          const bwo_query* qq = &qs[qidx[a]];
          uint64_t rl = 0, rh = 0;
          for (uint32_t i = qq->lo; i > 0; i -= i & (0u - i)) rl += fen[i];
          for (uint32_t i = qq->hi; i > 0; i -= i & (0u - i)) rh += fen[i];
          lv[2 * qidx[a]] = rl;
          lv[2 * qidx[a] + 1] = rh;
        }
      }
    }
    free(fen);
  }
  /* phase 2 */
  uint64_t* vstart = (uint64_t*)calloc(Cp, 8);
  for (int32_t b = 0; b < B; ++b) {
    uint64_t* c = cp + (size_t)b * Cp;
    c[0] = 0;
    for (size_t k = 1; k < Cp; ++k) c[k] = c[k - 1] + vstart[k];
    const uint64_t* d = dV + (size_t)b * Cp;
    for (size_t k = 1; k < Cp; ++k) vstart[k] += d[k];
  }
  /* phase 3 */
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < Q; ++j) {
    const bwo_query* qq = &qs[j];
    uint64_t r = 0;
    if (qq->hi > qq->lo) {
      const uint64_t* c = cp + (size_t)bidx[qq->state] * Cp;
      r = (c[qq->hi] - c[qq->lo]) + (lv[2 * j + 1] - lv[2 * j]);
    }
    answers[j] = (int64_t)r;
  }
  free(eidx); free(qidx); free(eoff); free(qoff); free(dV); free(cp); free(lv); free(bidx);
  free(vstart);
  return 0;
}

/* ---------------------------------------------------------- sparse-key rank index */
typedef struct { uint64_t key; int64_t amount; } bwo_pair;

static int bwo_pair_cmp(const void* a, const void* b) {
  const uint64_t x = ((const bwo_pair*)a)->key, y = ((const bwo_pair*)b)->key;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* build_csr_base (sparse_engine.hpp:287-360): there, pass 1 marks each (group,
 * class) support in a bitmap, the popcount table gives every support its rank, pass
 * 2 adds each row's amount at its rank and a final scan makes the cumulative prefix.
 * Over u64 keys the same result is the sorted distinct keys with summed amounts and
 * their running total. */
int bwo_csr_build(const uint64_t* keys, const int64_t* amounts, int64_t n, uint64_t* out_keys,
                  int64_t* out_pre, int64_t* m) {
  *m = 0;
  if (n <= 0) return 0;
  bwo_pair* p = (bwo_pair*)malloc((size_t)n * sizeof(bwo_pair));
  if (!p) return 1;
  for (int64_t i = 0; i < n; ++i) { p[i].key = keys[i]; p[i].amount = amounts[i]; }
  qsort(p, (size_t)n, sizeof(bwo_pair), bwo_pair_cmp);
  uint64_t run = 0;
  int64_t u = -1;
  for (int64_t i = 0; i < n; ++i) {
    run += (uint64_t)p[i].amount;
    if (u < 0 || out_keys[u] != p[i].key) out_keys[++u] = p[i].key;
    out_pre[u] = (int64_t)run;
  }
  *m = u + 1;
  free(p);
  return 0;
}

/* number of ukeys[0..m) below k (CsrBase::rank, sparse_engine.hpp:79-88) */
static int64_t bwo_csr_rank(const uint64_t* ukeys, int64_t m, uint64_t k) {
  int64_t lo = 0, hi = m;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (ukeys[mid] < k) lo = mid + 1; else hi = mid;
  }
  return lo;
}

void bwo_csr_point(const uint64_t* ukeys, int64_t m, const uint64_t* q, int64_t n, int64_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    const int64_t r = bwo_csr_rank(ukeys, m, q[i]);
    out[i] = (r < m && ukeys[r] == q[i]) ? r : -r - 1;
  }
}

/* CsrBase::range (sparse_engine.hpp:89-97) */
void bwo_csr_range(const uint64_t* ukeys, const int64_t* pre, int64_t m, const uint64_t* bounds,
                   int64_t n, int64_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    const int64_t a = bwo_csr_rank(ukeys, m, bounds[2 * i]);
    const int64_t b = bwo_csr_rank(ukeys, m, bounds[2 * i + 1]);
    uint64_t s = 0;
    if (a != b) s = (uint64_t)(b ? pre[b - 1] : 0) - (uint64_t)(a ? pre[a - 1] : 0);
    out[2 * i] = b - a;
    out[2 * i + 1] = (int64_t)s;
  }
}
