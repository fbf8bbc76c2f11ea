/* Deterministic synthetic CSR generators for the sparse workloads this library is measured on.
 *
 * Every random draw comes from a counter-based SplitMix64 stream keyed by (seed, stream, row),
 * so a matrix is a pure function of its spec: identical on every machine, thread count and
 * call order.  Host code only (OpenMP over rows); the same bytes feed the oracle in the tests
 * and the device buffers in the benchmark.
 *
 * Structures (the row-length law and the column law are independent):
 *   TACOGB_GEN_UNIFORM   row length uniform on [len_lo, len_hi], columns uniform over [0, cols)
 *   TACOGB_GEN_POWERLAW  row length L = min(max, max(1, round(c*K))), K ~ Zipf(2) on [1, max],
 *                        c solved by bisection so that E[L] = mean; columns uniform
 *   TACOGB_GEN_BANDED    min(band_len, window) distinct columns from the window [i-band, i+band)
 *                        clipped to the matrix (bandwidth 2*band)
 *   TACOGB_GEN_POISSON2D 5-point Laplacian on a g x g grid (diag 4, off-diagonal -1)
 * Columns of a row are distinct and sorted ascending (CSR {Dense,Sparse} as taco packs it,
 * src/format.cpp:403).  Values are U(-1,1) drawn as 2*u53-1.
 *
 * Build with -ffp-contract=off: the calibration below must give the same bits everywhere.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "taco_gb300_gen.h"

#define GOLDEN 0x9E3779B97F4A7C15ull

static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

typedef struct { uint64_t s; } rng_t;

static inline rng_t rng_make(uint64_t seed, uint64_t stream, uint64_t row) {
  rng_t r;
  r.s = mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ull + 1) ^ mix64(row + 0x632BE59BD9B4E019ull));
  return r;
}

static inline uint64_t rng_next(rng_t* r) { r->s += GOLDEN; return mix64(r->s); }

/* uniform integer in [0, m), m < 2^32 */
static inline uint32_t rng_below(rng_t* r, uint32_t m) {
  return (uint32_t)(((rng_next(r) >> 32) * (uint64_t)m) >> 32);
}

/* uniform double in [0, 1) with 53 random bits */
static inline double rng_u53(rng_t* r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

enum { STREAM_LEN = 1, STREAM_COL = 2, STREAM_VAL = 3, STREAM_DENSE = 4 };

/* ---------------------------------------------------------------- power-law calibration --- */

/* cdf[k-1] = P(K <= k) for K ~ Zipf(2) truncated to [1, kmax] */
static double* zipf2_cdf(int32_t kmax) {
  double* cdf = (double*)malloc(sizeof(double) * (size_t)kmax);
  double h = 0.0;
  for (int32_t k = 1; k <= kmax; k++) { h += 1.0 / ((double)k * (double)k); cdf[k - 1] = h; }
  for (int32_t k = 0; k < kmax; k++) cdf[k] /= h;
  cdf[kmax - 1] = 1.0;
  return cdf;
}

static inline int32_t powerlaw_len(double c, int32_t k, int32_t kmax) {
  double l = floor(c * (double)k + 0.5);
  if (l < 1.0) l = 1.0;
  if (l > (double)kmax) l = (double)kmax;
  return (int32_t)l;
}

static double powerlaw_mean(const double* cdf, int32_t kmax, double c) {
  double m = 0.0, prev = 0.0;
  for (int32_t k = 1; k <= kmax; k++) {
    double p = cdf[k - 1] - prev;
    prev = cdf[k - 1];
    m += p * (double)powerlaw_len(c, k, kmax);
  }
  return m;
}

double tacogb_gen_powerlaw_scale(double mean, int32_t kmax) {
  double* cdf = zipf2_cdf(kmax);
  double lo = 0.0, hi = (double)kmax;
  for (int it = 0; it < 200; it++) {
    double mid = 0.5 * (lo + hi);
    if (powerlaw_mean(cdf, kmax, mid) < mean) lo = mid; else hi = mid;
  }
  free(cdf);
  return 0.5 * (lo + hi);
}

/* ------------------------------------------------------------------------- row lengths --- */

static int32_t band_window(const tacogb_gen_spec* s, int32_t i, int32_t* lo_out) {
  int64_t lo = (int64_t)i - s->band, hi = (int64_t)i + s->band; /* [lo, hi) */
  if (lo < 0) lo = 0;
  if (hi > s->cols) hi = s->cols;
  *lo_out = (int32_t)lo;
  return (int32_t)(hi - lo);
}

static int32_t row_length(const tacogb_gen_spec* s, int32_t i, const double* cdf, double c) {
  switch (s->kind) {
    case TACOGB_GEN_UNIFORM: {
      rng_t r = rng_make(s->seed, STREAM_LEN, (uint64_t)i);
      int32_t span = s->len_hi - s->len_lo + 1;
      int32_t l = s->len_lo + (int32_t)rng_below(&r, (uint32_t)span);
      return l > s->cols ? s->cols : l;
    }
    case TACOGB_GEN_POWERLAW: {
      rng_t r = rng_make(s->seed, STREAM_LEN, (uint64_t)i);
      double u = rng_u53(&r);
      int32_t lo = 0, hi = s->len_max - 1; /* first k with cdf >= u */
      while (lo < hi) { int32_t mid = (lo + hi) >> 1; if (cdf[mid] >= u) hi = mid; else lo = mid + 1; }
      int32_t l = powerlaw_len(c, lo + 1, s->len_max);
      return l > s->cols ? s->cols : l;
    }
    case TACOGB_GEN_BANDED: {
      int32_t lo;
      int32_t w = band_window(s, i, &lo);
      return w < s->band_len ? w : s->band_len;
    }
    case TACOGB_GEN_POISSON2D: {
      int32_t g = s->grid, gi = i / g, gj = i % g;
      return 1 + (gi > 0) + (gi < g - 1) + (gj > 0) + (gj < g - 1);
    }
  }
  return 0;
}

int64_t tacogb_gen_pos(const tacogb_gen_spec* s, int32_t* pos) {
  double* cdf = NULL;
  double c = 0.0;
  if (s->kind == TACOGB_GEN_POWERLAW) {
    cdf = zipf2_cdf(s->len_max);
    c = tacogb_gen_powerlaw_scale(s->mean, s->len_max);
  }
  int32_t n = s->rows;
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < n; i++) pos[i + 1] = row_length(s, i, cdf, c);
  pos[0] = 0;
  int64_t acc = 0;
  for (int32_t i = 0; i < n; i++) {
    acc += pos[i + 1];
    if (acc > INT32_MAX) { free(cdf); return -1; } /* taco's pos arrays are int32 */
    pos[i + 1] = (int32_t)acc;
  }
  free(cdf);
  return acc;
}

/* ---------------------------------------------------------------------------- columns --- */

static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

static void sort_i32(int32_t* v, int32_t n) {
  if (n <= 32) {
    for (int32_t a = 1; a < n; a++) {
      int32_t t = v[a], b = a - 1;
      while (b >= 0 && v[b] > t) { v[b + 1] = v[b]; b--; }
      v[b + 1] = t;
    }
  } else {
    qsort(v, (size_t)n, sizeof(int32_t), cmp_i32);
  }
}

/* L distinct sorted values uniform over [base, base+m): draw the missing count iid, sort,
 * drop repeats, repeat.  The kept set is exchangeable over the m values, so every L-subset is
 * equally likely. */
static void distinct_sorted(rng_t* r, int32_t base, int32_t m, int32_t L, int32_t* out) {
  if (L == m) { for (int32_t t = 0; t < L; t++) out[t] = base + t; return; }
  int32_t have = 0;
  while (have < L) {
    for (int32_t t = have; t < L; t++) out[t] = base + (int32_t)rng_below(r, (uint32_t)m);
    sort_i32(out, L);
    int32_t u = 0;
    for (int32_t t = 0; t < L; t++) if (u == 0 || out[t] != out[u - 1]) out[u++] = out[t];
    have = u;
  }
}

int tacogb_gen_fill(const tacogb_gen_spec* s, const int32_t* pos, int32_t* crd, double* vals) {
  int32_t n = s->rows;
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < n; i++) {
    int32_t p0 = pos[i], L = pos[i + 1] - pos[i];
    if (crd) {
      rng_t r = rng_make(s->seed, STREAM_COL, (uint64_t)i);
      switch (s->kind) {
        case TACOGB_GEN_UNIFORM:
        case TACOGB_GEN_POWERLAW:
          distinct_sorted(&r, 0, s->cols, L, crd + p0);
          break;
        case TACOGB_GEN_BANDED: {
          int32_t lo, w = band_window(s, i, &lo);
          distinct_sorted(&r, lo, w, L, crd + p0);
          break;
        }
        case TACOGB_GEN_POISSON2D: {
          int32_t g = s->grid, gi = i / g, gj = i % g, t = p0;
          if (gi > 0) crd[t++] = i - g;
          if (gj > 0) crd[t++] = i - 1;
          crd[t++] = i;
          if (gj < g - 1) crd[t++] = i + 1;
          if (gi < g - 1) crd[t++] = i + g;
          break;
        }
      }
    }
    if (vals) {
      if (s->kind == TACOGB_GEN_POISSON2D) {
        for (int32_t t = 0; t < L; t++) vals[p0 + t] = (crd[p0 + t] == i) ? 4.0 : -1.0;
      } else {
        rng_t r = rng_make(s->seed, STREAM_VAL, (uint64_t)i);
        for (int32_t t = 0; t < L; t++) vals[p0 + t] = 2.0 * rng_u53(&r) - 1.0;
      }
    }
  }
  return 0;
}

/* U(-1,1) dense values; element e of the array is drawn from stream (seed, e / 1024). */
void tacogb_gen_dense(uint64_t seed, int64_t count, double* out) {
  int64_t blocks = (count + 1023) / 1024;
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < blocks; b++) {
    rng_t r = rng_make(seed, STREAM_DENSE, (uint64_t)b);
    int64_t e1 = (b + 1) * 1024 < count ? (b + 1) * 1024 : count;
    for (int64_t e = b * 1024; e < e1; e++) out[e] = 2.0 * rng_u53(&r) - 1.0;
  }
}

/* ---------------------------------------------------------------- batched collections --- */

/* Matrix m of a batched collection: rows log-uniform in [rows_lo, rows_hi], square, mean
 * nnz/row drawn from {2,4,...,64}, structure uniform / power-law / banded by m mod 3. */
void tacogb_gen_batch_spec(uint64_t seed, int32_t m, int32_t rows_lo, int32_t rows_hi,
                           tacogb_gen_spec* out) {
  rng_t r = rng_make(seed, 7, (uint64_t)m);
  double u = rng_u53(&r);
  double lr = log((double)rows_lo) + u * (log((double)rows_hi) - log((double)rows_lo));
  int32_t n = (int32_t)floor(exp(lr) + 0.5);
  if (n < rows_lo) n = rows_lo;
  if (n > rows_hi) n = rows_hi;
  int32_t mean = 2 * (1 + (int32_t)rng_below(&r, 32)); /* {2,...,64} */
  memset(out, 0, sizeof(*out));
  out->rows = n;
  out->cols = n;
  out->seed = mix64(seed + 0x5EEDull * (uint64_t)(m + 1));
  out->mean = (double)mean;
  switch (m % 3) {
    case 0:
      out->kind = TACOGB_GEN_UNIFORM;
      out->len_lo = 1;
      out->len_hi = 2 * mean - 1;
      break;
    case 1:
      out->kind = TACOGB_GEN_POWERLAW;
      out->len_max = n < 20000 ? n : 20000;
      if (out->len_max < mean) out->len_max = mean;
      break;
    default:
      out->kind = TACOGB_GEN_BANDED;
      out->band = 16; /* bandwidth 32: window [i-16, i+16), so at most 32 nnz per row */
      out->band_len = mean < 32 ? mean : 32;
      break;
  }
}
