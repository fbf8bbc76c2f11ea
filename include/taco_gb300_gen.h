/* Deterministic synthetic CSR generators (host code, C ABI).
 *
 * Not part of taco's interface: taco fills tensors with insert()/pack() from user data
 * (src/tensor.cpp:295-463).  These generators produce the synthetic matrices the library is
 * tested and measured on, directly as CSR arrays (int32 pos/crd, FP64 values), so that
 * multi-gigabyte inputs need no COO sort.
 */
#ifndef TACO_GB300_GEN_H
#define TACO_GB300_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TACOGB_GEN_UNIFORM = 0,   /* row length uniform on [len_lo, len_hi] */
  TACOGB_GEN_POWERLAW = 1,  /* L = min(len_max, max(1, round(c*K))), K ~ Zipf(2), E[L] = mean */
  TACOGB_GEN_BANDED = 2,    /* min(band_len, window) columns from [i-band, i+band) */
  TACOGB_GEN_POISSON2D = 3  /* 5-point Laplacian on a grid x grid mesh */
};

typedef struct tacogb_gen_spec {
  int32_t rows, cols, kind;
  int32_t len_lo, len_hi;   /* uniform */
  double mean;              /* power-law target mean row length */
  int32_t len_max;          /* power-law clip (and Zipf support) */
  int32_t band, band_len;   /* banded half-width and row length */
  int32_t grid;             /* poisson grid side (rows = grid*grid) */
  uint64_t seed;
} tacogb_gen_spec;

/* Writes pos[0..rows] and returns nnz, or -1 if nnz would not fit an int32 position. */
int64_t tacogb_gen_pos(const tacogb_gen_spec* spec, int32_t* pos);
/* Fills crd (sorted distinct columns per row) and vals (U(-1,1)); either may be NULL. */
int tacogb_gen_fill(const tacogb_gen_spec* spec, const int32_t* pos, int32_t* crd, double* vals);
/* count U(-1,1) doubles. */
void tacogb_gen_dense(uint64_t seed, int64_t count, double* out);
/* Power-law scale c with E[min(kmax, max(1, round(c*K)))] = mean, K ~ Zipf(2) on [1, kmax]. */
double tacogb_gen_powerlaw_scale(double mean, int32_t kmax);
/* Spec of matrix m of a batched collection (rows log-uniform in [rows_lo, rows_hi]). */
void tacogb_gen_batch_spec(uint64_t seed, int32_t m, int32_t rows_lo, int32_t rows_hi,
                           tacogb_gen_spec* out);

#ifdef __cplusplus
}
#endif
#endif
