/* ORACLE — test infrastructure only.  Nothing in the taco_gb300 product links or calls this
 * file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and only
 * as the checker (or as the timed CPU port).
 *
 * A plain-C restatement of the code taco generates for the three hot-path statements, each
 * function following the loop nest taco's lowering emits:
 *
 *   SpMV   y(i) = A(i,j) * x(j), A {Dense,Sparse}
 *          generated `compute`: a row loop (src/lower/lowerer_impl_imperative.cpp:1304,
 *          lowerForallPosition over A2_pos/A2_crd), the reduction scalar `tjy_val` introduced by
 *          scalarPromote (src/index_notation/transformations.cpp:1982), and the OpenMP pragma
 *          emitted for the outer loop (src/codegen/codegen_c.cpp:393-446).
 *   SpMM   C(i,k) = A(i,j) * B(j,k), B and C dense row-major
 *          generated `compute`: zero C, then for i, for p in row i, for k: C[i*N+k] += A[p]*B[j*N+k]
 *          (same lowering, dense k loop; flat int32 index i*N+k as the generated code uses).
 *   SpGEMM C(i,k) = A(i,j) * B(j,k), all CSR
 *          workspace form forall(i, where(forall(k, C(i,k)=w(k)), forall(j,k, w(k) += A*B))) made by
 *          insertTemporaries (src/index_notation/transformations.cpp:2083); the dense accelerator
 *          arrays w_already_set/w_index_list (src/lower/lowerer_impl_imperative.cpp:2197), the
 *          per-row qsort of the index list, and compressed appends
 *          (src/lower/mode_format_compressed.cpp:107-213).  `assemble` builds pos/crd; `compute`
 *          fills vals, initialising w[k] with the first product and adding later products in
 *          A-row order.
 *
 * The SpGEMM functions are also given in a row-parallel two-pass form (per-row counts, scan,
 * fill), the shape taco's scheduleSpGEMMCPU produces through lowerAssemble
 * (test/tests-scheduling-eval.cpp:68-94, src/lower/lowerer_impl_imperative.cpp:2616-2781); its
 * output is identical to the serial form.
 *
 *   pack   COO coordinates -> CSR, as TensorBase::pack does for a {Dense,Sparse} tensor
 *          (src/tensor.cpp:295-463): sort the coordinates lexicographically (taco: qsort with
 *          lexicographicalCmp, :253-261 and :420-422), then merge runs of equal coordinates
 *          into one entry whose value is their sum (the generated pack over the COO buffer,
 *          :935-1020; duplicates sum, tests-tensor.cpp:68-79).  taco's qsort is not stable;
 *          this restatement breaks ties by input position, so duplicates sum in input order.
 *
 *   SDDMM  A(i,k) = B(i,k) * C(i,j) * D(j,k), B {Dense,Sparse}, A, C, D dense row-major
 *          generated `compute` (taco's CLI, -f=A:dd -f=B:ds -f=C:dd -f=D:dd): zero A, then for
 *          i, for j, for p in row i: A[i*K+k] += (B[p]*C[i*J+j]) * D[j*K+k] (the statement of
 *          test/tests-scheduling-eval.cpp:783-840 and 1360-1417).
 *
 *   TTV    A(i,j) = B(i,j,k) * c(k);  TTM  A(i,j,l) = B(i,j,k) * C(k,l);
 *   MTTKRP A(i,j) = B(i,k,l) * C(k,j) * D(l,j);  B {Sparse,Sparse,Sparse}, the rest dense
 *          generated `compute` of each (taco's CLI, -f=B:sss): zero A, then walk B's three
 *          levels; TTV sums a fiber into a scalar and stores it; TTM adds B*C(k,:) into
 *          A(i,j,:); MTTKRP adds (B*C(k,j))*D(l,j) over j for every nonzero.
 *
 * Compiled with -O2 -fopenmp -ffp-contract=off: products and sums are rounded separately, in
 * the written order.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

int oracle_num_threads(void) { return omp_get_max_threads(); }
void oracle_set_num_threads(int n) { omp_set_num_threads(n); }

/* y(i) = A(i,j) * x(j) */
void oracle_spmv_f64(int32_t rows, const int32_t* pos, const int32_t* crd, const double* vals,
                     const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < rows; i++) {
    double t = 0.0;
    for (int32_t p = pos[i]; p < pos[i + 1]; p++) t += vals[p] * x[crd[p]];
    y[i] = t;
  }
}

/* C(i,k) = A(i,j) * B(j,k), B: rowsB x N row-major, C: rows x N row-major */
void oracle_spmm_f64(int32_t rows, int32_t N, const int32_t* pos, const int32_t* crd,
                     const double* vals, const double* B, double* C) {
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)rows * N; q++) C[q] = 0.0;
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < rows; i++) {
    double* c = C + (int64_t)i * N;
    for (int32_t p = pos[i]; p < pos[i + 1]; p++) {
      const double a = vals[p];
      const double* b = B + (int64_t)crd[p] * N;
      for (int32_t k = 0; k < N; k++) c[k] = c[k] + a * b[k];
    }
  }
}

static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* Row i's sorted distinct output columns into list; returns the count.  `set` is all-zero on
 * entry and on exit. */
static int32_t spgemm_row_cols(int32_t i, const int32_t* Apos, const int32_t* Acrd,
                               const int32_t* Bpos, const int32_t* Bcrd, char* set,
                               int32_t* list) {
  int32_t cnt = 0;
  for (int32_t p = Apos[i]; p < Apos[i + 1]; p++) {
    int32_t j = Acrd[p];
    for (int32_t q = Bpos[j]; q < Bpos[j + 1]; q++) {
      int32_t k = Bcrd[q];
      if (!set[k]) { set[k] = 1; list[cnt++] = k; }
    }
  }
  qsort(list, (size_t)cnt, sizeof(int32_t), cmp_i32);
  for (int32_t t = 0; t < cnt; t++) set[list[t]] = 0;
  return cnt;
}

/* Symbolic phase.  Writes Cpos[0..rows]; returns nnz(C) and a malloc'd crd in *Ccrd_out, or
 * -1 when nnz(C) exceeds int32. */
int64_t oracle_spgemm_assemble(int32_t rows, int32_t K, const int32_t* Apos, const int32_t* Acrd,
                               const int32_t* Bpos, const int32_t* Bcrd, int32_t* Cpos,
                               int32_t** Ccrd_out) {
  int32_t* cnt = (int32_t*)malloc(sizeof(int32_t) * ((size_t)rows + 1));
#pragma omp parallel
  {
    char* set = (char*)calloc((size_t)K, 1);
    int32_t* list = (int32_t*)malloc(sizeof(int32_t) * (size_t)(K > 0 ? K : 1));
#pragma omp for schedule(dynamic, 64)
    for (int32_t i = 0; i < rows; i++) cnt[i] = spgemm_row_cols(i, Apos, Acrd, Bpos, Bcrd, set, list);
    free(set);
    free(list);
  }
  int64_t acc = 0;
  Cpos[0] = 0;
  for (int32_t i = 0; i < rows; i++) {
    acc += cnt[i];
    if (acc > INT32_MAX) { free(cnt); *Ccrd_out = NULL; return -1; }
    Cpos[i + 1] = (int32_t)acc;
  }
  free(cnt);
  int32_t* Ccrd = (int32_t*)malloc(sizeof(int32_t) * (size_t)(acc > 0 ? acc : 1));
#pragma omp parallel
  {
    char* set = (char*)calloc((size_t)K, 1);
#pragma omp for schedule(dynamic, 64)
    for (int32_t i = 0; i < rows; i++) spgemm_row_cols(i, Apos, Acrd, Bpos, Bcrd, set, Ccrd + Cpos[i]);
    free(set);
  }
  *Ccrd_out = Ccrd;
  return acc;
}

/* Numeric phase over the pattern from oracle_spgemm_assemble. */
void oracle_spgemm_compute(int32_t rows, int32_t K, const int32_t* Apos, const int32_t* Acrd,
                           const double* Avals, const int32_t* Bpos, const int32_t* Bcrd,
                           const double* Bvals, const int32_t* Cpos, const int32_t* Ccrd,
                           double* Cvals) {
#pragma omp parallel
  {
    char* set = (char*)calloc((size_t)K, 1);
    double* w = (double*)malloc(sizeof(double) * (size_t)(K > 0 ? K : 1));
#pragma omp for schedule(dynamic, 64)
    for (int32_t i = 0; i < rows; i++) {
      for (int32_t p = Apos[i]; p < Apos[i + 1]; p++) {
        int32_t j = Acrd[p];
        for (int32_t q = Bpos[j]; q < Bpos[j + 1]; q++) {
          int32_t k = Bcrd[q];
          double prod = Avals[p] * Bvals[q];
          if (!set[k]) { set[k] = 1; w[k] = prod; }
          else w[k] = w[k] + prod;
        }
      }
      for (int32_t t = Cpos[i]; t < Cpos[i + 1]; t++) { Cvals[t] = w[Ccrd[t]]; set[Ccrd[t]] = 0; }
    }
    free(set);
    free(w);
  }
}

/* pack: (row, col, input position) records sorted lexicographically */
typedef struct {
  int32_t r, c;
  int64_t k;
} PackRec;

static int cmp_pack(const void* a, const void* b) {
  const PackRec* x = (const PackRec*)a;
  const PackRec* y = (const PackRec*)b;
  if (x->r != y->r) return x->r < y->r ? -1 : 1;
  if (x->c != y->c) return x->c < y->c ? -1 : 1;
  return x->k < y->k ? -1 : (x->k > y->k);
}

/* COO -> CSR with duplicates summed in input order; pos has rows + 1 entries, crd and out have
 * room for n.  Returns nnz, or -1 when a coordinate is outside the matrix. */
int64_t oracle_pack_csr(int32_t rows, int32_t cols, int64_t n, const int32_t* ri,
                        const int32_t* ci, const double* v, int32_t* pos, int32_t* crd,
                        double* out) {
  PackRec* rec = (PackRec*)malloc((size_t)(n > 0 ? n : 1) * sizeof(PackRec));
  for (int64_t i = 0; i < n; i++) {
    if (ri[i] < 0 || ri[i] >= rows || ci[i] < 0 || ci[i] >= cols) {
      free(rec);
      return -1;
    }
    rec[i].r = ri[i];
    rec[i].c = ci[i];
    rec[i].k = i;
  }
  qsort(rec, (size_t)n, sizeof(PackRec), cmp_pack);
  int64_t m = 0;
  int32_t row = 0;
  pos[0] = 0;
  for (int64_t i = 0; i < n;) {
    const int32_t r = rec[i].r, c = rec[i].c;
    double sum = v[rec[i].k];
    int64_t j = i + 1;
    for (; j < n && rec[j].r == r && rec[j].c == c; j++) sum = sum + v[rec[j].k];
    while (row < r) pos[++row] = (int32_t)m;
    crd[m] = c;
    out[m] = sum;
    m++;
    i = j;
  }
  while (row < rows) pos[++row] = (int32_t)m;
  free(rec);
  return m;
}

void oracle_free(void* p) { free(p); }

/* A(i,k) = B(i,k) * C(i,j) * D(j,k): B CSR (I x K), C I x J and D J x K dense row-major.
 * taco's tests use a dense I x K result (test/tests-scheduling-eval.cpp:783-840, 1360-1417);
 * its default lowering of that statement zero-fills A, then for each row i, for each j, runs
 * over row i's nonzeros k adding the term (B*C)*D into A(i,k), so each result sums its J terms
 * in j order.  oracle_sddmm_f64 restates that loop; oracle_sddmm_sampled_f64 is the same loop
 * with the result kept at B's nonzeros (out[p] for nonzero p) instead of a dense I x K array,
 * for sizes where the dense result cannot be held. */
void oracle_sddmm_f64(int32_t I, int32_t K, int32_t J, const int32_t* pos, const int32_t* crd,
                      const double* bv, const double* C, const double* D, double* A) {
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)I * K; q++) A[q] = 0.0;
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < I; i++) {
    double* a = A + (int64_t)i * K;
    for (int32_t j = 0; j < J; j++) {
      const double c = C[(int64_t)i * J + j];
      const double* d = D + (int64_t)j * K;
      for (int32_t p = pos[i]; p < pos[i + 1]; p++) {
        const int32_t k = crd[p];
        a[k] = a[k] + (bv[p] * c) * d[k];
      }
    }
  }
}

void oracle_sddmm_sampled_f64(int32_t I, int32_t K, int32_t J, const int32_t* pos,
                              const int32_t* crd, const double* bv, const double* C,
                              const double* D, double* out) {
  (void)K;
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < I; i++) {
    for (int32_t p = pos[i]; p < pos[i + 1]; p++) out[p] = 0.0;
    for (int32_t j = 0; j < J; j++) {
      const double c = C[(int64_t)i * J + j];
      const double* d = D + (int64_t)j * K;
      for (int32_t p = pos[i]; p < pos[i + 1]; p++) out[p] = out[p] + (bv[p] * c) * d[crd[p]];
    }
  }
}

/* Order-3 kernels over B in taco's {Sparse,Sparse,Sparse} format (CSF): level 0 holds the n0
 * distinct i (crd0; taco's pos0 is {0, n0}); level 1 pos1 (n0 + 1) and crd1 (one entry per
 * (i, j) fiber); level 2 pos2 (fibers + 1), crd2 and vals per nonzero.  Results are dense
 * row-major, as in taco's tests (test/tests-scheduling-eval.cpp:993-1043 ttvCPU, 1094-1146
 * ttmCPU, 1148-1206 mttkrpCPU; GPU forms :1420-1580).  Each function restates the loop taco's
 * default lowering emits for the statement (taco's CLI, -f=B:sss, dense A, C, D, c). */

/* A(i,j) = B(i,j,k) * c(k): per fiber a running sum over k, stored (not added) into A(i,j). */
void oracle_ttv_f64(int32_t I, int32_t J, int32_t n0, const int32_t* crd0, const int32_t* pos1,
                    const int32_t* crd1, const int32_t* pos2, const int32_t* crd2,
                    const double* bv, const double* c, double* A) {
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)I * J; q++) A[q] = 0.0;
#pragma omp parallel for schedule(static)
  for (int32_t e = 0; e < n0; e++) {
    const int32_t i = crd0[e];
    for (int32_t f = pos1[e]; f < pos1[e + 1]; f++) {
      double t = 0.0;
      for (int32_t p = pos2[f]; p < pos2[f + 1]; p++) t += bv[p] * c[crd2[p]];
      A[(int64_t)i * J + crd1[f]] = t;
    }
  }
}

/* A(i,j,l) = B(i,j,k) * C(k,l): for each nonzero, the row C(k,:) scaled by B added into A(i,j,:). */
void oracle_ttm_f64(int32_t I, int32_t J, int32_t L, int32_t n0, const int32_t* crd0,
                    const int32_t* pos1, const int32_t* crd1, const int32_t* pos2,
                    const int32_t* crd2, const double* bv, const double* C, double* A) {
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)I * J * L; q++) A[q] = 0.0;
#pragma omp parallel for schedule(static)
  for (int32_t e = 0; e < n0; e++) {
    const int32_t i = crd0[e];
    for (int32_t f = pos1[e]; f < pos1[e + 1]; f++) {
      double* a = A + ((int64_t)i * J + crd1[f]) * L;
      for (int32_t p = pos2[f]; p < pos2[f + 1]; p++) {
        const double b = bv[p];
        const double* cr = C + (int64_t)crd2[p] * L;
        for (int32_t l = 0; l < L; l++) a[l] = a[l] + b * cr[l];
      }
    }
  }
}

/* A(i,j) = B(i,k,l) * C(k,j) * D(l,j): for each nonzero (i,k,l), for each j,
 * A(i,j) += (B * C(k,j)) * D(l,j). */
void oracle_mttkrp_f64(int32_t I, int32_t J, int32_t n0, const int32_t* crd0,
                       const int32_t* pos1, const int32_t* crd1, const int32_t* pos2,
                       const int32_t* crd2, const double* bv, const double* C, const double* D,
                       double* A) {
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < (int64_t)I * J; q++) A[q] = 0.0;
#pragma omp parallel for schedule(static)
  for (int32_t e = 0; e < n0; e++) {
    double* a = A + (int64_t)crd0[e] * J;
    for (int32_t f = pos1[e]; f < pos1[e + 1]; f++) {
      const double* cr = C + (int64_t)crd1[f] * J;
      for (int32_t p = pos2[f]; p < pos2[f + 1]; p++) {
        const double b = bv[p];
        const double* dr = D + (int64_t)crd2[p] * J;
        for (int32_t j = 0; j < J; j++) a[j] = a[j] + (b * cr[j]) * dr[j];
      }
    }
  }
}

/* TTM with the result kept per (i,j) fiber (out[f * L + l]), the loop of oracle_ttm_f64 without
 * the dense I x J x L array, for sizes where that array cannot be held. */
void oracle_ttm_fibers_f64(int32_t L, int32_t nfib, const int32_t* pos2, const int32_t* crd2,
                           const double* bv, const double* C, double* out) {
#pragma omp parallel for schedule(static)
  for (int32_t f = 0; f < nfib; f++) {
    double* o = out + (int64_t)f * L;
    for (int32_t l = 0; l < L; l++) o[l] = 0.0;
    for (int32_t p = pos2[f]; p < pos2[f + 1]; p++) {
      const double b = bv[p];
      const double* cr = C + (int64_t)crd2[p] * L;
      for (int32_t l = 0; l < L; l++) o[l] = o[l] + b * cr[l];
    }
  }
}
