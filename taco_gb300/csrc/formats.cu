// Operand formats beside CSR on the SpMV/SpMM path: DCSR ({Sparse,Sparse}: only the nonempty
// rows are stored), CSC ({Dense,Sparse} with mode ordering {1,0}), sparse vectors ({Sparse}),
// and the sparse SpMV result whose pattern is a DCSR matrix's rows.  taco's tests:
// test/tests-expr_storage.cpp:873-937 (spmv with B {Dense,Sparse} / {Sparse,Sparse}, c
// {Dense} / {Sparse}, a {Dense} / {Sparse}), tests-scheduling-eval.cpp:1309-1358 (spmmDCSRGPU,
// scheduleSpMMNZRowsGPU at :358-370) and :655-662 (DCSR / CSC operands of SpGEMM).
//
// Each format reaches the merge-tile kernels without a new inner loop: a DCSR matrix is a CSR
// matrix over its n0 stored rows (pos, crd, vals as they are), whose results go to rows crd0 —
// scattered into a zero-filled dense result, or kept as the values of the sparse result (its
// pattern is crd0).  A CSC matrix is transposed to CSR on the GPU by the COO pack (stable radix
// sort of (row, column) keys; columns come out ascending in each row).  A sparse vector is
// scattered into a zero-filled dense one: the products it drops are exact zeros.  For SpGEMM a
// DCSR (or DCSC) operand's pointer array is expanded to every row (or column) and a CSC one
// transposed, so that the CSR x CSR kernels take every combination of taco's spgemm test.
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace tacogb {

namespace {

// out[dest[e]] = y[e] for e < n (out zero-filled by the caller).
template <class V>
__global__ void fmt_scatter(const int32_t* __restrict__ dest, const V* __restrict__ y, int32_t n,
                            V* __restrict__ out) {
  const int32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) out[dest[e]] = y[e];
}

// Row dest[e] of out (N values) = row e of Y.
template <class V>
__global__ void fmt_scatter_rows(const int32_t* __restrict__ dest, const V* __restrict__ Y,
                                 int32_t n, int32_t N, V* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * N) return;
  const int64_t e = idx / N;
  out[(int64_t)dest[e] * N + (idx - e * N)] = Y[idx];
}

// The column of every nonzero of a CSC matrix: the last column c with colpos[c] <= p.
__global__ void fmt_expand_cols(const int32_t* __restrict__ colpos, int32_t cols, int64_t nnz,
                                int32_t* __restrict__ colidx) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nnz) return;
  int lo = 0, hi = cols - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(colpos + mid) <= p)
      lo = mid;
    else
      hi = mid - 1;
  }
  colidx[p] = lo;
}

// Full pointer array of a doubly compressed level: pos[i] = pos1[e] with e the number of stored
// outer coordinates crd0 below i (binary search), for i in [0, outer]; rows (or columns) that
// are not stored get empty ranges.
__global__ void fmt_expand_pos(const int32_t* __restrict__ crd0, const int32_t* __restrict__ pos1,
                               int32_t n0, int32_t outer, int32_t* __restrict__ pos) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > outer) return;
  int lo = 0, hi = n0;  // first e with crd0[e] >= i
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(crd0 + mid) < i)
      lo = mid + 1;
    else
      hi = mid;
  }
  pos[i] = __ldg(pos1 + lo);
}

unsigned blocks_for(int64_t n) { return (unsigned)((n + 255) / 256); }
size_t vbytes(int vt) { return vt == TACOGB_F64 ? 8 : 4; }

int check_dcsr(const tacogb_dcsr* A, const char* what) {
  TACOGB_CHECK_ARG(A != nullptr, "%s: null matrix", what);
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->n0 >= 0 && A->nnz >= 0 && A->n0 <= A->rows,
                   "%s: bad sizes", what);
  TACOGB_CHECK_ARG(A->nnz <= INT32_MAX, "%s: nnz exceeds int32 positions", what);
  TACOGB_CHECK_ARG(A->n0 == 0 || (A->crd0 != nullptr && A->pos != nullptr),
                   "%s: null row list or pos", what);
  TACOGB_CHECK_ARG(A->nnz == 0 || (A->crd != nullptr && A->vals != nullptr),
                   "%s: null crd or values", what);
  TACOGB_CHECK_ARG(A->vtype == TACOGB_F64 || A->vtype == TACOGB_F32,
                   "%s: unsupported value type %d", what, A->vtype);
  return 0;
}

tacogb_csr stored_rows(const tacogb_dcsr* A) {
  return tacogb_csr{A->n0, A->cols, A->nnz, A->pos, A->crd, A->vals, A->vtype};
}

}  // namespace

int spmv_dcsr_run(const tacogb_dcsr* A, const void* x, void* y, bool dense, cudaStream_t st) {
  if (int rc = check_dcsr(A, "DCSR SpMV")) return rc;
  TACOGB_CHECK_ARG(A->nnz == 0 || x != nullptr, "DCSR SpMV: null x");
  const size_t vb = vbytes(A->vtype);
  const tacogb_csr c = stored_rows(A);
  if (!dense) {  // the values of the sparse result, whose coordinates are crd0
    TACOGB_CHECK_ARG(A->n0 == 0 || y != nullptr, "DCSR SpMV: null result");
    return A->n0 ? spmv_run(&c, x, y, TACOGB_VARIANT_AUTO, st) : 0;
  }
  TACOGB_CHECK_ARG(A->rows == 0 || y != nullptr, "DCSR SpMV: null result");
  if (A->rows) TACOGB_CUDA_TRY(cudaMemsetAsync(y, 0, (size_t)A->rows * vb, st));
  if (A->n0 == 0) return 0;
  void* yc = scratch(((size_t)A->n0 * vb + 255) & ~(size_t)255, 8);
  if (!yc) return last_code();
  if (int rc = spmv_run(&c, x, yc, TACOGB_VARIANT_AUTO, st)) return rc;
  if (A->vtype == TACOGB_F64)
    TACOGB_LAUNCH("fmt_scatter", st,
                  (fmt_scatter<double><<<blocks_for(A->n0), 256, 0, st>>>(
                      A->crd0, (const double*)yc, A->n0, (double*)y)));
  else
    TACOGB_LAUNCH("fmt_scatter", st,
                  (fmt_scatter<float><<<blocks_for(A->n0), 256, 0, st>>>(
                      A->crd0, (const float*)yc, A->n0, (float*)y)));
  return 0;
}

int spmm_dcsr_run(const tacogb_dcsr* A, int32_t N, const void* B, void* C, cudaStream_t st) {
  if (int rc = check_dcsr(A, "DCSR SpMM")) return rc;
  TACOGB_CHECK_ARG(N >= 0, "DCSR SpMM: negative N");
  TACOGB_CHECK_ARG((int64_t)A->rows * N == 0 || C != nullptr, "DCSR SpMM: null C");
  const size_t vb = vbytes(A->vtype);
  if ((int64_t)A->rows * N)
    TACOGB_CUDA_TRY(cudaMemsetAsync(C, 0, (size_t)A->rows * N * vb, st));
  if ((int64_t)A->n0 * N == 0) return 0;
  void* Yc = scratch(((size_t)A->n0 * N * vb + 255) & ~(size_t)255, 8);
  if (!Yc) return last_code();
  const tacogb_csr c = stored_rows(A);
  if (int rc = spmm_run(&c, N, B, A->vtype, Yc, TACOGB_VARIANT_AUTO, st)) return rc;
  const int64_t n = (int64_t)A->n0 * N;
  if (A->vtype == TACOGB_F64)
    TACOGB_LAUNCH("fmt_scatter_rows", st,
                  (fmt_scatter_rows<double><<<blocks_for(n), 256, 0, st>>>(
                      A->crd0, (const double*)Yc, A->n0, N, (double*)C)));
  else
    TACOGB_LAUNCH("fmt_scatter_rows", st,
                  (fmt_scatter_rows<float><<<blocks_for(n), 256, 0, st>>>(
                      A->crd0, (const float*)Yc, A->n0, N, (float*)C)));
  return 0;
}

int densify_run(int32_t n, int64_t k, const int32_t* idx, const void* vals, int32_t vtype,
                void* out, cudaStream_t st) {
  TACOGB_CHECK_ARG(n >= 0 && k >= 0 && k <= n, "densify: bad sizes");
  TACOGB_CHECK_ARG(vtype == TACOGB_F64 || vtype == TACOGB_F32, "densify: bad value type");
  TACOGB_CHECK_ARG(n == 0 || out != nullptr, "densify: null output");
  TACOGB_CHECK_ARG(k == 0 || (idx != nullptr && vals != nullptr), "densify: null input");
  if (n) TACOGB_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)n * vbytes(vtype), st));
  if (k == 0) return 0;
  if (vtype == TACOGB_F64)
    TACOGB_LAUNCH("fmt_scatter", st,
                  (fmt_scatter<double><<<blocks_for(k), 256, 0, st>>>(
                      idx, (const double*)vals, (int32_t)k, (double*)out)));
  else
    TACOGB_LAUNCH("fmt_scatter", st,
                  (fmt_scatter<float><<<blocks_for(k), 256, 0, st>>>(
                      idx, (const float*)vals, (int32_t)k, (float*)out)));
  return 0;
}

int csc_to_csr_run(int32_t rows, int32_t cols, int64_t nnz, const int32_t* colpos,
                   const int32_t* rowidx, const void* vals, int32_t vtype, int32_t* pos,
                   int32_t* crd, void* out_vals, cudaStream_t st) {
  TACOGB_CHECK_ARG(rows >= 0 && cols >= 0 && nnz >= 0 && nnz <= INT32_MAX, "CSC: bad sizes");
  TACOGB_CHECK_ARG(cols == 0 || colpos != nullptr, "CSC: null column pos");
  TACOGB_CHECK_ARG(nnz == 0 || (rowidx != nullptr && vals != nullptr), "CSC: null rows or values");
  int32_t* colidx = (int32_t*)scratch(((size_t)nnz * 4 + 255) & ~(size_t)255, 9);
  if (!colidx) return last_code();
  if (nnz)
    TACOGB_LAUNCH("fmt_expand_cols", st,
                  (fmt_expand_cols<<<blocks_for(nnz), 256, 0, st>>>(colpos, cols, nnz, colidx)));
  int64_t out_nnz = 0;
  if (int rc = pack_csr(rows, cols, nnz, rowidx, colidx, vals, vtype, pos, crd, out_vals,
                        &out_nnz, st))
    return rc;
  TACOGB_CHECK_ARG(out_nnz == nnz, "CSC: repeated coordinates (%lld of %lld distinct)",
                   (long long)out_nnz, (long long)nnz);
  return 0;
}

int expand_pos_run(const int32_t* crd0, const int32_t* pos1, int32_t n0, int32_t outer,
                   int32_t* pos, cudaStream_t st) {
  TACOGB_CHECK_ARG(n0 >= 0 && outer >= 0 && n0 <= outer, "expand: bad sizes");
  TACOGB_CHECK_ARG(pos != nullptr && pos1 != nullptr && (n0 == 0 || crd0 != nullptr),
                   "expand: null array");
  TACOGB_LAUNCH("fmt_expand_pos", st,
                (fmt_expand_pos<<<blocks_for((int64_t)outer + 1), 256, 0, st>>>(crd0, pos1, n0,
                                                                                outer, pos)));
  return 0;
}

int spmv_csc_run(const tacogb_csr* Acsc, const void* x, void* y, cudaStream_t st) {
  TACOGB_CHECK_ARG(Acsc != nullptr, "CSC SpMV: null matrix");
  const int32_t rows = Acsc->rows, cols = Acsc->cols;
  const int64_t nnz = Acsc->nnz;
  const size_t vb = vbytes(Acsc->vtype);
  const size_t a = (((size_t)rows + 1) * 4 + 255) & ~(size_t)255;
  const size_t b = ((size_t)nnz * 4 + 255) & ~(size_t)255;
  unsigned char* ws = (unsigned char*)scratch(a + b + (size_t)nnz * vb, 10);
  if (!ws) return last_code();
  int32_t* pos = (int32_t*)ws;
  int32_t* crd = (int32_t*)(ws + a);
  void* v = ws + a + b;
  if (int rc = csc_to_csr_run(rows, cols, nnz, Acsc->pos, Acsc->crd, Acsc->vals, Acsc->vtype, pos,
                              crd, v, st))
    return rc;
  const tacogb_csr c{rows, cols, nnz, pos, crd, v, Acsc->vtype};
  return spmv_run(&c, x, y, TACOGB_VARIANT_AUTO, st);
}

}  // namespace tacogb
