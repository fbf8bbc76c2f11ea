// Internal entry points shared between the translation units of libtacogb.
#pragma once

#include <cuda_runtime.h>
#include "taco_gb300.h"

namespace tacogb {

// SpMV (spmv.cu)
int spmv_variant_count();
const char* spmv_variant_name(int v);
int spmv_default_variant(const tacogb_csr* A);
// The variant TACOGB_VARIANT_AUTO runs for A (a cached per-matrix choice; may sync st once).
int spmv_auto_variant(const tacogb_csr* A, cudaStream_t st);
int spmv_run(const tacogb_csr* A, const void* x, void* y, int variant, cudaStream_t st);

// Merge-path tile boundaries (spmv.cu): part[0..tiles] = (rows ended, nonzeros consumed) at
// diagonals b*tile_items; rows shorter than snap_len are never split (0 = split anywhere).
int merge_partition(const int32_t* pos, int32_t n, int64_t nnz, int64_t tile_items,
                    int32_t tiles, int2* part, cudaStream_t st, int32_t snap_len = 0);

// SpMM (spmm.cu)
int spmm_variant_count();
const char* spmm_variant_name(int v);
int spmm_variant_index(const char* name);  // -1 when no variant has that name
// One split of an FP64 B (cols x N, N even, B and bdf 16-byte aligned; bdf holds cols*N
// double-float pairs) for several products over it, and the product of one CSR A over that
// split (the merge_w512_dfs tile; an entry of B outside the double-float range, recorded in
// *flag by the split, sends every tile to native FP64 over B).  Used by the pipelined taco-ABI
// SpMM, whose chunks share one B; products that may run at the same time on different streams
// take different scratch slots (the partition and carries live there).
bool spmm_presplit_applies(const void* B, int32_t N);
int spmm_split_once(const double* B, int32_t cols, int32_t N, void* bdf, int* flag,
                    cudaStream_t st);
int spmm_run_presplit(const tacogb_csr* A, int32_t N, const double* B, const void* bdf, int* flag,
                      double* C, cudaStream_t st, int scratch_slot = 1);
int spmm_run(const tacogb_csr* A, int32_t N, const void* B, int32_t btype, void* C, int variant,
             cudaStream_t st);

// SpGEMM (spgemm.cu)
int spgemm_symbolic(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos, int64_t* nnzC,
                    cudaStream_t st);
int spgemm_fill(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos, int32_t* Ccrd,
                cudaStream_t st);
// One pass (assemble while computing): pos of C and nnz(C) (synchronises); the columns and
// values wait in scratch until spgemm_onepass_finish moves them into C's arrays.
int spgemm_onepass(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos, int64_t* nnzC,
                   cudaStream_t st);
int spgemm_onepass_finish(const int32_t* Cpos, int32_t* Ccrd, void* Cvals, cudaStream_t st);
int spgemm_numeric(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos,
                   const int32_t* Ccrd, void* Cvals, cudaStream_t st);

// SDDMM (sddmm.cu): values of B .* (C * D) at B's nonzeros (out_ld == 0) or into a dense
// rows x cols result of row stride out_ld (zero-filled first).
int sddmm_variant_count();
const char* sddmm_variant_name(int v);
int sddmm_run(const tacogb_csr* B, int32_t J, const void* C, const void* D, void* out,
              int64_t out_ld, int variant, cudaStream_t st);
// The same product in two steps over one transposed D (J <= 512, the default variant, values at
// B's nonzeros): D transposed once into Dt (sddmm_pre_bytes of it), then any number of products
// of row blocks of B (with their rows of C) against it.  sddmm_pre_bytes is 0 for J outside
// (0, 512].
size_t sddmm_pre_bytes(int32_t J, int32_t K, int vtype);
int sddmm_pre_transpose(const void* D, int32_t J, int32_t K, int vtype, void* Dt, cudaStream_t st);
int sddmm_pre_run(const tacogb_csr* B, int32_t J, const void* C, const void* D, const void* Dt,
                  void* out, cudaStream_t st);

// Order-3 kernels (tensor3.cu); dense selects taco's dense result form.
int ttv_run(const tacogb_csf3* B, const void* c, void* out, bool dense, int variant,
            cudaStream_t st);
int ttm_run(const tacogb_csf3* B, int32_t L, const void* C, void* out, bool dense, int variant,
            cudaStream_t st);
// MTTKRP's second step alone: A (already zeroed) += C rows times the fiber rows T (nfib x J,
// the fiber level times D); reads only B's upper levels (crd0, pos1, crd1) and its sizes.
int mttkrp_combine_launch(const tacogb_csf3* B, int32_t J, const void* C, const void* T, void* A,
                          cudaStream_t st);
int mttkrp_run(const tacogb_csf3* B, int32_t J, const void* C, const void* D, void* A,
               int variant, cudaStream_t st);

// Operand formats (formats.cu): DCSR SpMV (dense result, or the values of the sparse result
// whose pattern is the stored rows) and SpMM, CSC SpMV by a GPU transpose, sparse -> dense x.
int spmv_dcsr_run(const tacogb_dcsr* A, const void* x, void* y, bool dense, cudaStream_t st);
int spmm_dcsr_run(const tacogb_dcsr* A, int32_t N, const void* B, void* C, cudaStream_t st);
int spmv_csc_run(const tacogb_csr* Acsc, const void* x, void* y, cudaStream_t st);
int csc_to_csr_run(int32_t rows, int32_t cols, int64_t nnz, const int32_t* colpos,
                   const int32_t* rowidx, const void* vals, int32_t vtype, int32_t* pos,
                   int32_t* crd, void* out_vals, cudaStream_t st);
int densify_run(int32_t n, int64_t k, const int32_t* idx, const void* vals, int32_t vtype,
                void* out, cudaStream_t st);
// pos[0..outer] of a doubly compressed level with n0 stored outer coordinates crd0.
int expand_pos_run(const int32_t* crd0, const int32_t* pos1, int32_t n0, int32_t outer,
                   int32_t* pos, cudaStream_t st);

// COO -> CSR pack (pack.cu): device arrays in and out; *nnz read back (synchronises).
int pack_csr(int32_t rows, int32_t cols, int64_t n, const int32_t* coord_rows,
             const int32_t* coord_cols, const void* vals, int32_t vtype, int32_t* pos,
             int32_t* crd, void* out_vals, int64_t* nnz, cudaStream_t st);
// taco's coordinate-buffer records (int32 row, int32 column, value) -> separate arrays.
int pack_split_records(const void* buf, int64_t n, int32_t vtype, int32_t* r, int32_t* c,
                       void* v, cudaStream_t st);

}  // namespace tacogb
