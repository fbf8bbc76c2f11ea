/* libtacogb — the GB300 (sm_103a) implementation of taco's sparse hot path behind a C ABI.
 *
 * Two layers are exported:
 *
 *  1. taco's kernel ABI.  For each of the three statements
 *       SpMV   y(i)   = A(i,j) * x(j)     A {Dense,Sparse} (CSR), x, y {Dense}
 *       SpMM   C(i,k) = A(i,j) * B(j,k)   A CSR, B and C {Dense,Dense} row-major
 *       SpGEMM C(i,k) = A(i,j) * B(j,k)   A, B, C CSR
 *     the library exports `assemble`, `compute` and `evaluate` with the signature taco's code
 *     generator emits (int f(taco_tensor_t* result, taco_tensor_t* operand...), result first,
 *     operands in TensorBase::getArguments order — src/tensor.cpp:779-806,
 *     src/codegen/codegen_c.cpp:591-630) and the packed `_shim_` form that
 *     ir::Module::callFuncPackedRaw resolves with dlsym (src/codegen/module.cpp:178-218).
 *     Names carry a pattern prefix here; the per-pattern objects libtacogb_<pattern>.so export
 *     the unprefixed names (assemble, compute, evaluate, _shim_*) exactly as a taco-compiled
 *     module does.
 *
 *     Memory: operand arrays may be host memory (malloc, as taco allocates without CUDA),
 *     pinned host memory, managed memory (taco's CUDA build, cudaMallocManaged —
 *     src/cuda.cpp:54-63) or device memory.  Host arrays are staged to the GPU inside the call.
 *     Result arrays allocated by `assemble`/`evaluate` use malloc when the operands are host
 *     memory and cudaMallocManaged otherwise, matching the allocator taco frees them with
 *     (src/storage/array.cpp:22-33).  Calls are synchronous, like taco's generated CUDA
 *     (cudaDeviceSynchronize after each launch, src/codegen/codegen_cuda.cpp:609).
 *
 *  2. A device-pointer layer (tacogb_spmv, tacogb_spmm, tacogb_spgemm_*) on a caller stream,
 *     which the taco ABI forwards to and which may be captured in CUDA graphs.
 *
 * Errors: every function returns 0 on success and a TACOGB_ERR_* code otherwise; the message
 * is available from tacogb_last_error().  Generated taco CUDA exits the process on a CUDA
 * error (src/codegen/codegen_cuda.cpp:58-67); this library never does.
 *
 * Threads: the library keeps per-device state (scratch and staging buffers, a small mapped
 * host mailbox for kernel results, the taco ABI's streams, the last one-pass SpGEMM between
 * tacogb_spgemm_onepass and _finish).  Calls for one device must not overlap in time from
 * different host threads — serialise them, as taco's single-threaded compute() does; calls on
 * different devices may run at the same time.  Device-layer calls on one caller stream are
 * ordered by that stream like any other work on it.
 */
#ifndef TACO_GB300_H
#define TACO_GB300_H

#include <stdint.h>
#include "taco_gb300_tensor.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TACOGB_OK 0
#define TACOGB_ERR_ARG 1       /* invalid argument, unsupported format or type */
#define TACOGB_ERR_CUDA 2      /* CUDA runtime error */
#define TACOGB_ERR_OVERFLOW 3  /* a result does not fit taco's int32 positions */
#define TACOGB_ERR_TIMEOUT 4   /* a bounded device-side wait gave up */
#define TACOGB_ERR_ALLOC 5     /* allocation failed */

/* Value types (taco's csize in bits: 64 -> F64, 32 -> F32; 16 -> BF16 is an extension). */
#define TACOGB_F64 0
#define TACOGB_F32 1
#define TACOGB_BF16 2

/* Message of the last failing call on this thread ("" if none). */
const char* tacogb_last_error(void);
/* Library version string. */
const char* tacogb_version(void);

/* Reads and clears this device's status word: bit 1 = a bounded device-side wait (an mbarrier
 * on an asynchronous copy) gave up.  The taco-ABI entry points check it themselves and return
 * TACOGB_ERR_TIMEOUT; stream-ordered callers of the device layer check it when they sync. */
int tacogb_device_status(int32_t* status);

/* Index validation.  taco's pack produces valid compressed levels by construction
 * (src/tensor.cpp:295-463) and its generated kernels trust them; this library's taco-ABI entry
 * points instead check every compressed level they are handed before any kernel gathers through
 * it: pos[0] == 0, pos non-decreasing with pos[outer] == nnz, 0 <= crd < the level's dimension,
 * and crd strictly increasing within each segment (taco's sorted, distinct coordinates).  A
 * violation returns TACOGB_ERR_ARG naming the first offending segment or position.
 * The check is one kernel reading pos and crd once, on the arrays the kernels will read (the
 * caller's device arrays or the staged copies of host arrays), before any gathering kernel; a
 * call that cannot reach a GPU checks host-resident levels on the host, so invalid input is
 * still reported as TACOGB_ERR_ARG.  tacogb_spmv_compute and tacogb_spmm_compute check host
 * operands on their staged copies without waiting for the verdict: a level that fails is
 * rewritten on the device into a harmless one before the product runs, the error is returned
 * when the call ends (over host operands of 2^23 nonzeros or more, which are copied, checked
 * and multiplied chunk by chunk, with the position in the whole operand), and the result's
 * contents are then unspecified.  tacogb_sddmm_compute does the same over host operands of
 * 2^23 nonzeros or more with values kept at B's nonzeros and J <= 512 (D copied and
 * transposed first, then B's rows with their rows of C chunk by chunk), and so does
 * tacogb_mttkrp_compute when B's fiber level holds 2^23 nonzeros or more (that level chunk by
 * chunk, the upper levels checked after it).  The device layer (tacogb_spmv
 * and the other functions on tacogb_csr) trusts its arguments; tacogb_csr_validate checks a
 * device CSR explicitly (declared with the device layer below).  tacogb_set_validation(0) turns
 * the taco-ABI checks off (and returns the previous setting); they are on by default. */
int tacogb_set_validation(int32_t on);
/* Checks one compressed level held in host memory (outer segments over a dimension of size
 * inner, nnz = pos[outer]); 0 or TACOGB_ERR_ARG.  Uses host threads only; needs no GPU. */
int tacogb_validate_level_host(int64_t outer, int32_t inner, const int32_t* pos,
                               const int32_t* crd, int64_t nnz);

/* Number of kernels this library has launched in this process. */
long long tacogb_launch_count(void);
/* Per-kernel device timing: between begin and end every launch is bracketed by CUDA events on
 * its stream.  end() waits for the events and writes, per distinct kernel name (64-byte slots
 * in `names`), the summed milliseconds and the launch count; returns the number of kernels. */
void tacogb_profile_begin(void);
int tacogb_profile_end(int32_t max_kernels, char* names, double* total_ms, int32_t* launches);
/* Between begin and end, pauses (on = 0) or resumes (on != 0) the bracketing without clearing
 * what was recorded, so that a caller can sample some of its launches and keep the event
 * records out of the rest. */
void tacogb_profile_enable(int32_t on);

/* COO -> CSR pack on the GPU.  Replaces the host sort and generated pack of TensorBase::pack
 * (src/tensor.cpp:295-463, qsort at :420-422) for a rows x cols CSR ({Dense,Sparse}) tensor:
 * n coordinates (coord_rows[i], coord_cols[i]) with values vals[i] (vtype TACOGB_F64 or
 * TACOGB_F32), in any order and with duplicates, become pos (rows + 1 entries), crd and
 * out_vals (capacity n each) with columns ascending per row and duplicates summed in input
 * order; explicit zeros are kept, as taco keeps them.  Device (or managed) arrays, work on
 * `stream`; *nnz is read back (the call synchronises).  A coordinate outside the matrix
 * returns TACOGB_ERR_ARG. */
int tacogb_pack_csr(int32_t rows, int32_t cols, int64_t n, const int32_t* coord_rows,
                    const int32_t* coord_cols, const void* vals, int32_t vtype, int32_t* pos,
                    int32_t* crd, void* out_vals, int64_t* nnz, void* stream);

/* The same on taco's own data: `buffer` holds n records laid out as taco's coordinate buffer
 * (int32 row, int32 column, then the value: 16 bytes per FP64 record, 12 per FP32), host or
 * device memory; T is the 2-D CSR result tensor (dimensions, csize set).  Allocates pos, crd
 * and vals (malloc, or cudaMallocManaged when the buffer is device-accessible, the allocators
 * taco frees them with, src/storage/array.cpp:22-33) and stores them in T->indices[1] and
 * T->vals as unpackTensorData does (src/tensor.cpp:263-292). */
int tacogb_pack_taco(taco_tensor_t* T, const void* buffer, int64_t n);

/* Reads a 2-D Matrix Market (.mtx: coordinate or array, real, general or symmetric) or FROSTT
 * (.tns: "i j value" lines) file into COO records, as taco's readMTX / readTNS insert them
 * (src/storage/file_io_mtx.cpp:38-215, src/storage/file_io_tns.cpp:37-85): 0-based
 * coordinates, symmetric off-diagonal entries followed by their mirror, values by strtod; the
 * format is taken from the first line ("%%MatrixMarket" or not).  Lines are parsed by all host
 * threads.  *coord_rows, *coord_cols and *vals are malloc'ed (free with tacogb_free_host); pass
 * them to tacogb_pack_csr (after copying them to the GPU) for CSR. */
int tacogb_read_coo(const char* path, int32_t* rows, int32_t* cols, int64_t* n,
                    int32_t** coord_rows, int32_t** coord_cols, double** vals);
/* A Rutherford-Boeing file as taco's readRB loads it (src/storage/file_io_rb.cpp:319-350): real
 * unsymmetric assembled (RUA) only, as CSC — colptr (cols + 1), rowidx and vals (nnz), 0-based,
 * in host memory released with tacogb_free_host.  tacogb_csc_to_csr turns it into CSR. */
int tacogb_read_rb(const char* path, int32_t* rows, int32_t* cols, int64_t* nnz,
                   int32_t** colptr, int32_t** rowidx, double** vals);
void tacogb_free_host(void* p);

/* ------------------------------------------------------------------ device layer -------- */

/* A CSR matrix in device (or managed) memory: {Dense,Sparse} with int32 pos/crd. */
typedef struct tacogb_csr {
  int32_t rows, cols;
  int64_t nnz;
  const int32_t* pos;  /* rows+1 */
  const int32_t* crd;  /* nnz, sorted within each row */
  const void* vals;    /* nnz values of type vtype */
  int32_t vtype;       /* TACOGB_F64 or TACOGB_F32 */
} tacogb_csr;

/* Checks a device-resident CSR matrix on the GPU, as the taco-ABI entry points check their
 * operands (A->nnz must equal pos[rows]); synchronises stream. */
int tacogb_csr_validate(const tacogb_csr* A, void* stream);

/* SpMV kernel variants.  TACOGB_VARIANT_AUTO lets the library choose (tuning database, cost
 * model, then a structural rule). */
#define TACOGB_VARIANT_AUTO (-1)

/* y = A x.  F64 values: x, y FP64.  F32 values: x, y FP32 with compensated (TwoSum/TwoProduct)
 * row accumulation.  Replaces the generated compute of y(i)=A(i,j)*x(j)
 * (src/lower/lowerer_impl_imperative.cpp:1304 + src/index_notation/transformations.cpp:1982). */
int tacogb_spmv(const tacogb_csr* A, const void* x, void* y, int32_t variant, void* stream);
int tacogb_spmv_variant_count(void);
const char* tacogb_spmv_variant_name(int32_t variant);
/* The variant TACOGB_VARIANT_AUTO runs for A: warp tiles sized for scattered columns, or, for a
 * matrix of at least 2^21 nonzeros, for local columns when most gaps between consecutive stored
 * columns (4096 samples) are under 64; a matrix of fewer nonzeros whose rows all hold at most 32
 * runs vector_g4 (one launch, four lanes per row).  The choice is cached per matrix (pos and crd
 * pointers, rows, nonzeros); the first call for a matrix with rows and nonzeros runs one small
 * kernel on stream and synchronises it, unless the stream is capturing. */
int tacogb_spmv_auto_variant(const tacogb_csr* A, void* stream);

/* y = A x like tacogb_spmv (merge-path kernel, default accumulation per value type), for
 * callers that cannot allocate GPU memory during the call: code running under another
 * framework's memory pool or allocator hooks, latency-critical paths where cudaMalloc/cudaFree
 * may synchronise the device, and deployments with a fixed memory budget.  No counterpart in
 * taco (taco's generated kernels allocate their outputs and never need scratch).
 * It calls no cudaMalloc, cudaFree or other allocating routine: its temporary memory is a
 * 4 MiB static device array that every GPU loading this library holds until the process exits,
 * which bounds the problem to about 2.9e8 rows + nonzeros; larger problems are rejected with
 * TACOGB_ERR_ARG and a message (use tacogb_spmv).  The first call on each device looks the
 * array's address up (cudaGetSymbolAddress) and caches it, so make that first call before any
 * stream capture.  The cached address belongs to the device's primary context: after a
 * cudaDeviceReset in this process it is stale, so do not call this function again after a
 * reset.  All calls share the one array: calls that overlap on the GPU (different
 * streams, or graphs replayed concurrently) race and must be serialised by the caller. */
int tacogb_spmv_noalloc(const tacogb_csr* A, const void* x, void* y, void* stream);

/* Batched SpMV: y_m = A_m x_m for count independent CSR matrices in one persistent launch.
 * taco has no batched statement: a taco user calls the generated compute of y(i)=A(i,j)*x(j)
 * once per matrix (TensorBase::compute, src/tensor.cpp:829-850); a plan replaces that loop.
 * tacogb_batch_create validates every matrix (all of one value type, F64 or F32), cuts each into
 * work units of the kind variants[m] names (tacogb_batch_variant_name; NULL = merge_ipt7 for
 * all), uploads the work queue and captures the launches in a CUDA graph.  The pointers in
 * mats, x and y are kept: the plan computes from whatever those device arrays hold when
 * tacogb_batch_run is called.  precision 0 = the default accumulation (double-float on the FP32
 * pipe for F64 values, with native FP64 for tiles outside its range; compensated FP32 for F32
 * values), 1 = native FP64 (F64 values only).  Merge kinds need pos, crd and vals 16-byte
 * aligned; a matrix whose arrays are not is planned with vector_g4.
 * tacogb_batch_run launches the graph on stream (one graph launch; stream-ordered; one run of
 * a plan at a time). */
typedef struct tacogb_batch tacogb_batch;
int tacogb_batch_create(int32_t count, const tacogb_csr* mats, const void* const* x,
                        void* const* y, int32_t precision, const int32_t* variants,
                        tacogb_batch** plan);
/* Batched SpMM: C_m = A_m B_m with B_m (A_m->cols x N) and C_m (A_m->rows x N) dense row-major,
 * N shared by the batch; value types as tacogb_spmm (F64/F64, F32/F32, F32 values with BF16 B).
 * Units are row-snapped merge tiles of 512 items; every warp of the persistent kernel takes
 * units from the queue.  precision 0 = double-float (F64) or compensated FP32 accumulation,
 * 1 = native FMA; BF16 B always accumulates in FP32.  Run, cost and destroy with the
 * tacogb_batch_* calls below. */
int tacogb_batch_spmm_create(int32_t count, const tacogb_csr* mats, int32_t N,
                             const void* const* B, int32_t btype, void* const* C,
                             int32_t precision, tacogb_batch** plan);
int tacogb_batch_run(tacogb_batch* plan, void* stream);
int tacogb_batch_destroy(tacogb_batch* plan);
/* Cost of each matrix in the last run of the plan: the sum over its work units of the SM cycles
 * the persistent kernel spent on each unit (read with clock64 by the unit's CTA).  Writes count
 * entries to the host array cycles; synchronises stream.  The autotuner's measure. */
int tacogb_batch_matrix_cycles(tacogb_batch* plan, int64_t* cycles, void* stream);
int tacogb_batch_variant_count(void);
const char* tacogb_batch_variant_name(int32_t variant);

/* ---- batch autotuning: sparsity features and the MLP cost model (tuner.cu) ----
 * The model predicts, for each batch work-unit kind, log2 of the SM cycles the kind spends per
 * (row + nonzero) of a matrix; the selection is the argmin.  It changes only which kernel runs.
 * Parameters: TACOGB_MLP_FEATURES inputs -> TACOGB_MLP_HIDDEN ReLU -> TACOGB_MLP_HIDDEN ReLU ->
 * TACOGB_MLP_KINDS outputs, packed as W1[H][F] b1[H] W2[H][H] b2[H] W3[K][H] b3[K] (float).
 * norm holds the feature means (F floats) then standard deviations (F floats); features are
 * z-scored with it inside the kernels.  All pointers except tacogb_batch_features' are device
 * pointers; calls are stream-ordered. */
#define TACOGB_MLP_FEATURES 10
#define TACOGB_MLP_HIDDEN 32
#define TACOGB_MLP_KINDS 6
int tacogb_mlp_param_count(void);
/* Features of every matrix (device CSR arrays) into the host array feats (count x F, row-major):
 * log2(rows+1), log2(nnz+1), log2(mean row length+1), std/mean of row lengths, log2(max+1),
 * Gini of row lengths (histogram: exact below 2048, 16 bins per octave above), max |j-i|/cols,
 * mean |j-i|/cols, fraction of empty rows, log2(cols+1).  Synchronises stream. */
int tacogb_batch_features(int32_t count, const tacogb_csr* mats, float* feats, void* stream);
/* Predictions (n x K; may be NULL) and argmin kinds (n; may be NULL) for n feature rows X. */
int tacogb_mlp_predict(const float* params, const float* norm, const float* X, int32_t n,
                       float* pred, int32_t* kinds, void* stream);
/* Gradient of the masked mean squared error sum(M*(y-Y)^2)/sum(M) with respect to the
 * parameters (grad: param_count floats) and the loss (one float; may be NULL).  Y, M: n x K. */
int tacogb_mlp_grad(const float* params, const float* norm, const float* X, const float* Y,
                    const float* M, int32_t n, float* grad, float* loss, void* stream);
/* steps full-batch Adam steps (beta1 0.9, beta2 0.999, eps 1e-8, learning rate lr), numbered
 * step0+1 .. step0+steps for bias correction; adam_state holds 2 x param_count floats (first and
 * second moments, zero before the first step); losses (steps floats; may be NULL) receives the
 * loss before each step.  Deterministic: the same inputs give the same parameters bit for bit. */
int tacogb_mlp_train(float* params, const float* norm, const float* X, const float* Y,
                     const float* M, int32_t n, int32_t steps, int32_t step0, float lr,
                     float* adam_state, float* losses, void* stream);
/* Exhaustive autotuner, the model's reference labels and fallback: plans the batch once per kind (every
 * matrix with that kind), runs it reps times after one warm-up, keeps each matrix's minimum
 * cycles (tacogb_batch_matrix_cycles) and writes the cheapest kind per matrix to the host array
 * kinds; cycles (host, count x TACOGB_MLP_KINDS, may be NULL) receives the table.  x and y are
 * written as in tacogb_batch_run.  Synchronises stream. */
int tacogb_batch_autotune(int32_t count, const tacogb_csr* mats, const void* const* x,
                          void* const* y, int32_t precision, int32_t reps, int32_t* kinds,
                          int64_t* cycles, void* stream);
/* Learned selection: tacogb_batch_features on the GPU, then tacogb_mlp_predict's argmin per
 * matrix into the host array kinds (params and norm: device pointers).  Synchronises stream. */
int tacogb_batch_select(int32_t count, const tacogb_csr* mats, const float* params,
                        const float* norm, int32_t* kinds, void* stream);

/* C = A B with B (rows = A->cols) x N and C (A->rows x N) dense row-major.
 * Types: A F64 with B F64 -> C FP64; A F32 with B F32 -> C FP32; A F32 with B BF16 -> C FP32
 * (BF16 dense operand, FP32 accumulation).  Replaces the generated compute of
 * C(i,k)=A(i,j)*B(j,k) with A {Dense,Sparse} (src/lower/lowerer_impl_imperative.cpp:1304, dense
 * k loop) and the GPU schedules of test/tests-scheduling-eval.cpp:249-370. */
int tacogb_spmm(const tacogb_csr* A, int32_t N, const void* B, int32_t btype, void* C,
                int32_t variant, void* stream);
int tacogb_spmm_variant_count(void);
const char* tacogb_spmm_variant_name(int32_t variant);

/* Two-phase C = A B with A, B, C CSR ({Dense,Sparse}, int32 pos/crd).  Keeps taco's result
 * structure exactly: every structural product (no numerical-zero dropping), columns sorted per
 * row; each value is the A-row-ordered sum of its products with separately rounded multiplies
 * and adds (taco's serial loop order).  Replaces the generated assemble/compute of
 * C(i,k)=A(i,j)*B(j,k) over the workspace form of src/index_notation/transformations.cpp:2083
 * (dense accelerator src/lower/lowerer_impl_imperative.cpp:2197, appends
 * src/lower/mode_format_compressed.cpp:107-213).
 *   symbolic  writes Cpos[0..A->rows] (device) and returns nnz(C) (synchronises the stream);
 *             TACOGB_ERR_OVERFLOW when nnz(C) exceeds int32.
 *   fill      writes the sorted columns Ccrd[0..nnz(C)) for that Cpos.
 *   numeric   writes Cvals (A's value type; A and B share it) for that pattern. */
int tacogb_spgemm_symbolic(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos,
                           int64_t* nnzC, void* stream);
int tacogb_spgemm_fill(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos,
                       int32_t* Ccrd, void* stream);
int tacogb_spgemm_numeric(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos,
                          const int32_t* Ccrd, void* Cvals, void* stream);
/* The same product in one pass, as taco's assemble-while-compute (one sort per row where the
 * three phases sort three times): tacogb_spgemm_onepass writes Cpos and returns nnz(C)
 * (synchronises the stream), leaving C's columns and values in library scratch; the caller
 * allocates Ccrd and Cvals for nnz(C) and tacogb_spgemm_onepass_finish moves them there (same
 * device, same stream, before the next one-pass product on that device).  Same results as the
 * three phases, bit for bit.  Products beyond int32 are refused (TACOGB_ERR_ARG): use the
 * phases. */
int tacogb_spgemm_onepass(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos,
                          int64_t* nnzC, void* stream);
int tacogb_spgemm_onepass_finish(const int32_t* Cpos, int32_t* Ccrd, void* Cvals, void* stream);

/* SDDMM, A(i,k) = B(i,k) * C(i,j) * D(j,k): B CSR (rows I, cols K), C dense row-major I x J,
 * D dense row-major J x K, all of B's value type (FP64 or FP32).  tacogb_sddmm writes the result
 * at B's nonzeros, out[p] = B.vals[p] * sum_j C(i,j) D(j,k) for nonzero p = (i,k);
 * tacogb_sddmm_dense writes taco's test form, a dense I x K result of row stride lda, zero
 * outside B's pattern.  FP64 within 1e-12 normwise of taco's serial loop (double-float or
 * DFMA, variant 1 or 0); FP32 natively.  Replaces the generated compute of that statement
 * (test/tests-scheduling-eval.cpp:783-840 CPU, 1360-1417 with the GPU schedule at :270-286).
 * Uses a K x J scratch copy of D (transposed) per call. */
int tacogb_sddmm(const tacogb_csr* B, int32_t J, const void* C, const void* D, void* out,
                 int32_t variant, void* stream);
int tacogb_sddmm_dense(const tacogb_csr* B, int32_t J, const void* C, const void* D, void* A,
                       int64_t lda, int32_t variant, void* stream);
int tacogb_sddmm_variant_count(void);
const char* tacogb_sddmm_variant_name(int32_t variant);

/* An order-3 tensor in taco's {Sparse,Sparse,Sparse} or {Dense,Sparse,Sparse} storage (CSF),
 * device pointers, int32 positions (taco's TensorStorage, src/storage/storage.cpp:127-177).
 * Level 0: n0 entries with coordinates crd0 (NULL for a dense level: n0 == dims[0], entry e is
 * i = e); level 1: pos1 (n0 + 1), crd1 (nfib = pos1[n0]), one entry per (i, j) fiber;
 * level 2: pos2 (nfib + 1), crd2 and vals (nnz = pos2[nfib]). */
typedef struct tacogb_csf3 {
  int32_t dims[3];
  int32_t n0;
  int32_t nfib;
  int64_t nnz;
  const int32_t* crd0;
  const int32_t* pos1;
  const int32_t* crd1;
  const int32_t* pos2;
  const int32_t* crd2;
  const void* vals;
  int32_t vtype; /* TACOGB_F64 or TACOGB_F32; the dense operands and results share it */
} tacogb_csf3;

/* A(i,j) = B(i,j,k) * c(k) (taco: test/tests-scheduling-eval.cpp:993-1043, 1474-1524).
 * tacogb_ttv writes one value per fiber (out[f] for fiber f = (i,j)); tacogb_ttv_dense taco's
 * dense dims[0] x dims[1] result, zero where B has no fiber.  SpMV over the fibers (variant: a
 * tacogb_spmv variant, TACOGB_VARIANT_AUTO for the library's choice). */
int tacogb_ttv(const tacogb_csf3* B, const void* c, void* out, int32_t variant, void* stream);
int tacogb_ttv_dense(const tacogb_csf3* B, const void* c, void* A, int32_t variant,
                     void* stream);
/* A(i,j,l) = B(i,j,k) * C(k,l), C dims[2] x L row-major (taco: :1094-1146, 1420-1472).
 * tacogb_ttm writes one row of L values per fiber (nfib x L); tacogb_ttm_dense the dense
 * dims[0] x dims[1] x L result.  SpMM over the fibers (variant: a tacogb_spmm variant,
 * TACOGB_VARIANT_AUTO for the library's choice). */
int tacogb_ttm(const tacogb_csf3* B, int32_t L, const void* C, void* out, int32_t variant,
               void* stream);
int tacogb_ttm_dense(const tacogb_csf3* B, int32_t L, const void* C, void* A, int32_t variant,
                     void* stream);
/* A(i,j) = B(i,k,l) * C(k,j) * D(l,j), C dims[1] x J, D dims[2] x J, A dims[0] x J, all
 * row-major (taco: :1148-1206, 1526-1580).  SpMM of the fibers with D (variant as for
 * tacogb_ttm), then per i the sum of C(k,:) times the fiber rows; variant -2 (FP64 only) runs one
 * fused kernel over nonzero chunks instead.  Either way partial row sums are added into A
 * atomically (the order of those adds is not fixed).  FP64 within 1e-12 normwise of taco's
 * loop. */
int tacogb_mttkrp(const tacogb_csf3* B, int32_t J, const void* C, const void* D, void* A,
                  int32_t variant, void* stream);

/* Operand formats on the SpMV / SpMM path (taco's tests: test/tests-expr_storage.cpp:873-937,
 * tests-scheduling-eval.cpp:1309-1358 and :655-662).  A DCSR matrix ({Sparse,Sparse}) stores n0
 * nonempty rows: crd0 their row numbers, pos (n0 + 1) and crd/vals their entries. */
typedef struct tacogb_dcsr {
  int32_t rows;
  int32_t cols;
  int32_t n0;
  int64_t nnz;
  const int32_t* crd0;
  const int32_t* pos;
  const int32_t* crd;
  const void* vals;
  int32_t vtype;
} tacogb_dcsr;
/* y = A x for DCSR A: dense_y != 0 writes all rows of y (zero where A stores no row); otherwise
 * y holds n0 values, the sparse result whose coordinates are crd0. */
int tacogb_spmv_dcsr(const tacogb_dcsr* A, const void* x, void* y, int32_t dense_y, void* stream);
/* C = A B for DCSR A, dense row-major B (cols x N) and C (rows x N; rows A does not store are
 * zero). */
int tacogb_spmm_dcsr(const tacogb_dcsr* A, int32_t N, const void* B, void* C, void* stream);
/* y = A x for CSC A given as a tacogb_csr whose pos has cols + 1 column starts and whose crd
 * holds row numbers (rows, cols are A's).  Transposes to CSR on the GPU per call. */
int tacogb_spmv_csc(const tacogb_csr* A, const void* x, void* y, void* stream);
/* CSC (colpos, rowidx, vals) -> CSR (pos rows + 1, crd, out_vals), rows sorted by column;
 * synchronises the stream.  TACOGB_ERR_ARG when a coordinate repeats. */
int tacogb_csc_to_csr(int32_t rows, int32_t cols, int64_t nnz, const int32_t* colpos,
                      const int32_t* rowidx, const void* vals, int32_t vtype, int32_t* pos,
                      int32_t* crd, void* out_vals, void* stream);
/* A sparse vector (k entries idx/vals) as a dense one of n entries. */
int tacogb_densify(int32_t n, int64_t k, const int32_t* idx, const void* vals, int32_t vtype,
                   void* out, void* stream);

/* ------------------------------------------------------------------ taco kernel ABI ----- */

/* y(i) = A(i,j) * x(j).  Replaces the generated assemble/compute/evaluate of that statement
 * (taco "y(i) = A(i,j) * x(j)" -f=A:ds; generated text at the lowering cited above).  Also the
 * format combinations of taco's spmv tests (test/tests-expr_storage.cpp:873-937): A CSC
 * ({Dense,Sparse} ordered {1,0}) or DCSR ({Sparse,Sparse}), x {Sparse}, and y {Sparse} with a
 * DCSR A (assemble gives y A's stored rows as its coordinates). */
int tacogb_spmv_assemble(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x);
int tacogb_spmv_compute(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x);
int tacogb_spmv_evaluate(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x);
int _shim_tacogb_spmv_assemble(void** args);
int _shim_tacogb_spmv_compute(void** args);
int _shim_tacogb_spmv_evaluate(void** args);

/* C(i,k) = A(i,j) * B(j,k), A CSR, B and C {Dense,Dense} row-major.  Replaces the generated
 * assemble/compute/evaluate of taco "C(i,k) = A(i,j) * B(j,k)" -f=A:ds (same lowering as
 * tacogb_spmm).  csize 64/64 -> FP64; 32/32 -> FP32; A 32 with B 16 -> BF16 B (extension). */
int tacogb_spmm_assemble(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);
int tacogb_spmm_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);
int tacogb_spmm_evaluate(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);
int _shim_tacogb_spmm_assemble(void** args);
int _shim_tacogb_spmm_compute(void** args);
int _shim_tacogb_spmm_evaluate(void** args);

/* C(i,k) = A(i,j) * B(j,k), C CSR; A and B CSR, DCSR ({Sparse,Sparse}), CSC ({Dense,Sparse}
 * ordered {1,0}) or DCSC ({Sparse,Sparse} ordered {1,0}), converted to CSR on the GPU (taco's
 * spgemm format test, test/tests-scheduling-eval.cpp:655-662).  assemble allocates and fills C's pos and crd and
 * allocates its vals (taco's generated assemble, which leaves vals for compute); compute fills
 * vals over the assembled pattern; evaluate does both.  Result arrays come from malloc for
 * host operands and cudaMallocManaged for GPU operands (taco's allocator choice,
 * src/storage/array.cpp:22-33); taco owns them afterwards (pos/crd UserOwns, vals Free,
 * src/tensor.cpp:263-292). */
int tacogb_spgemm_assemble(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);
int tacogb_spgemm_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);
int tacogb_spgemm_evaluate(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);
int _shim_tacogb_spgemm_assemble(void** args);
int _shim_tacogb_spgemm_compute(void** args);
int _shim_tacogb_spgemm_evaluate(void** args);

/* A(i,k) = B(i,k) * C(i,j) * D(j,k), B CSR, C and D {Dense,Dense} row-major; A either
 * {Dense,Dense} (taco's test form: assemble allocates I*K values, compute zero-fills and writes
 * B's pattern) or CSR with B's pattern (assemble copies B's pos and crd, allocates vals). */
int tacogb_sddmm_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
int tacogb_sddmm_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
int tacogb_sddmm_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
int _shim_tacogb_sddmm_assemble(void** args);
int _shim_tacogb_sddmm_compute(void** args);
int _shim_tacogb_sddmm_evaluate(void** args);

/* Order-3 statements with B {Sparse,Sparse,Sparse} or {Dense,Sparse,Sparse} and dense
 * row-major operands and results (taco's test forms): A(i,j) = B(i,j,k) * c(k);
 * A(i,j,l) = B(i,j,k) * C(k,l); A(i,j) = B(i,k,l) * C(k,j) * D(l,j).  assemble allocates A's
 * values, compute fills them, evaluate does both. */
int tacogb_ttv_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c);
int tacogb_ttv_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c);
int tacogb_ttv_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c);
int _shim_tacogb_ttv_assemble(void** args);
int _shim_tacogb_ttv_compute(void** args);
int _shim_tacogb_ttv_evaluate(void** args);
int tacogb_ttm_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C);
int tacogb_ttm_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C);
int tacogb_ttm_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C);
int _shim_tacogb_ttm_assemble(void** args);
int _shim_tacogb_ttm_compute(void** args);
int _shim_tacogb_ttm_evaluate(void** args);
int tacogb_mttkrp_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C,
                           taco_tensor_t* D);
int tacogb_mttkrp_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
int tacogb_mttkrp_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C,
                           taco_tensor_t* D);
int _shim_tacogb_mttkrp_assemble(void** args);
int _shim_tacogb_mttkrp_compute(void** args);
int _shim_tacogb_mttkrp_evaluate(void** args);

#ifdef __cplusplus
}
#endif
#endif
