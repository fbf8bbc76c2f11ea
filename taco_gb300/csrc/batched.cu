// Batched SpMV over thousands of uneven CSR matrices in one persistent, graph-captured launch.
//
// taco computes one statement per call; a batch of independent y_m = A_m x_m has no counterpart
// there beyond calling the generated compute once per matrix.  Here every matrix is cut into
// work units of its own kind (the per-matrix variant):
//   merge_ipt7 / merge_ipt3  merge-path tiles of 128*IPT items (rows + nonzeros): nnz-balanced,
//                            skew-proof, the same per-tile code as the single-matrix kernel;
//   vector_g4 / vector_g16   blocks of 128 rows, G lanes per row with a shuffle butterfly:
//                            cheapest for short regular rows.
// All units of all matrices form one global work queue.  A persistent kernel (one resident CTA
// per slot) takes units from an atomic counter, finds the unit's matrix by binary search over the
// unit offsets, and runs the unit; rows split between merge tiles are fixed up afterwards in tile
// order (deterministic).  The plan captures partition + main + fix-up in a CUDA graph once, so a
// batch costs one graph launch.  The variant only changes how work is cut, never the arithmetic:
// the accumulation policy (double-float or native FP64 for FP64 values, compensated FP32 for
// FP32 values) is fixed per plan.

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "batched.cuh"
#include "wmerge.cuh"

namespace tacogb {
namespace {

enum BatchKind { kMerge7 = 0, kMerge3 = 1, kVec2 = 2, kVec4 = 3, kVec8 = 4, kVec16 = 5 };
constexpr int kNumBatchKinds = 6;
const char* const kBatchKindNames[kNumBatchKinds] = {"merge_ipt7", "merge_ipt3", "vector_g2",
                                                     "vector_g4", "vector_g8", "vector_g16"};
__host__ __device__ __forceinline__ bool is_merge(int kind) { return kind <= kMerge3; }
// Lanes per row of a vector kind, and rows per vector unit (every lane group takes 4 rows).
__host__ __device__ __forceinline__ int vec_lanes(int kind) { return 2 << (kind - kVec2); }
__host__ __device__ __forceinline__ int vec_rows(int kind) { return 4 * kWmBlock / vec_lanes(kind); }
constexpr int kChunk = 4;  // units taken from the queue per atomic
static_assert(kNumBatchKinds == TACOGB_MLP_KINDS, "the cost model predicts one output per kind");


__host__ __device__ __forceinline__ int64_t kind_tile_items(int kind) {
  return kind == kMerge7 ? (int64_t)kWmBlock * 7 : (int64_t)kWmBlock * 3;
}


// Rows [R*lu, R*lu+R) of matrix d (R = 4*128/G) with G lanes per row and a shuffle butterfly.
// Returns false when a checked policy met a value it cannot represent (the caller redoes the
// unit natively).
template <class P, int G>
__device__ __forceinline__ bool batch_vector_unit(const BatchDesc& d, int lu,
                                                  const typename P::XG* __restrict__ x,
                                                  typename P::Out* __restrict__ y) {
  using Val = typename P::Val;
  const Val* __restrict__ vals = (const Val*)d.vals;
  constexpr int GROUPS = kWmBlock / G, R = 4 * GROUPS;
  const int g = threadIdx.x / G, lane = threadIdx.x % G;
  const int rb = lu * R, re = min(d.rows, rb + R);
  bool ok = true;
  for (int base = rb; base < re; base += GROUPS) {  // uniform trip count across the CTA
    const int row = base + g;
    typename P::Acc acc = P::zero();
    if (row < re) {
      const int32_t p1 = __ldg(d.pos + row + 1);
      for (int32_t p = __ldg(d.pos + row) + lane; p < p1; p += G)
        ok &= P::madd(acc, vals[p], ldg_xg(x + __ldg(d.crd + p)));
    }
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) acc = P::add(acc, P::shfl_xor(acc, m));
    if (row < re && lane == 0) y[row] = P::out(acc);
  }
  return ok;
}

template <class P, int IPT>
__device__ __forceinline__ double batch_merge_unit(unsigned char* smem, const BatchDesc& d,
                                                   int2 c0, int2 c1, int* status) {
  using Val = typename P::Val;
  WmSmem<P, IPT>& s = *reinterpret_cast<WmSmem<P, IPT>*>(smem);
  const Val* vals = (const Val*)d.vals;
  const typename P::XG* xg = (const typename P::XG*)d.x;
  const Val* x64 = (const Val*)d.x;
  typename P::Out* y = (typename P::Out*)d.y;
  // Merge kinds are only planned for 16-byte aligned arrays, so the tile is always staged with
  // bulk copies (one instantiation per IPT keeps the persistent kernel free of spills).
  return wm_process_tile<P, IPT, true>(s, d.pos, d.crd, vals, xg, x64, nullptr, y, d.rows,
                                       d.nnz, c0.x, c1.x - c0.x, c0.y, c1.y - c0.y, status);
}

template <class P, int G>
__device__ __forceinline__ void batch_vector_checked(const BatchDesc& d, int lu) {
  const bool ok = batch_vector_unit<P, G>(d, lu, (const typename P::XG*)d.x,
                                          (typename P::Out*)d.y);
  if constexpr (P::kChecked) {
    if (!__syncthreads_and(ok))
      batch_vector_unit<PolNative64, G>(d, lu, (const double*)d.x, (double*)d.y);
  }
}

template <class P>
__device__ __forceinline__ void batch_vector_any(const BatchDesc& d, int lu) {
  switch (d.kind) {
    case kVec2: batch_vector_checked<P, 2>(d, lu); break;
    case kVec4: batch_vector_checked<P, 4>(d, lu); break;
    case kVec8: batch_vector_checked<P, 8>(d, lu); break;
    default: batch_vector_checked<P, 16>(d, lu); break;
  }
}

// Persistent worker: CTAs take chunks of kChunk consecutive units from the queue until it runs
// dry.  The next chunk's atomic is issued when a chunk starts and its result is only needed when
// the chunk ends, so the queue round trip overlaps the work; within a chunk the matrix index
// advances incrementally.  Thread 0 records each unit's duration in SM cycles (the autotuner's
// cost measure: the CTA time a unit holds one of the resident slots).
template <class P>
__global__ void __launch_bounds__(kWmBlock, 8)
batch_spmv_kernel(const BatchDesc* __restrict__ desc, const int32_t* __restrict__ unit_off,
                  int count, int32_t total, const int2* __restrict__ part,
                  int32_t* __restrict__ carry_row, double* __restrict__ carry_val,
                  int* __restrict__ counter, long long* __restrict__ unit_cycles, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_next;
  if (threadIdx.x == 0) s_next = atomicAdd(counter, kChunk);
  __syncthreads();
  int c = s_next;
  while (c < total) {
    __syncthreads();  // every thread holds c before s_next is written again
    int next = 0;
    if (threadIdx.x == 0) next = atomicAdd(counter, kChunk);
    int m = find_matrix(unit_off, count, c);
    const int cend = min(c + kChunk, total);
    for (int u = c; u < cend; u++) {
      const long long t0 = clock64();
      while (u >= __ldg(unit_off + m + 1)) m++;
      const BatchDesc d = desc[m];
      const int lu = u - d.unit0;
      if (is_merge(d.kind)) {
        const int2* p = part + d.part0;
        const int2 c0 = p[lu], c1 = p[lu + 1];
        const double cd = d.kind == kMerge7 ? batch_merge_unit<P, 7>(smem_raw, d, c0, c1, status)
                                            : batch_merge_unit<P, 3>(smem_raw, d, c0, c1, status);
        if (threadIdx.x == 0) {
          carry_row[u] = c1.x;
          carry_val[u] = cd;
        }
      } else {
        batch_vector_any<P>(d, lu);
        if (threadIdx.x == 0) carry_row[u] = INT_MAX;
      }
      if (threadIdx.x == 0) {
        if (u == cend - 1) s_next = next;
        unit_cycles[u] = clock64() - t0;
      }
      __syncthreads();  // shared memory is reused by the next unit; s_next is published
    }
    c = s_next;
  }
}

// Adds merge-tile carries (runs of consecutive units of one matrix ending inside the same row,
// summed in unit order) and resets the work queue for the next launch.
template <typename Out>
__global__ void batch_fixup(const BatchDesc* __restrict__ desc, const int32_t* __restrict__ unit_off,
                            int count, int32_t total, const int32_t* __restrict__ carry_row,
                            const double* __restrict__ carry_val, int* __restrict__ counter) {
  const int32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u == 0) *counter = 0;
  if (u >= total) return;
  const int32_t r = carry_row[u];
  if (r == INT_MAX) return;
  const int m = find_matrix(unit_off, count, u);
  const BatchDesc& d = desc[m];
  if (r >= d.rows) return;
  if (u > d.unit0 && carry_row[u - 1] == r) return;
  double tot = carry_val[u];
  for (int32_t v = u + 1; v < d.unit0 + d.units && carry_row[v] == r; v++) tot += carry_val[v];
  Out* y = (Out*)d.y;
  y[r] = (Out)((double)y[r] + tot);
}

// Per-matrix sum of the unit cycles of the last run (one warp per matrix).
__global__ void batch_matrix_cycles(const BatchDesc* __restrict__ desc, int count,
                                    const long long* __restrict__ unit_cycles,
                                    long long* __restrict__ out) {
  const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (m >= count) return;
  const BatchDesc& d = desc[m];
  long long t = 0;
  for (int u = lane; u < d.units; u += 32) t += unit_cycles[d.unit0 + u];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[m] = t;
}

}  // namespace
}  // namespace tacogb

// ================================================================= plan (C ABI) ==========

namespace tacogb {

void batch_free(tacogb_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->cap) cudaStreamDestroy(b->cap);
  cudaFree(b->d_desc);
  cudaFree(b->d_unit_off);
  cudaFree(b->d_blk_off);
  cudaFree(b->d_part);
  cudaFree(b->d_carry_row);
  cudaFree(b->d_carry_val);
  cudaFree(b->d_counter);
  cudaFree(b->d_unit_cycles);
  cudaFree(b->d_mat_cycles);
  cudaFree(b->d_unit_mat);
  delete b;
}

int batch_alloc(tacogb_batch* b, const BatchDesc* desc, const int32_t* unit_off,
                const int32_t* blk_off, int64_t parts, int64_t carry_cols, bool with_unit_mat) {
  const int count = b->count;
  const int64_t u1 = std::max<int64_t>(b->total_units, 1);
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  alloc((void**)&b->d_desc, sizeof(BatchDesc) * count);
  alloc((void**)&b->d_unit_off, sizeof(int32_t) * (count + 1));
  alloc((void**)&b->d_blk_off, sizeof(int32_t) * (count + 1));
  alloc((void**)&b->d_part, sizeof(int2) * std::max<int64_t>(parts, 1));
  alloc((void**)&b->d_carry_row, sizeof(int32_t) * u1);
  alloc((void**)&b->d_carry_val, sizeof(double) * u1 * carry_cols);
  if (with_unit_mat) alloc((void**)&b->d_unit_mat, sizeof(int32_t) * u1);
  alloc((void**)&b->d_counter, sizeof(int));
  alloc((void**)&b->d_unit_cycles, sizeof(long long) * u1);
  alloc((void**)&b->d_mat_cycles, sizeof(long long) * count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(TACOGB_ERR_ALLOC, "batch: allocating the plan: %s", cudaGetErrorString(e));
    return TACOGB_ERR_ALLOC;
  }
  TACOGB_CUDA_TRY(cudaMemset(b->d_unit_cycles, 0, sizeof(long long) * u1));
  TACOGB_CUDA_TRY(cudaMemset(b->d_counter, 0, sizeof(int)));
  TACOGB_CUDA_TRY(cudaMemcpy(b->d_desc, desc, sizeof(BatchDesc) * count, cudaMemcpyHostToDevice));
  TACOGB_CUDA_TRY(cudaMemcpy(b->d_unit_off, unit_off, sizeof(int32_t) * (count + 1),
                             cudaMemcpyHostToDevice));
  TACOGB_CUDA_TRY(cudaMemcpy(b->d_blk_off, blk_off, sizeof(int32_t) * (count + 1),
                             cudaMemcpyHostToDevice));
  return 0;
}

int batch_end_capture(tacogb_batch* b) {
  const cudaError_t le = cudaGetLastError();
  const cudaError_t ce = cudaStreamEndCapture(b->cap, &b->graph);
  if (le != cudaSuccess || ce != cudaSuccess) {
    set_error(TACOGB_ERR_CUDA, "batch: graph capture failed: %s",
              cudaGetErrorString(le != cudaSuccess ? le : ce));
    return TACOGB_ERR_CUDA;
  }
  TACOGB_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return 0;
}

namespace {

template <class P>
int batch_capture(tacogb_batch* b, int32_t total_blocks, int* status) {
  auto kern = batch_spmv_kernel<P>;
  const size_t smem = sizeof(WmSmem<P, 7>);
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, -1));
  int per_sm = 0;
  TACOGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWmBlock, smem));
  const int grid = sm_count() * std::max(per_sm, 1);
  TACOGB_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
  TACOGB_CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
  b->kernels_per_run = 0;
  if (total_blocks > 0) {
    batch_partition<<<total_blocks, kPartBlock, 0, b->cap>>>(b->d_desc, b->d_blk_off, b->count,
                                                             b->d_part);
    b->kernels_per_run++;
  }
  if (b->total_units > 0) {
    kern<<<grid, kWmBlock, smem, b->cap>>>(b->d_desc, b->d_unit_off, b->count, b->total_units,
                                           b->d_part, b->d_carry_row, b->d_carry_val,
                                           b->d_counter, b->d_unit_cycles, status);
    b->kernels_per_run++;
  }
  batch_fixup<typename P::Out><<<(std::max(b->total_units, 1) + 255) / 256, 256, 0, b->cap>>>(
      b->d_desc, b->d_unit_off, b->count, b->total_units, b->d_carry_row, b->d_carry_val,
      b->d_counter);
  b->kernels_per_run++;
  return batch_end_capture(b);
}

}  // namespace
}  // namespace tacogb

using namespace tacogb;

extern "C" {

int tacogb_batch_variant_count(void) { return kNumBatchKinds; }
const char* tacogb_batch_variant_name(int32_t v) {
  return (v >= 0 && v < kNumBatchKinds) ? kBatchKindNames[v] : "";
}

int tacogb_batch_create(int32_t count, const tacogb_csr* mats, const void* const* x,
                        void* const* y, int32_t precision, const int32_t* variants,
                        tacogb_batch** out) {
  TACOGB_CHECK_ARG(out != nullptr, "batch: null output handle");
  *out = nullptr;
  TACOGB_CHECK_ARG(count > 0 && mats && x && y, "batch: empty or null batch");
  const int vt = mats[0].vtype;
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "batch: unsupported value type %d", vt);
  TACOGB_CHECK_ARG(precision == 0 || (precision == 1 && vt == TACOGB_F64),
                   "batch: precision %d (0 = default, 1 = native FP64 for FP64 values)", precision);
  std::vector<BatchDesc> desc(count);
  std::vector<int32_t> unit_off(count + 1), blk_off(count + 1);
  int64_t units = 0, parts = 0, blocks = 0;
  for (int m = 0; m < count; m++) {
    const tacogb_csr& A = mats[m];
    TACOGB_CHECK_ARG(A.vtype == vt, "batch: matrix %d has value type %d, expected %d", m, A.vtype, vt);
    TACOGB_CHECK_ARG(A.rows >= 0 && A.cols >= 0 && A.nnz >= 0 && A.nnz <= INT32_MAX,
                     "batch: matrix %d has a bad size", m);
    TACOGB_CHECK_ARG(A.rows == 0 || (A.pos && y[m]), "batch: matrix %d has null pos or y", m);
    TACOGB_CHECK_ARG(A.nnz == 0 || (A.crd && A.vals && x[m]), "batch: matrix %d has null arrays", m);
    int kind = variants ? variants[m] : kMerge7;
    TACOGB_CHECK_ARG(kind >= 0 && kind < kNumBatchKinds, "batch: matrix %d variant %d", m, kind);
    const bool aligned = (((uintptr_t)A.pos | (uintptr_t)A.crd | (uintptr_t)A.vals) & 15) == 0;
    if (is_merge(kind) && !aligned) kind = kVec4;  // merge tiles are staged with bulk copies
    BatchDesc& d = desc[m];
    d.pos = A.pos;
    d.crd = A.crd;
    d.vals = A.vals;
    d.x = x[m];
    d.y = y[m];
    d.rows = A.rows;
    d.cols = A.cols;
    d.nnz = (int32_t)A.nnz;
    d.kind = kind;
    d.tma = aligned;
    d.tile = is_merge(kind) ? (int32_t)kind_tile_items(kind) : 0;
    d.snap = 0;
    const int64_t u = is_merge(kind) ? ((int64_t)A.rows + A.nnz + d.tile - 1) / d.tile
                                     : ((int64_t)A.rows + vec_rows(kind) - 1) / vec_rows(kind);
    d.unit0 = (int32_t)units;
    d.units = (int32_t)u;
    d.part0 = (int32_t)parts;
    d.blk0 = (int32_t)blocks;
    unit_off[m] = (int32_t)units;
    blk_off[m] = (int32_t)blocks;
    units += u;
    if (is_merge(kind) && u > 0) {
      parts += u + 1;
      blocks += ((int64_t)A.rows + 1 + kPartBlock - 1) / kPartBlock;
    }
    TACOGB_CHECK_ARG(units < INT32_MAX / 2 && parts < INT32_MAX / 2 && blocks < INT32_MAX / 2,
                     "batch: too much work for one plan");
  }
  unit_off[count] = (int32_t)units;
  blk_off[count] = (int32_t)blocks;

  int* status = device_status();
  if (!status) return last_code();
  tacogb_batch* b = new tacogb_batch();
  cudaGetDevice(&b->device);
  b->count = count;
  b->vt = vt;
  b->total_units = (int32_t)units;
  int rc = batch_alloc(b, desc.data(), unit_off.data(), blk_off.data(), parts, 1, false);
  if (rc == 0) {
    if (vt == TACOGB_F32) rc = batch_capture<PolComp32>(b, (int32_t)blocks, status);
    else if (precision == 1) rc = batch_capture<PolNative64>(b, (int32_t)blocks, status);
    else rc = batch_capture<PolDF64X>(b, (int32_t)blocks, status);
  }
  if (rc) {
    batch_free(b);
    return rc;
  }
  *out = b;
  return 0;
}

int tacogb_batch_run(tacogb_batch* b, void* stream) {
  TACOGB_CHECK_ARG(b != nullptr && b->exec != nullptr, "batch: null plan");
  TACOGB_CUDA_TRY(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  for (int k = 0; k < b->kernels_per_run; k++) count_launch();
  return 0;
}

int tacogb_batch_matrix_cycles(tacogb_batch* b, int64_t* cycles, void* stream) {
  TACOGB_CHECK_ARG(b != nullptr && b->exec != nullptr && cycles != nullptr, "batch: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  batch_matrix_cycles<<<(b->count * 32 + 255) / 256, 256, 0, st>>>(b->d_desc, b->count,
                                                                     b->d_unit_cycles, b->d_mat_cycles);
  count_launch();
  TACOGB_CUDA_TRY(cudaGetLastError());
  TACOGB_CUDA_TRY(cudaMemcpyAsync(cycles, b->d_mat_cycles, sizeof(long long) * b->count,
                                  cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return 0;
}

int tacogb_batch_destroy(tacogb_batch* b) {
  batch_free(b);
  return 0;
}

}  // extern "C"
