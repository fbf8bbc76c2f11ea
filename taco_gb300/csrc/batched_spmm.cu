// Batched SpMM: C_m = A_m B_m for thousands of uneven CSR matrices in one persistent,
// graph-captured launch (B_m: cols x N, C_m: rows x N, dense row-major, N shared).
//
// taco computes one SpMM statement per call; the batch replaces a loop of those calls.  Units
// are the row-snapped merge tiles of the single-matrix SpMM (kMmBatchTile rows + nonzeros; rows
// shorter than half a tile are never split), listed over all matrices in one work queue.  Every
// warp of the persistent kernel is an independent worker: it takes chunks of kMmChunk units
// with one atomic (the next chunk's atomic overlaps the current chunk) and runs the sub-warp
// tile (spmm_tile_sub) on each unit, column slice by column slice.  Rows split between units
// are fixed up afterwards in unit order (deterministic, no atomics on C).

#include <algorithm>
#include <climits>
#include <vector>

#include "batched.cuh"
#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "spmm_tile.cuh"

namespace tacogb {
namespace {

constexpr int kMmBatchBlock = 256;
constexpr int kMmBatchTile = 512;
constexpr int kMmChunk = 4;

// The native recomputation of a tile whose values left the double-float range: rare, so kept
// out of line (its registers do not add to the hot path's).
template <int VEC, int SUB>
__device__ __noinline__ void batch_spmm_native(const BatchDesc& d, int32_t N, int2 c0, int2 c1,
                                               int u, int ct, int32_t* carry_row,
                                               double* carry_val) {
  spmm_tile_sub<MmNative64, VEC, SUB>(d.pos, d.crd, (const double*)d.vals, (const double*)d.x,
                                      (double*)d.y, d.rows, N, c0, c1, u, ct, carry_row,
                                      carry_val);
}

template <class P, int VEC, int SUB>
__device__ __forceinline__ void batch_spmm_unit(const BatchDesc& d, int32_t N, int2 c0, int2 c1,
                                                int u, int32_t* carry_row, double* carry_val) {
  using AV = typename P::AV;
  using BV = typename P::BV;
  using Out = typename P::Out;
  constexpr int COLS = (32 / SUB) * VEC;  // columns per slice
  for (int ct = 0; ct < N; ct += COLS) {
    const bool ok = spmm_tile_sub<P, VEC, SUB>(d.pos, d.crd, (const AV*)d.vals, (const BV*)d.x,
                                               (Out*)d.y, d.rows, N, c0, c1, u, ct, carry_row,
                                               carry_val);
    if constexpr (P::kChecked) {
      if (!__all_sync(0xffffffffu, ok)) batch_spmm_native<VEC, SUB>(d, N, c0, c1, u, ct, carry_row, carry_val);
    }
  }
}

#ifndef TACOGB_MM_BATCH_BLOCKS
#define TACOGB_MM_BATCH_BLOCKS 3  // resident blocks per SM the register budget is sized for
#endif
template <class P, int VEC, int SUB>
__global__ void __launch_bounds__(kMmBatchBlock, TACOGB_MM_BATCH_BLOCKS)
batch_spmm_kernel(const BatchDesc* __restrict__ desc, const int32_t* __restrict__ unit_off,
                  int count, int32_t total, int32_t N, const int2* __restrict__ part,
                  int32_t* __restrict__ carry_row, double* __restrict__ carry_val,
                  int32_t* __restrict__ unit_mat, int* __restrict__ counter,
                  long long* __restrict__ unit_cycles) {
  const int lane = threadIdx.x & 31;
  int c = 0;
  if (lane == 0) c = atomicAdd(counter, kMmChunk);
  c = __shfl_sync(0xffffffffu, c, 0);
  while (c < total) {
    int next = 0;
    if (lane == 0) next = atomicAdd(counter, kMmChunk);  // needed only when this chunk ends
    int m = find_matrix(unit_off, count, c);
    const int cend = min(c + kMmChunk, total);
    for (int u = c; u < cend; u++) {
      const long long t0 = clock64();
      while (u >= __ldg(unit_off + m + 1)) m++;
      const BatchDesc& d = desc[m];
      const int lu = u - d.unit0;
      const int2* p = part + d.part0;
      batch_spmm_unit<P, VEC, SUB>(d, N, p[lu], p[lu + 1], u, carry_row, carry_val);
      if (lane == 0) {
        const int32_t r = carry_row[u];  // written by this lane inside the tile
        carry_row[u] = r < d.rows ? r : -1;
        unit_mat[u] = m;
        unit_cycles[u] = clock64() - t0;
      }
    }
    c = __shfl_sync(0xffffffffu, next, 0);
  }
}

// One thread per (unit, column): the first unit of each run that ends inside the same row adds
// the run's carries in unit order.  Resets the work queue for the next launch.
template <typename Out>
__global__ void batch_spmm_fixup(const BatchDesc* __restrict__ desc, int32_t total, int32_t N,
                                 const int32_t* __restrict__ carry_row,
                                 const double* __restrict__ carry_val,
                                 const int32_t* __restrict__ unit_mat, int* __restrict__ counter) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx == 0) *counter = 0;
  const int64_t u = idx / N;
  const int32_t col = (int32_t)(idx % N);
  if (u >= total) return;
  const int32_t r = carry_row[u];
  if (r < 0) return;
  const int32_t m = unit_mat[u];
  if (u > 0 && carry_row[u - 1] == r && unit_mat[u - 1] == m) return;
  double tot = carry_val[u * N + col];
  for (int64_t v = u + 1; v < total && carry_row[v] == r && unit_mat[v] == m; v++)
    tot += carry_val[v * N + col];
  Out* c = (Out*)desc[m].y + (int64_t)r * N + col;
  *c = (Out)((double)*c + tot);
}

template <class P, int VEC, int SUB>
int batch_capture_spmm(tacogb_batch* b, int32_t N, int32_t total_blocks) {
  auto kern = batch_spmm_kernel<P, VEC, SUB>;
  int per_sm = 0;
  TACOGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMmBatchBlock, 0));
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
    kern<<<grid, kMmBatchBlock, 0, b->cap>>>(b->d_desc, b->d_unit_off, b->count, b->total_units,
                                             N, b->d_part, b->d_carry_row, b->d_carry_val,
                                             b->d_unit_mat, b->d_counter, b->d_unit_cycles);
    b->kernels_per_run++;
  }
  const int64_t fix = std::max<int64_t>((int64_t)b->total_units * N, 1);
  batch_spmm_fixup<typename P::Out><<<(unsigned)((fix + 255) / 256), 256, 0, b->cap>>>(
      b->d_desc, b->total_units, N, b->d_carry_row, b->d_carry_val, b->d_unit_mat, b->d_counter);
  b->kernels_per_run++;
  return batch_end_capture(b);
}

// Lane shape: full 16-byte vectors (VF = 16 / sizeof(B element)) when N allows and every B and
// C is 16-byte aligned, with the fewest lanes per B row that cover N (at least 4); otherwise
// single elements across the whole warp.
template <class P>
int batch_spmm_shape(tacogb_batch* b, int32_t N, int32_t blocks, bool full, int sub) {
  constexpr int VF = 16 / (int)sizeof(typename P::BV);
  if (full) {
    switch (sub) {
      case 8: return batch_capture_spmm<P, VF, 8>(b, N, blocks);
      case 4: return batch_capture_spmm<P, VF, 4>(b, N, blocks);
      case 2: return batch_capture_spmm<P, VF, 2>(b, N, blocks);
      default: return batch_capture_spmm<P, VF, 1>(b, N, blocks);
    }
  }
  return batch_capture_spmm<P, 1, 1>(b, N, blocks);
}

}  // namespace
}  // namespace tacogb

using namespace tacogb;

extern "C" int tacogb_batch_spmm_create(int32_t count, const tacogb_csr* mats, int32_t N,
                                        const void* const* B, int32_t btype, void* const* C,
                                        int32_t precision, tacogb_batch** out) {
  TACOGB_CHECK_ARG(out != nullptr, "batch: null output handle");
  *out = nullptr;
  TACOGB_CHECK_ARG(count > 0 && mats && B && C, "batch: empty or null batch");
  TACOGB_CHECK_ARG(N > 0, "batch: N must be positive");
  const int vt = mats[0].vtype;
  const bool f64 = vt == TACOGB_F64 && btype == TACOGB_F64;
  const bool f32 = vt == TACOGB_F32 && btype == TACOGB_F32;
  const bool bf16 = vt == TACOGB_F32 && btype == TACOGB_BF16;
  TACOGB_CHECK_ARG(f64 || f32 || bf16, "batch: unsupported value types (A %d, B %d)", vt, btype);
  TACOGB_CHECK_ARG(precision == 0 || (precision == 1 && !bf16),
                   "batch: precision %d (0 = default, 1 = native)", precision);
  const int esz = f64 ? 8 : (f32 ? 4 : 2), vf = 16 / esz;
  bool full = N % vf == 0;
  for (int m = 0; m < count && full; m++)
    full = ((uintptr_t)B[m] % 16) == 0 && ((uintptr_t)C[m] % 16) == 0;
  int sub = 1;
  if (full) {
    int lanes = 4;  // lanes per B row: the smallest power of two >= N / vf, at least 4
    while (lanes < 32 && lanes * vf < N) lanes <<= 1;
    sub = 32 / lanes;
  }
  std::vector<BatchDesc> desc(count);
  std::vector<int32_t> unit_off(count + 1), blk_off(count + 1);
  int64_t units = 0, parts = 0, blocks = 0;
  for (int m = 0; m < count; m++) {
    const tacogb_csr& A = mats[m];
    TACOGB_CHECK_ARG(A.vtype == vt, "batch: matrix %d has value type %d, expected %d", m, A.vtype, vt);
    TACOGB_CHECK_ARG(A.rows >= 0 && A.cols >= 0 && A.nnz >= 0 && A.nnz <= INT32_MAX,
                     "batch: matrix %d has a bad size", m);
    TACOGB_CHECK_ARG((int64_t)A.rows * N <= INT32_MAX,
                     "batch: matrix %d: rows*N exceeds taco's int32 dense positions", m);
    TACOGB_CHECK_ARG(A.rows == 0 || (A.pos && C[m]), "batch: matrix %d has null pos or C", m);
    TACOGB_CHECK_ARG(A.nnz == 0 || (A.crd && A.vals && B[m]), "batch: matrix %d has null arrays", m);
    BatchDesc& d = desc[m];
    d.pos = A.pos;
    d.crd = A.crd;
    d.vals = A.vals;
    d.x = B[m];
    d.y = C[m];
    d.rows = A.rows;
    d.cols = A.cols;
    d.nnz = (int32_t)A.nnz;
    d.tile = kMmBatchTile;
    d.snap = kMmBatchTile / 2;
    const int64_t u = ((int64_t)A.rows + A.nnz + kMmBatchTile - 1) / kMmBatchTile;
    d.unit0 = (int32_t)units;
    d.units = (int32_t)u;
    d.part0 = (int32_t)parts;
    d.blk0 = (int32_t)blocks;
    unit_off[m] = (int32_t)units;
    blk_off[m] = (int32_t)blocks;
    units += u;
    if (u > 0) {
      parts += u + 1;
      blocks += ((int64_t)A.rows + 1 + kPartBlock - 1) / kPartBlock;
    }
    TACOGB_CHECK_ARG(units < INT32_MAX / 2 && parts < INT32_MAX / 2 && blocks < INT32_MAX / 2,
                     "batch: too much work for one plan");
  }
  unit_off[count] = (int32_t)units;
  blk_off[count] = (int32_t)blocks;
  if (!device_status()) return last_code();
  tacogb_batch* b = new tacogb_batch();
  cudaGetDevice(&b->device);
  b->count = count;
  b->vt = vt;
  b->total_units = (int32_t)units;
  int rc = batch_alloc(b, desc.data(), unit_off.data(), blk_off.data(), parts, N, true);
  if (rc == 0) {
    const int32_t nb = (int32_t)blocks;
    if (f64) rc = precision == 1 ? batch_spmm_shape<MmNative64>(b, N, nb, full, sub)
                                 : batch_spmm_shape<MmDF64>(b, N, nb, full, sub);
    else if (f32) rc = precision == 1 ? batch_spmm_shape<MmF32>(b, N, nb, full, sub)
                                      : batch_spmm_shape<MmComp32>(b, N, nb, full, sub);
    else rc = batch_spmm_shape<MmBF16>(b, N, nb, full, sub);
  }
  if (rc) {
    batch_free(b);
    return rc;
  }
  *out = b;
  return 0;
}
