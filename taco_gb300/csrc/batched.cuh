// Shared parts of the batched plans (batched.cu: SpMV, batched_spmm.cu: SpMM): the per-matrix
// descriptor, the unit-to-matrix search, the merge partition over all matrices and the plan.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace tacogb {

constexpr int kPartBlock = 256;

struct BatchDesc {
  const int32_t* pos;
  const int32_t* crd;
  const void* vals;
  const void* x;
  void* y;
  int32_t rows, cols, nnz, kind;
  int32_t unit0, units;  // global unit range
  int32_t part0;         // first merge-partition entry (merge kinds: units + 1 entries)
  int32_t blk0;          // first block of the partition kernel (merge kinds)
  int32_t tma;           // 1 when pos/crd/vals are 16-byte aligned (required by merge kinds)
  int32_t tile;          // merge-tile items (0: not merge-partitioned)
  int32_t snap;          // rows shorter than this are never split between tiles (0: none)
};

// Largest m in [0, count) with off[m] <= u.
__device__ __forceinline__ int find_matrix(const int32_t* __restrict__ off, int count, int32_t u) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Merge-tile boundaries of every merge-kind matrix (the scatter partition of the single-matrix
// path, one block range per matrix).
static __global__ void batch_partition(const BatchDesc* __restrict__ desc,
                                const int32_t* __restrict__ blk_off, int count,
                                int2* __restrict__ part) {
  __shared__ int s_m;
  if (threadIdx.x == 0) s_m = find_matrix(blk_off, count, blockIdx.x);
  __syncthreads();
  const BatchDesc& d = desc[s_m];
  const int64_t i = (int64_t)(blockIdx.x - d.blk0) * blockDim.x + threadIdx.x;
  if (d.tile == 0 || i > d.rows) return;
  int2* p = part + d.part0;
  if (i == d.rows) {
    p[d.units] = make_int2(d.rows, d.nnz);
    return;
  }
  const uint32_t T = (uint32_t)d.tile;
  const int32_t p0 = __ldg(d.pos + i), p1 = __ldg(d.pos + i + 1);
  const uint32_t lo = (uint32_t)p0 + (uint32_t)i;
  const uint32_t hi = (uint32_t)p1 + (uint32_t)i;
  const bool snap = (p1 - p0) < d.snap;
  for (uint32_t b = lo / T + (lo % T != 0); (uint64_t)b * T <= hi && (int32_t)b < d.units; b++)
    p[b] = (snap && b > 0) ? make_int2((int)i + 1, p1)
                           : make_int2((int)i, (int)((uint64_t)b * T - (uint64_t)i));
}

void batch_free(struct ::tacogb_batch* b);
// Allocates and uploads a plan's arrays (descriptors, offsets, partition, carries of carry_cols
// doubles per unit, queue, cycle counters; unit matrix ids when with_unit_mat).
int batch_alloc(struct ::tacogb_batch* b, const BatchDesc* desc, const int32_t* unit_off,
                const int32_t* blk_off, int64_t parts, int64_t carry_cols, bool with_unit_mat);
// Ends the capture on b->cap, instantiates the graph.
int batch_end_capture(struct ::tacogb_batch* b);

}  // namespace tacogb

struct tacogb_batch {
  int device = 0;
  int count = 0;
  int vt = TACOGB_F64;
  int32_t total_units = 0;
  int kernels_per_run = 0;
  tacogb::BatchDesc* d_desc = nullptr;
  int32_t* d_unit_off = nullptr;
  int32_t* d_blk_off = nullptr;
  int2* d_part = nullptr;
  int32_t* d_carry_row = nullptr;
  double* d_carry_val = nullptr;
  int* d_counter = nullptr;
  long long* d_unit_cycles = nullptr;
  long long* d_mat_cycles = nullptr;
  int32_t* d_unit_mat = nullptr;  // SpMM plans: matrix of each unit
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};
