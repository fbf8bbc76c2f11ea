// CSR SpMV for sm_103a: y(i) = A(i,j) * x(j).
//
// Replaces the compute function taco generates for this statement: a row loop over
// A2_pos/A2_crd with a promoted scalar accumulator (src/lower/lowerer_impl_imperative.cpp:1304,
// src/index_notation/transformations.cpp:1982), and the GPU schedules of
// test/tests-scheduling-eval.cpp:193-247 (thread-per-row, warp-per-row, nnz-split with
// atomics + taco_binarySearchBeforeBlock, src/codegen/codegen_cuda.cpp:110-125).
//
// Two kernel families:
//
//  merge  Merge-path over the sequence (row ends, nonzeros): tile t owns merge items
//         [t*TILE, (t+1)*TILE), so every CTA does the same work whatever the row-length skew.
//         The CTA stages its nonzeros (vals and the gathered x[crd]) and its row ends in shared
//         memory with coalesced loads, then each thread walks IPT consecutive merge items and
//         accumulates with one FMA per nonzero.  A row split across threads is summed from
//         per-thread carries in shared memory; a row split across tiles gets its earlier part
//         from a tile carry-out that a fix-up kernel adds.  No atomics on values: results are
//         deterministic.  On GB300 the FP64 pipe issues about as many DFMA per clock as HBM
//         delivers nonzeros, so this family spends one FP64 op per nonzero plus one per
//         thread-boundary crossing, and no FP64 shuffle trees.
//  vector G lanes per row (G = 1 is thread-per-row, G = 32 is warp-per-row); lanes stride the
//         row with coalesced loads and combine with a shuffle butterfly.  Cheapest for short
//         regular rows; its log2(G) FP64 adds per row make it lose on long rows.
//
// FP64 values accumulate in FP64.  FP32 values accumulate with TwoProduct + TwoSum
// compensation (CompF32) and round once at the end.

#include <cstdio>

#include "common.cuh"
#include "kernels.h"

namespace tacogb {

// ------------------------------------------------------------------ accumulators ----------

template <typename V> struct Acc;

template <> struct Acc<double> {
  double v;
  __device__ __forceinline__ void zero() { v = 0.0; }
  __device__ __forceinline__ void add_prod(double a, double b) { v = __fma_rn(a, b, v); }
  __device__ __forceinline__ void add(const Acc& o) { v = __dadd_rn(v, o.v); }
  __device__ __forceinline__ void add_value(double o) { v = __dadd_rn(v, o); }
  __device__ __forceinline__ double result() const { return v; }
  __device__ __forceinline__ void shfl_xor_add(int m) {
    v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, m));
  }
};

template <> struct Acc<float> {
  CompF32 c;
  __device__ __forceinline__ void zero() { c.zero(); }
  __device__ __forceinline__ void add_prod(float a, float b) { c.add_prod(a, b); }
  __device__ __forceinline__ void add(const Acc& o) { c.add(o.c); }
  __device__ __forceinline__ void add_value(float o) {
    CompF32 t;
    t.hi = o;
    t.lo = 0.f;
    c.add(t);
  }
  __device__ __forceinline__ float result() const { return c.result(); }
  __device__ __forceinline__ void shfl_xor_add(int m) {
    CompF32 o;
    o.hi = __shfl_xor_sync(0xffffffffu, c.hi, m);
    o.lo = __shfl_xor_sync(0xffffffffu, c.lo, m);
    c.add(o);
  }
};

template <typename V>
__device__ __forceinline__ V ld_stream(const V* p);
template <>
__device__ __forceinline__ double ld_stream<double>(const double* p) { return ld_stream_f64(p); }
template <>
__device__ __forceinline__ float ld_stream<float>(const float* p) { return ld_stream_f32(p); }

// ------------------------------------------------------------------ merge path ------------

// Coordinate (rows ended, nonzeros consumed) of merge diagonal t*tile_items over the row ends
// pos[1..n] and the nonzero indices 0..nnz-1.  Row end r sorts before nonzero k iff
// pos[r+1] <= k.
__global__ void spmv_merge_partition(const int32_t* __restrict__ pos, int32_t n, int64_t nnz,
                                     int64_t tile_items, int32_t num_tiles,
                                     int2* __restrict__ part) {
  int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > num_tiles) return;
  int64_t total = (int64_t)n + nnz;
  int64_t d = (int64_t)t * tile_items;
  if (d > total) d = total;
  int64_t lo = d - nnz > 0 ? d - nnz : 0;
  int64_t hi = d < (int64_t)n ? d : (int64_t)n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if ((int64_t)__ldg(pos + mid + 1) <= d - mid - 1) lo = mid + 1; else hi = mid;
  }
  part[t] = make_int2((int)lo, (int)(d - lo));
}

template <typename V, int BLOCK, int IPT>
struct MergeSmem {
  static constexpr int TILE = BLOCK * IPT;
  static constexpr int LONG_RUN = 16;                 // carries summed serially up to this
  static constexpr int MAX_JOBS = BLOCK / LONG_RUN + 2;  // disjoint runs longer than LONG_RUN
  V v[TILE];
  V x[TILE];
  int32_t re[TILE];
  int32_t crow[BLOCK];
  Acc<V> cval[BLOCK];
  Acc<V> job_first[MAX_JOBS];
  int32_t job_a[MAX_JOBS], job_b[MAX_JOBS], job_dst[MAX_JOBS];
  int32_t njobs;
};

template <typename V, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK, 4)
spmv_merge_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                  const V* __restrict__ vals, const V* __restrict__ x, V* __restrict__ y,
                  const int2* __restrict__ part, int32_t* __restrict__ carry_row,
                  Acc<V>* __restrict__ carry_val) {
  using S = MergeSmem<V, BLOCK, IPT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);

  const int tid = threadIdx.x;
  const int tile = blockIdx.x;
  const int2 c0 = part[tile], c1 = part[tile + 1];
  const int r0 = c0.x, k0 = c0.y;
  const int rn = c1.x - c0.x, kn = c1.y - c0.y;
  if (tid == 0) s.njobs = 0;

  for (int j = tid; j < rn; j += BLOCK) s.re[j] = __ldg(pos + r0 + 1 + j);
  {
    int32_t cc[IPT];
    V vv[IPT];
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      int idx = tid + j * BLOCK;
      if (idx < kn) {
        cc[j] = ld_stream_i32(crd + k0 + idx);
        vv[j] = ld_stream<V>(vals + k0 + idx);
      }
    }
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      int idx = tid + j * BLOCK;
      if (idx < kn) {
        s.v[idx] = vv[j];
        s.x[idx] = __ldg(x + cc[j]);
      }
    }
  }
  __syncthreads();

  // This thread's start on the tile-local merge path.
  const int items = rn + kn;
  const int dt = min(tid * IPT, items);
  int lo = max(dt - kn, 0), hi = min(dt, rn);
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (s.re[mid] <= k0 + dt - mid - 1) lo = mid + 1; else hi = mid;
  }
  int row = lo, k = dt - lo;

  Acc<V> acc, first;
  acc.zero();
  first.zero();
  int first_row = -1;
#pragma unroll
  for (int it = 0; it < IPT; it++) {
    if (row < rn && s.re[row] <= k0 + k) {
      if (first_row < 0) {
        first_row = row;
        first = acc;
      } else {
        y[r0 + row] = acc.result();
      }
      acc.zero();
      row++;
    } else if (k < kn) {
      acc.add_prod(s.v[k], s.x[k]);
      k++;
    }
  }
  s.crow[tid] = r0 + row;  // row still open after this thread's items (n past the end)
  s.cval[tid] = acc;
  __syncthreads();

  // s.crow is non-decreasing in thread order, so the threads that ended inside one row form a
  // contiguous run; lower_bound finds its first thread.
  auto run_start = [&](int target, int limit) {
    int a = 0, b = limit;
    while (a < b) {
      int m = (a + b) >> 1;
      if (s.crow[m] < target) a = m + 1; else b = m;
    }
    return a;
  };
  auto push_job = [&](int a, int b, int dst, const Acc<V>& f) {
    int slot = atomicAdd(&s.njobs, 1);
    s.job_a[slot] = a;
    s.job_b[slot] = b;
    s.job_dst[slot] = dst;
    s.job_first[slot] = f;
  };

  // First completed row of this thread: its carries from the preceding threads plus `first`.
  if (first_row >= 0) {
    const int fr = r0 + first_row;
    const int a = run_start(fr, tid);
    if (tid - a <= S::LONG_RUN) {
      Acc<V> tot;
      tot.zero();
      for (int t = a; t < tid; t++) tot.add(s.cval[t]);
      tot.add(first);
      y[fr] = tot.result();
    } else {
      push_job(a, tid - 1, fr, first);
    }
  }
  // Tile carry-out: the run of threads whose open row is still open at the tile end.
  if (tid == BLOCK - 1) {
    const int cr = r0 + rn;
    const int a = run_start(cr, BLOCK - 1);
    Acc<V> zero;
    zero.zero();
    if (BLOCK - a <= S::LONG_RUN) {
      Acc<V> tot;
      tot.zero();
      for (int t = a; t < BLOCK; t++) tot.add(s.cval[t]);
      carry_row[tile] = cr;
      carry_val[tile] = tot;
    } else {
      push_job(a, BLOCK - 1, -1, zero);
    }
  }
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int njobs = s.njobs;
  for (int job = warp; job < njobs; job += BLOCK / 32) {
    const int a = s.job_a[job], b = s.job_b[job];
    Acc<V> part;
    part.zero();
    for (int t = a + lane; t <= b; t += 32) part.add(s.cval[t]);
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) part.shfl_xor_add(m);
    if (lane == 0) {
      part.add(s.job_first[job]);
      const int dst = s.job_dst[job];
      if (dst >= 0) {
        y[dst] = part.result();
      } else {
        carry_row[tile] = r0 + rn;
        carry_val[tile] = part;
      }
    }
  }
}

// Adds the tile carry-outs to the rows that continue into later tiles.  Tiles carrying the same
// row are consecutive; the first tile of each run sums the run in tile order.
template <typename V>
__global__ void spmv_merge_fixup(const int32_t* __restrict__ carry_row,
                                 const Acc<V>* __restrict__ carry_val, int32_t num_tiles,
                                 V* __restrict__ y, int32_t n) {
  int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= num_tiles) return;
  const int32_t r = carry_row[t];
  if (r >= n) return;
  if (t > 0 && carry_row[t - 1] == r) return;
  Acc<V> tot = carry_val[t];
  for (int32_t u = t + 1; u < num_tiles && carry_row[u] == r; u++) tot.add(carry_val[u]);
  tot.add_value(y[r]);
  y[r] = tot.result();
}

// ------------------------------------------------------------------ vector ----------------

template <typename V, int G>
__global__ void __launch_bounds__(256)
spmv_vector_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                   const V* __restrict__ vals, const V* __restrict__ x, V* __restrict__ y,
                   int32_t n) {
  const int lane = threadIdx.x & (G - 1);
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  // Every lane of a warp runs the same number of outer iterations so that the shuffles below
  // always see the full warp.
  const int64_t warp_first = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll) / G;
  for (int64_t base = warp_first; base < n; base += ngroups) {
    const int64_t row = base + (gid - warp_first);
    Acc<V> acc;
    acc.zero();
    if (row < n) {
      const int32_t p1 = __ldg(pos + row + 1);
      for (int32_t p = __ldg(pos + row) + lane; p < p1; p += G)
        acc.add_prod(ld_stream<V>(vals + p), __ldg(x + ld_stream_i32(crd + p)));
    }
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) acc.shfl_xor_add(m);
    if (row < n && lane == 0) y[row] = acc.result();
  }
}

// ------------------------------------------------------------------ host side -------------

namespace {

struct SpmvVariant {
  const char* name;
  int family;  // 0 merge, 1 vector
  int param;   // IPT for merge, G for vector
};

const SpmvVariant kSpmvVariants[] = {
    {"merge_ipt5", 0, 5},   {"merge_ipt7", 0, 7},   {"merge_ipt11", 0, 11},
    {"vector_g1", 1, 1},    {"vector_g2", 1, 2},    {"vector_g4", 1, 4},
    {"vector_g8", 1, 8},    {"vector_g16", 1, 16},  {"vector_g32", 1, 32},
};
constexpr int kNumSpmvVariants = sizeof(kSpmvVariants) / sizeof(kSpmvVariants[0]);
constexpr int kMergeBlock = 256;

template <typename V, int IPT>
int launch_merge(const tacogb_csr* A, const V* x, V* y, cudaStream_t st) {
  using S = MergeSmem<V, kMergeBlock, IPT>;
  const int64_t tile_items = S::TILE;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + tile_items - 1) / tile_items;
  if (tiles64 == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31), "SpMV: too many merge tiles");
  const int32_t tiles = (int32_t)tiles64;
  const size_t part_bytes = ((size_t)tiles + 1) * sizeof(int2);
  const size_t crow_bytes = (size_t)tiles * sizeof(int32_t);
  const size_t cval_bytes = (size_t)tiles * sizeof(Acc<V>);
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + 256, 0);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  Acc<V>* cval = (Acc<V>*)(ws + ((part_bytes + crow_bytes + 15) & ~(size_t)15));

  TACOGB_LAUNCH("spmv_merge_partition", st,
                spmv_merge_partition<<<(tiles + 1 + 255) / 256, 256, 0, st>>>(
                    A->pos, A->rows, A->nnz, tile_items, tiles, part));
  auto kern = spmv_merge_kernel<V, kMergeBlock, IPT>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(S)));
  TACOGB_LAUNCH("spmv_merge_kernel", st,
                kern<<<tiles, kMergeBlock, sizeof(S), st>>>(A->pos, A->crd, (const V*)A->vals, x,
                                                           y, part, crow, cval));
  TACOGB_LAUNCH("spmv_merge_fixup", st,
                spmv_merge_fixup<V><<<(tiles + 255) / 256, 256, 0, st>>>(crow, cval, tiles, y,
                                                                         A->rows));
  return 0;
}

template <typename V, int G>
int launch_vector(const tacogb_csr* A, const V* x, V* y, cudaStream_t st) {
  if (A->rows == 0) return 0;
  const int64_t threads = (int64_t)A->rows * G;
  int64_t blocks = (threads + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  TACOGB_LAUNCH("spmv_vector_kernel", st,
                spmv_vector_kernel<V, G><<<(int)blocks, 256, 0, st>>>(
                    A->pos, A->crd, (const V*)A->vals, x, y, A->rows));
  return 0;
}

template <typename V>
int spmv_typed(const tacogb_csr* A, const V* x, V* y, int variant, cudaStream_t st) {
  const SpmvVariant& v = kSpmvVariants[variant];
  if (v.family == 0) {
    switch (v.param) {
      case 5: return launch_merge<V, 5>(A, x, y, st);
      case 7: return launch_merge<V, 7>(A, x, y, st);
      case 11: return launch_merge<V, 11>(A, x, y, st);
    }
  } else {
    switch (v.param) {
      case 1: return launch_vector<V, 1>(A, x, y, st);
      case 2: return launch_vector<V, 2>(A, x, y, st);
      case 4: return launch_vector<V, 4>(A, x, y, st);
      case 8: return launch_vector<V, 8>(A, x, y, st);
      case 16: return launch_vector<V, 16>(A, x, y, st);
      case 32: return launch_vector<V, 32>(A, x, y, st);
    }
  }
  set_error(TACOGB_ERR_ARG, "SpMV: bad variant %d", variant);
  return TACOGB_ERR_ARG;
}

}  // namespace

int spmv_variant_count() { return kNumSpmvVariants; }
const char* spmv_variant_name(int v) {
  return (v >= 0 && v < kNumSpmvVariants) ? kSpmvVariants[v].name : "";
}

// Structural rule used when neither a tuning record nor the cost model gives a choice: the
// merge family is robust to any skew; regular short rows go to thread/sub-warp per row.
int spmv_default_variant(const tacogb_csr* A) {
  (void)A;
  return 1;  // merge_ipt7
}

int spmv_run(const tacogb_csr* A, const void* x, void* y, int variant, cudaStream_t st) {
  TACOGB_CHECK_ARG(A != nullptr && x != nullptr && y != nullptr, "SpMV: null argument");
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->nnz >= 0, "SpMV: negative size");
  TACOGB_CHECK_ARG(A->nnz <= INT32_MAX, "SpMV: nnz exceeds int32 positions");
  TACOGB_CHECK_ARG(A->rows == 0 || A->pos != nullptr, "SpMV: null pos");
  TACOGB_CHECK_ARG(A->nnz == 0 || (A->crd != nullptr && A->vals != nullptr),
                   "SpMV: null crd/vals");
  if (variant < 0) variant = spmv_default_variant(A);
  TACOGB_CHECK_ARG(variant < kNumSpmvVariants, "SpMV: variant %d out of range", variant);
  if (A->vtype == TACOGB_F64)
    return spmv_typed<double>(A, (const double*)x, (double*)y, variant, st);
  if (A->vtype == TACOGB_F32)
    return spmv_typed<float>(A, (const float*)x, (float*)y, variant, st);
  set_error(TACOGB_ERR_ARG, "SpMV: unsupported value type %d", A->vtype);
  return TACOGB_ERR_ARG;
}

}  // namespace tacogb
