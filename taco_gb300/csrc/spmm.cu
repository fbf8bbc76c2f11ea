// CSR x dense SpMM for sm_103a: C(i,k) = A(i,j) * B(j,k), B and C dense row-major.
//
// Replaces the compute function taco generates for this statement (zero C, then for i, for p in
// row i, for k: C[i*N+k] += A[p] * B[crd[p]*N+k]; src/lower/lowerer_impl_imperative.cpp:1304
// over the CSR operand with a dense k loop) and the GPU schedules of
// test/tests-scheduling-eval.cpp:249-370 (nnz-split with one FP64 atomicAdd per product into a
// column-major C, N <= 128).
//
// Work unit: a merge-path tile of W items over (row ends, nonzeros), so every warp does the
// same amount of work whatever the row-length skew.  Boundaries that would split a row shorter
// than W/2 move to that row's end, so only long rows are shared between tiles; their partial
// rows go to a carry buffer that a fix-up kernel adds in tile order (deterministic, no atomics).
// Each warp owns one tile and one column tile of 32*VEC columns: per nonzero, every lane loads
// VEC consecutive B elements (a 16-byte vector when N allows), so a warp reads a contiguous
// slice of the gathered B row; crd/vals are loaded 32 at a time and broadcast with shuffles,
// and U nonzeros are unrolled so U B rows are in flight per warp.  Every row of C is written
// exactly once by the tile holding its row end (empty rows write zeros), so C needs no
// zero-fill pass.
//
// Accumulation policies:
//   F64 values/B  native: DFMA.  df: double-float on the FP32 pipe (see df.cuh), with a warp
//                 tile recomputed natively when a value falls outside the double-float range.
//   F32 values/B  native: FFMA.  df: TwoProduct/TwoSum-compensated FP32.
//   F32 values, BF16 B: FFMA in FP32 (B converted by a shift), C in FP32.

#include <cstdio>
#include <type_traits>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "spmm_tile.cuh"

namespace tacogb {

template <class P, int VEC>
__global__ void __launch_bounds__(kMmBlock, 3)
spmm_merge_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                  const typename P::AV* __restrict__ vals, const typename P::BV* __restrict__ B,
                  typename P::Out* __restrict__ C, int32_t n, int32_t N,
                  const int2* __restrict__ part, int32_t tiles, int32_t* __restrict__ carry_row,
                  double* __restrict__ carry_val) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * kMmWarps + warp;
  if (tile >= tiles) return;
  const int col0 = blockIdx.y * (32 * VEC) + lane * VEC;
  const bool active = col0 < N;
  const int2 c0 = part[tile], c1 = part[tile + 1];
  const bool ok = spmm_tile<P, VEC>(pos, crd, vals, B, C, n, N, c0, c1, tile, col0, active,
                                    carry_row, carry_val);
  if constexpr (P::kChecked) {
    if (!__all_sync(0xffffffffu, ok))
      spmm_tile<MmNative64, VEC>(pos, crd, vals, B, C, n, N, c0, c1, tile, col0, active,
                                 carry_row, carry_val);
  }
}

// Adds carried partial rows, in tile order, into the row where each run of tiles ends.
template <typename Out>
__global__ void spmm_carry_fixup(const int32_t* __restrict__ carry_row,
                                 const double* __restrict__ carry_val, int32_t tiles, int32_t N,
                                 Out* __restrict__ C, int32_t n) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t t = idx / N;
  const int32_t col = (int32_t)(idx % N);
  if (t >= tiles) return;
  const int32_t r = carry_row[t];
  if (r >= n) return;
  if (t > 0 && carry_row[t - 1] == r) return;
  double tot = carry_val[t * N + col];
  for (int64_t u = t + 1; u < tiles && carry_row[u] == r; u++) tot += carry_val[u * N + col];
  Out* c = C + (int64_t)r * N + col;
  *c = (Out)((double)*c + tot);
}

// ------------------------------------------------------------------ host side -------------

namespace {

struct SpmmVariant {
  const char* name;
  bool df;          // double-float (F64) / compensated (F32) accumulation
  int tile_items;   // W
};

const SpmmVariant kSpmmVariants[] = {
    {"merge_w512_native", false, 512},
    {"merge_w512_df", true, 512},
    {"merge_w256_native", false, 256},
    {"merge_w256_df", true, 256},
};
constexpr int kNumSpmmVariants = sizeof(kSpmmVariants) / sizeof(kSpmmVariants[0]);

template <class P, int VEC>
int launch_spmm(const tacogb_csr* A, int32_t N, const void* B, void* C, int W, cudaStream_t st) {
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + W - 1) / W;
  if (tiles64 == 0 || N == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) / kMmWarps, "SpMM: too many tiles");
  const int32_t tiles = (int32_t)tiles64;
  const size_t part_bytes = (((size_t)tiles + 1) * sizeof(int2) + 255) & ~(size_t)255;
  const size_t crow_bytes = ((size_t)tiles * sizeof(int32_t) + 255) & ~(size_t)255;
  const size_t cval_bytes = (size_t)tiles * (size_t)N * sizeof(double);
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes, 1);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  if (int rc = merge_partition(A->pos, A->rows, A->nnz, W, tiles, part, st, W / 2)) return rc;
  constexpr int TW = 32 * VEC;
  dim3 grid((unsigned)((tiles + kMmWarps - 1) / kMmWarps), (unsigned)((N + TW - 1) / TW));
  TACOGB_CHECK_ARG(grid.y <= 65535, "SpMM: N too large");
  TACOGB_LAUNCH("spmm_merge_kernel", st,
                (spmm_merge_kernel<P, VEC><<<grid, kMmBlock, 0, st>>>(
                    A->pos, A->crd, (const typename P::AV*)A->vals,
                    (const typename P::BV*)B, (typename P::Out*)C, A->rows, N, part, tiles, crow,
                    cval)));
  const int64_t fix_threads = (int64_t)tiles * N;
  TACOGB_LAUNCH("spmm_carry_fixup", st,
                spmm_carry_fixup<typename P::Out><<<(unsigned)((fix_threads + 255) / 256), 256, 0,
                                                    st>>>(crow, cval, tiles, N,
                                                          (typename P::Out*)C, A->rows));
  return 0;
}

// Widest lane vector (up to 16 bytes) whose column tile divides N.
template <class P>
int spmm_dispatch_vec(const tacogb_csr* A, int32_t N, const void* B, void* C, int W,
                      cudaStream_t st) {
  constexpr int esz = sizeof(typename P::BV);
  if constexpr (esz == 8) {
    if (N % 64 == 0) return launch_spmm<P, 2>(A, N, B, C, W, st);
    return launch_spmm<P, 1>(A, N, B, C, W, st);
  } else if constexpr (esz == 4) {
    if (N % 128 == 0) return launch_spmm<P, 4>(A, N, B, C, W, st);
    if (N % 64 == 0) return launch_spmm<P, 2>(A, N, B, C, W, st);
    return launch_spmm<P, 1>(A, N, B, C, W, st);
  } else {
    if (N % 256 == 0) return launch_spmm<P, 8>(A, N, B, C, W, st);
    if (N % 128 == 0) return launch_spmm<P, 4>(A, N, B, C, W, st);
    if (N % 64 == 0) return launch_spmm<P, 2>(A, N, B, C, W, st);
    return launch_spmm<P, 1>(A, N, B, C, W, st);
  }
}

}  // namespace

int spmm_variant_count() { return kNumSpmmVariants; }
const char* spmm_variant_name(int v) {
  return (v >= 0 && v < kNumSpmmVariants) ? kSpmmVariants[v].name : "";
}

int spmm_run(const tacogb_csr* A, int32_t N, const void* B, int32_t btype, void* C, int variant,
             cudaStream_t st) {
  TACOGB_CHECK_ARG(A != nullptr, "SpMM: null matrix");
  TACOGB_CHECK_ARG((int64_t)A->rows * N == 0 || C != nullptr, "SpMM: null C");
  TACOGB_CHECK_ARG(A->nnz == 0 || N == 0 || B != nullptr, "SpMM: null B");
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->nnz >= 0 && N >= 0, "SpMM: negative size");
  TACOGB_CHECK_ARG(A->nnz <= INT32_MAX, "SpMM: nnz exceeds int32 positions");
  TACOGB_CHECK_ARG((int64_t)A->rows * N <= INT32_MAX,
                   "SpMM: rows*N exceeds taco's int32 dense positions");
  TACOGB_CHECK_ARG(A->rows == 0 || A->pos != nullptr, "SpMM: null pos");
  if (variant < 0) variant = 1;
  TACOGB_CHECK_ARG(variant < kNumSpmmVariants, "SpMM: variant %d out of range", variant);
  const SpmmVariant& v = kSpmmVariants[variant];
  if (A->vtype == TACOGB_F64 && btype == TACOGB_F64)
    return v.df ? spmm_dispatch_vec<MmDF64>(A, N, B, C, v.tile_items, st)
                : spmm_dispatch_vec<MmNative64>(A, N, B, C, v.tile_items, st);
  if (A->vtype == TACOGB_F32 && btype == TACOGB_F32)
    return v.df ? spmm_dispatch_vec<MmComp32>(A, N, B, C, v.tile_items, st)
                : spmm_dispatch_vec<MmF32>(A, N, B, C, v.tile_items, st);
  if (A->vtype == TACOGB_F32 && btype == TACOGB_BF16)
    return spmm_dispatch_vec<MmBF16>(A, N, B, C, v.tile_items, st);
  set_error(TACOGB_ERR_ARG, "SpMM: unsupported value types (A %d, B %d)", A->vtype, btype);
  return TACOGB_ERR_ARG;
}

}  // namespace tacogb
