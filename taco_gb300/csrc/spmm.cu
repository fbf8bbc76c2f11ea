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

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "spmm_tile.cuh"

namespace tacogb {

// B64: B as FP64 for the native redo of checked policies (the same array as B unless B was
// pre-split); bflag (optional): non-zero when B has entries outside the double-float range.
// CTAs per SM the merge kernel is compiled for: four (64 registers) except the compensated FP32
// tile four columns wide, which spills there.  Measured against three: FP64 N=64 3.36 -> 3.29
// ms, BF16 N=64 1.88 -> 1.58 ms, MTTKRP's fiber SpMM 4.01 -> 3.59 ms; FP32 N=256 7.67 -> 8.82
// ms with four, hence three for that tile.
template <class P, int VEC>
constexpr int mm_min_blocks() {
  return (std::is_same<P, MmComp32>::value && VEC == 4) ? 3 : 4;
}

template <class P, int VEC, bool STREAM>
__global__ void __launch_bounds__(kMmBlock, mm_min_blocks<P, VEC>())
spmm_merge_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                  const typename P::AV* __restrict__ vals, const typename P::BV* __restrict__ B,
                  const double* __restrict__ B64, const int* __restrict__ bflag,
                  typename P::Out* __restrict__ C, int32_t n, int32_t N,
                  const int2* __restrict__ part, int32_t tiles, int32_t* __restrict__ carry_row,
                  double* __restrict__ carry_val) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * kMmWarps + warp;
  if (tile >= tiles) return;
  const int col0 = blockIdx.y * (32 * VEC) + lane * VEC;
  const bool active = col0 < N;
  const int2 c0 = part[tile], c1 = part[tile + 1];
  bool ok = !P::kChecked || bflag == nullptr || *bflag == 0;
  if (ok) {
    if constexpr (STREAM)
      ok = spmm_tile_stream<P, VEC>(pos, crd, vals, B, C, n, N, c0, c1, tile, col0, active,
                                    carry_row, carry_val);
    else
      ok = spmm_tile<P, VEC>(pos, crd, vals, B, C, n, N, c0, c1, tile, col0, active, carry_row,
                             carry_val);
  }
  if constexpr (P::kChecked) {
    if (!__all_sync(0xffffffffu, ok)) {
      if constexpr (STREAM)
        spmm_tile_stream<MmNative64, VEC>(pos, crd, (const double*)vals, B64, (double*)C, n, N,
                                          c0, c1, tile, col0, active, carry_row, carry_val);
      else
        spmm_tile<MmNative64, VEC>(pos, crd, (const double*)vals, B64, (double*)C, n, N, c0, c1,
                                   tile, col0, active, carry_row, carry_val);
    }
  }
}

// The TMA-staged warp tile (spmm_tile_tma): one ring of S B-row slots per warp in dynamic
// shared memory.  Checked policies redo a tile natively (register-staged stream tile) when a
// value or B entry is out of range.
template <class P, int VEC, int S>
__global__ void __launch_bounds__(kMmBlock, 3)
spmm_tma_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                const typename P::AV* __restrict__ vals, const typename P::BV* __restrict__ B,
                const double* __restrict__ B64, const int* __restrict__ bflag,
                typename P::Out* __restrict__ C, int32_t n, int32_t N,
                const int2* __restrict__ part, int32_t tiles, int32_t* __restrict__ carry_row,
                double* __restrict__ carry_val, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * kMmWarps + warp;
  if (tile >= tiles) return;
  MmRing<P, VEC, S>& ring = reinterpret_cast<MmRing<P, VEC, S>*>(smem_raw)[warp];
  const int colt = blockIdx.y * (32 * VEC);
  const int2 c0 = part[tile], c1 = part[tile + 1];
  bool ok = !P::kChecked || bflag == nullptr || *bflag == 0;
  if (ok)
    ok = spmm_tile_tma<P, VEC, S>(ring, pos, crd, vals, B, C, n, N, c0, c1, tile, colt, status,
                                  carry_row, carry_val);
  if constexpr (P::kChecked) {
    if (!__all_sync(0xffffffffu, ok))
      spmm_tile_stream<MmNative64, VEC>(pos, crd, (const double*)vals, B64, (double*)C, n, N, c0,
                                        c1, tile, colt + lane * VEC, true, carry_row, carry_val);
  }
}

// Adds carried partial rows, in tile order, into the row where each run of tiles ends.
// bflag (optional) is the B-range flag of the product, cleared here for the next one.
template <typename Out>
__global__ void spmm_carry_fixup(const int32_t* __restrict__ carry_row,
                                 const double* __restrict__ carry_val, int32_t tiles, int32_t N,
                                 Out* __restrict__ C, int32_t n, int* __restrict__ bflag = nullptr) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx == 0 && bflag != nullptr) *bflag = 0;
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

// Splits B (count doubles, count even, both arrays 16-byte aligned) into double-float pairs,
// two elements per thread, setting *bflag when an element lies outside the pairs' range (the
// product then runs every tile natively).  *bflag is cleared by the fix-up kernel.
__global__ void spmm_split_b(const double* __restrict__ B, DF* __restrict__ Bdf, int64_t count,
                             int* __restrict__ bflag) {
  const int64_t i = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= count) return;
  const double2 v = __ldg(reinterpret_cast<const double2*>(B + i));
  float4 o;
  const bool ok = split_df(v.x, o.x, o.y) & split_df(v.y, o.z, o.w);
  *reinterpret_cast<float4*>(Bdf + i) = o;
  if (!ok) *bflag = 1;
}

// Sub-warp SpMM (spmm_tile_sub): warp `tile` of the merge partition, column slab blockIdx.y of
// LPR*VEC columns.  Blocks run slab by slab (blockIdx.x fastest), so the slab of B being
// gathered stays in L2 while A streams past once per slab.  Checked policies redo a tile with
// DFMA on the FP64 B (B64) when a value or a B entry (*bflag) is out of range.
template <class P, int VEC, int SUB, int LONG>
__global__ void __launch_bounds__(kMmBlock, 3)
spmm_sub_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                const typename P::AV* __restrict__ vals, const typename P::BV* __restrict__ B,
                const double* __restrict__ B64, const int* __restrict__ bflag,
                typename P::Out* __restrict__ C, int32_t n, int32_t N,
                const int2* __restrict__ part, int32_t tiles, int32_t* __restrict__ carry_row,
                double* __restrict__ carry_val) {
  constexpr int LPR = 32 / SUB;
  const int warp = threadIdx.x >> 5;
  const int tile = blockIdx.x * kMmWarps + warp;
  if (tile >= tiles) return;
  const int ct = blockIdx.y * (LPR * VEC);
  const int2 c0 = part[tile], c1 = part[tile + 1];
  bool ok = !P::kChecked || bflag == nullptr || *bflag == 0;
  if (ok)
    ok = spmm_tile_sub<P, VEC, SUB, LONG>(pos, crd, vals, B, C, n, N, c0, c1, tile, ct,
                                          carry_row, carry_val);
  if constexpr (P::kChecked) {
    if (!__all_sync(0xffffffffu, ok))
      spmm_tile_sub<MmNative64, VEC, SUB, LONG>(pos, crd, (const double*)vals, B64, (double*)C, n,
                                                N, c0, c1, tile, ct, carry_row, carry_val);
  }
}

// ------------------------------------------------------------------ host side -------------

namespace {

struct SpmmVariant {
  const char* name;
  int df;           // 0 native, 1 double-float (F64) / compensated (F32), 2 double-float over a
                    // pre-split B (F64; compensated for F32)
  int tile_items;   // W
  int lpr;          // 0: warp tile (spmm_tile); else sub-warp tile with LPR lanes per B row
  bool shared;      // sub-warp tile: every row shared by the whole warp (column slabs)
  bool stream;      // warp tile walked as one stream of nonzeros (spmm_tile_stream)
  int tma;          // > 0: streaming tile with B rows staged by bulk copies, this many in flight
};

const SpmmVariant kSpmmVariants[] = {
    {"merge_w512_native", 0, 512, 0},
    {"merge_w512_df", 1, 512, 0},
    {"merge_w256_native", 0, 256, 0},
    {"merge_w256_df", 1, 256, 0},
    {"sub8_w512_native", 0, 512, 8},
    {"sub8_w512_dfs", 2, 512, 8},
    {"sub4_w512_native", 0, 512, 4},
    {"sub4_w512_dfs", 2, 512, 4},
    {"merge_w512_dfs", 2, 512, 0},
    {"merge_w256_dfs", 2, 256, 0},
    {"slab8_w512_native", 0, 512, 8, true},
    {"slab8_w512_dfs", 2, 512, 8, true},
    {"slab4_w512_native", 0, 512, 4, true},
    {"slab4_w512_dfs", 2, 512, 4, true},
    {"stream_w512_native", 0, 512, 0, false, true},
    {"stream_w512_dfs", 2, 512, 0, false, true},
    {"stream_w1024_dfs", 2, 1024, 0, false, true},
    {"tma12_w512_dfs", 2, 512, 0, false, true, 12},
    {"tma16_w512_dfs", 2, 512, 0, false, true, 16},
    {"tma12_w512_native", 0, 512, 0, false, true, 12},
    {"tma12_w512_df", 1, 512, 0, false, true, 12},
};
constexpr int kNumSpmmVariants = sizeof(kSpmmVariants) / sizeof(kSpmmVariants[0]);

// presplit/pflag (MmDFS only): B already split into double-float pairs, with its range flag,
// by spmm_split_once for several products; the fix-up then leaves the flag alone.
template <class P, int VEC, bool STREAM, int TMA = 0>
int launch_spmm(const tacogb_csr* A, int32_t N, const void* B, void* C, int W, cudaStream_t st,
                const void* presplit = nullptr, int* pflag = nullptr, int slot = 1) {
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + W - 1) / W;
  if (tiles64 == 0 || N == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) / kMmWarps, "SpMM: too many tiles");
  const int32_t tiles = (int32_t)tiles64;
  const size_t part_bytes = (((size_t)tiles + 1) * sizeof(int2) + 255) & ~(size_t)255;
  const size_t crow_bytes = ((size_t)tiles * sizeof(int32_t) + 255) & ~(size_t)255;
  const size_t cval_bytes = (((size_t)tiles * (size_t)N * sizeof(double)) + 255) & ~(size_t)255;
  constexpr bool split = std::is_same<P, MmDFS>::value;
  const size_t bdf_bytes =
      split && presplit == nullptr ? (size_t)A->cols * (size_t)N * sizeof(DF) : 0;
  unsigned char* ws =
      (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + bdf_bytes, slot);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  const typename P::BV* Bk = (const typename P::BV*)B;
  int* bflag = nullptr;
  int* clear_flag = nullptr;  // the flag the fix-up clears (this call's own split only)
  if (split && presplit != nullptr) {
    Bk = (const typename P::BV*)presplit;
    bflag = pflag;
  } else if constexpr (split) {
    // B split once into double-float pairs: every B element is then used about nnz/cols times
    int* status = device_status();
    if (!status) return last_code();
    bflag = status + kBFlagWord;
    DF* bdf = (DF*)(ws + part_bytes + crow_bytes + cval_bytes);
    const int64_t count = (int64_t)A->cols * N;  // even: N is even whenever VEC is 2
    if (count > 0)
      TACOGB_LAUNCH("spmm_split_b", st,
                    spmm_split_b<<<(unsigned)((count / 2 + 255) / 256), 256, 0, st>>>(
                        (const double*)B, bdf, count, bflag));
    Bk = (const typename P::BV*)bdf;
    clear_flag = bflag;
  }
  if (int rc = merge_partition(A->pos, A->rows, A->nnz, W, tiles, part, st, W / 2)) return rc;
  constexpr int TW = 32 * VEC;
  dim3 grid((unsigned)((tiles + kMmWarps - 1) / kMmWarps), (unsigned)((N + TW - 1) / TW));
  TACOGB_CHECK_ARG(grid.y <= 65535, "SpMM: N too large");
  if constexpr (TMA > 0) {
    int* status = device_status();
    if (!status) return last_code();
    auto kern = spmm_tma_kernel<P, VEC, TMA>;
    const int smem = (int)(sizeof(MmRing<P, VEC, TMA>) * kMmWarps);
    TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    // room for the three CTAs per SM the registers allow
    const int pct = std::min(100, (3 * smem * 100 + 228 * 1024 - 1) / (228 * 1024));
    TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, pct));
    TACOGB_LAUNCH("spmm_tma_kernel", st,
                  (kern<<<grid, kMmBlock, smem, st>>>(
                      A->pos, A->crd, (const typename P::AV*)A->vals, Bk, (const double*)B, bflag,
                      (typename P::Out*)C, A->rows, N, part, tiles, crow, cval, status)));
  } else {
    TACOGB_LAUNCH("spmm_merge_kernel", st,
                  (spmm_merge_kernel<P, VEC, STREAM><<<grid, kMmBlock, 0, st>>>(
                      A->pos, A->crd, (const typename P::AV*)A->vals, Bk, (const double*)B,
                      bflag, (typename P::Out*)C, A->rows, N, part, tiles, crow, cval)));
  }
  const int64_t fix_threads = (int64_t)tiles * N;
  TACOGB_LAUNCH("spmm_carry_fixup", st,
                spmm_carry_fixup<typename P::Out><<<(unsigned)((fix_threads + 255) / 256), 256, 0,
                                                    st>>>(crow, cval, tiles, N,
                                                          (typename P::Out*)C, A->rows,
                                                          clear_flag));
  return 0;
}

__global__ void spmm_flag_clear(int* flag) { *flag = 0; }

// Sub-warp SpMM over column slabs.  For MmDFS, B is first split into double-float pairs in
// scratch (one pass over B; every B element is then used about nnz/cols times without further
// splitting).
template <class P, int VEC, int SUB, int LONG>
int launch_spmm_sub(const tacogb_csr* A, int32_t N, const void* B, void* C, int W,
                    cudaStream_t st) {
  constexpr int LPR = 32 / SUB;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + W - 1) / W;
  if (tiles64 == 0 || N == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) / kMmWarps, "SpMM: too many tiles");
  const int32_t tiles = (int32_t)tiles64;
  constexpr bool split = std::is_same<P, MmDFS>::value;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const size_t crow_bytes = al((size_t)tiles * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)tiles * (size_t)N * sizeof(double));
  const size_t bdf_bytes = split ? al((size_t)A->cols * (size_t)N * sizeof(DF)) : 0;
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + bdf_bytes, 1);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  const typename P::BV* Bk = (const typename P::BV*)B;
  int* bflag = nullptr;
  if constexpr (split) {
    int* status = device_status();
    if (!status) return last_code();
    bflag = status + kBFlagWord;
    DF* bdf = (DF*)(ws + part_bytes + crow_bytes + cval_bytes);
    const int64_t count = (int64_t)A->cols * N;  // even: N is even for 16-byte vectors
    if (count > 0)
      TACOGB_LAUNCH("spmm_split_b", st,
                    spmm_split_b<<<(unsigned)((count / 2 + 255) / 256), 256, 0, st>>>(
                        (const double*)B, bdf, count, bflag));
    Bk = (const typename P::BV*)bdf;
  }
  if (int rc = merge_partition(A->pos, A->rows, A->nnz, W, tiles, part, st, W / 2)) return rc;
  dim3 grid((unsigned)((tiles + kMmWarps - 1) / kMmWarps),
            (unsigned)((N + LPR * VEC - 1) / (LPR * VEC)));
  TACOGB_CHECK_ARG(grid.y <= 65535, "SpMM: N too large");
  TACOGB_LAUNCH("spmm_sub_kernel", st,
                (spmm_sub_kernel<P, VEC, SUB, LONG><<<grid, kMmBlock, 0, st>>>(
                    A->pos, A->crd, (const typename P::AV*)A->vals, Bk, (const double*)B, bflag,
                    (typename P::Out*)C, A->rows, N, part, tiles, crow, cval)));
  const int64_t fix_threads = (int64_t)tiles * N;
  TACOGB_LAUNCH("spmm_carry_fixup", st,
                spmm_carry_fixup<typename P::Out><<<(unsigned)((fix_threads + 255) / 256), 256, 0,
                                                    st>>>(crow, cval, tiles, N,
                                                          (typename P::Out*)C, A->rows, bflag));
  return 0;
}

// Sub-warp variants: 16-byte lane vectors when N and B's alignment allow, else one element.
template <class P, int LPR, int LONG>
int spmm_dispatch_sub(const tacogb_csr* A, int32_t N, const void* B, void* C, int W,
                      cudaStream_t st) {
  constexpr int SUB = 32 / LPR;
  constexpr int esz = sizeof(typename std::conditional<std::is_same<P, MmDFS>::value, double,
                                                       typename P::BV>::type);
  constexpr int V16 = 16 / esz;
  const bool aligned = ((uintptr_t)B & 15) == 0 && ((uintptr_t)C & 15) == 0 && N % V16 == 0;
  if (aligned) return launch_spmm_sub<P, V16, SUB, LONG>(A, N, B, C, W, st);
  if constexpr (std::is_same<P, MmDFS>::value) {
    // the split works on 16-byte pairs
    return launch_spmm_sub<MmNative64, 1, SUB, LONG>(A, N, B, C, W, st);
  } else {
    return launch_spmm_sub<P, 1, SUB, LONG>(A, N, B, C, W, st);
  }
}

// TMA-staged tiles for ring depth S: the widest lane vector whose column tile divides N, with
// B's row segments 16-byte aligned; otherwise the register-staged streaming tile.
template <class P, int S>
int spmm_dispatch_tma(const tacogb_csr* A, int32_t N, const void* B, void* C, int W,
                      cudaStream_t st) {
  constexpr int esz = sizeof(typename P::BV);
  const bool al16 = ((uintptr_t)B & 15) == 0 && ((int64_t)N * esz) % 16 == 0;
  if constexpr (esz == 8) {
    if (al16 && N % 64 == 0) return launch_spmm<P, 2, true, S>(A, N, B, C, W, st);
  } else if constexpr (esz == 4) {
    if (al16 && N % 128 == 0) return launch_spmm<P, 4, true, S>(A, N, B, C, W, st);
  } else {
    if (al16 && N % 256 == 0) return launch_spmm<P, 8, true, S>(A, N, B, C, W, st);
  }
  return -1;  // not applicable: the caller runs the streaming tile
}

// Widest lane vector (up to 16 bytes) whose column tile divides N.
template <class P, bool STREAM = false, int TMA = 0>
int spmm_dispatch_vec(const tacogb_csr* A, int32_t N, const void* B, void* C, int W,
                      cudaStream_t st) {
  if constexpr (std::is_same<P, MmDFS>::value) {
    // the B split works on 16-byte pairs of elements
    if (N % 2 != 0 || ((uintptr_t)B & 15) != 0)
      return spmm_dispatch_vec<MmDF64, STREAM>(A, N, B, C, W, st);
  }
  if constexpr (TMA > 0) {
    // the split B (MmDFS) lives in the library's scratch, 256-byte aligned, so the test on the
    // caller's B (16-byte aligned, N even) above covers it too
    const int rc = spmm_dispatch_tma<P, TMA>(A, N, B, C, W, st);
    if (rc >= 0) return rc;
  }
  constexpr int esz = sizeof(typename P::BV);
  if constexpr (esz == 8) {
    if (N % 64 == 0) return launch_spmm<P, 2, STREAM>(A, N, B, C, W, st);
    return launch_spmm<P, 1, STREAM>(A, N, B, C, W, st);
  } else if constexpr (esz == 4) {
    if (N % 128 == 0) return launch_spmm<P, 4, STREAM>(A, N, B, C, W, st);
    if (N % 64 == 0) return launch_spmm<P, 2, STREAM>(A, N, B, C, W, st);
    return launch_spmm<P, 1, STREAM>(A, N, B, C, W, st);
  } else {
    if (N % 256 == 0) return launch_spmm<P, 8, STREAM>(A, N, B, C, W, st);
    if (N % 128 == 0) return launch_spmm<P, 4, STREAM>(A, N, B, C, W, st);
    if (N % 64 == 0) return launch_spmm<P, 2, STREAM>(A, N, B, C, W, st);
    return launch_spmm<P, 1, STREAM>(A, N, B, C, W, st);
  }
}

}  // namespace

int spmm_variant_count() { return kNumSpmmVariants; }
const char* spmm_variant_name(int v) {
  return (v >= 0 && v < kNumSpmmVariants) ? kSpmmVariants[v].name : "";
}

int spmm_variant_index(const char* name) {
  for (int i = 0; i < kNumSpmmVariants; i++)
    if (strcmp(kSpmmVariants[i].name, name) == 0) return i;
  return -1;
}

bool spmm_presplit_applies(const void* B, int32_t N) {
  return N > 0 && N % 2 == 0 && ((uintptr_t)B & 15) == 0;
}

int spmm_split_once(const double* B, int32_t cols, int32_t N, void* bdf, int* flag,
                    cudaStream_t st) {
  TACOGB_CHECK_ARG(spmm_presplit_applies(B, N) && ((uintptr_t)bdf & 15) == 0,
                   "SpMM: B split needs even N and 16-byte aligned arrays");
  TACOGB_LAUNCH("spmm_flag_clear", st, spmm_flag_clear<<<1, 1, 0, st>>>(flag));
  const int64_t count = (int64_t)cols * N;
  if (count > 0)
    TACOGB_LAUNCH("spmm_split_b", st,
                  spmm_split_b<<<(unsigned)((count / 2 + 255) / 256), 256, 0, st>>>(
                      B, (DF*)bdf, count, flag));
  return 0;
}

int spmm_run_presplit(const tacogb_csr* A, int32_t N, const double* B, const void* bdf, int* flag,
                      double* C, cudaStream_t st, int scratch_slot) {
  TACOGB_CHECK_ARG(A != nullptr && A->vtype == TACOGB_F64, "SpMM: pre-split B needs FP64 A");
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->nnz >= 0 && N >= 0, "SpMM: negative size");
  TACOGB_CHECK_ARG((int64_t)A->rows * N <= INT32_MAX,
                   "SpMM: rows*N exceeds taco's int32 dense positions");
  TACOGB_CHECK_ARG(spmm_presplit_applies(B, N), "SpMM: B split needs even N, 16-byte aligned B");
  static const int W = kSpmmVariants[spmm_variant_index("merge_w512_dfs")].tile_items;
  if (N % 64 == 0)
    return launch_spmm<MmDFS, 2, false>(A, N, B, C, W, st, bdf, flag, scratch_slot);
  return launch_spmm<MmDFS, 1, false>(A, N, B, C, W, st, bdf, flag, scratch_slot);
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
  if (variant < 0) {
    // measured fastest on the 1,048,576-row power-law matrix: FP64 double-float over a
    // pre-split B on the warp tile; FP32 compensated on the streaming tile; BF16 B plain FFMA
    const char* pick = A->vtype == TACOGB_F64 ? "merge_w512_dfs"
                       : btype == TACOGB_BF16 ? "merge_w512_native"
                                              : "stream_w512_dfs";
    variant = 0;
    for (int i = 0; i < kNumSpmmVariants; i++)
      if (strcmp(kSpmmVariants[i].name, pick) == 0) variant = i;
  }
  TACOGB_CHECK_ARG(variant < kNumSpmmVariants, "SpMM: variant %d out of range", variant);
  const SpmmVariant& v = kSpmmVariants[variant];
  const int W = v.tile_items;
  if (v.lpr > 0) {
    auto sub = [&](auto tag) -> int {
      using P = decltype(tag);
      if (v.shared)
        return v.lpr == 8 ? spmm_dispatch_sub<P, 8, 0>(A, N, B, C, W, st)
                          : spmm_dispatch_sub<P, 4, 0>(A, N, B, C, W, st);
      return v.lpr == 8 ? spmm_dispatch_sub<P, 8, kSubLong>(A, N, B, C, W, st)
                        : spmm_dispatch_sub<P, 4, kSubLong>(A, N, B, C, W, st);
    };
    if (A->vtype == TACOGB_F64 && btype == TACOGB_F64)
      return v.df == 2 ? sub(MmDFS{}) : v.df == 1 ? sub(MmDF64{}) : sub(MmNative64{});
    if (A->vtype == TACOGB_F32 && btype == TACOGB_F32)
      return v.df ? sub(MmComp32{}) : sub(MmF32{});
    if (A->vtype == TACOGB_F32 && btype == TACOGB_BF16) return sub(MmBF16{});
  } else {
    auto run = [&](auto tag) -> int {
      using P = decltype(tag);
      if (v.tma == 12) return spmm_dispatch_vec<P, true, 12>(A, N, B, C, W, st);
      if (v.tma == 16) return spmm_dispatch_vec<P, true, 16>(A, N, B, C, W, st);
      return v.stream ? spmm_dispatch_vec<P, true>(A, N, B, C, W, st)
                      : spmm_dispatch_vec<P, false>(A, N, B, C, W, st);
    };
    if (A->vtype == TACOGB_F64 && btype == TACOGB_F64)
      return v.df == 2 ? run(MmDFS{}) : v.df == 1 ? run(MmDF64{}) : run(MmNative64{});
    if (A->vtype == TACOGB_F32 && btype == TACOGB_F32)
      return v.df ? run(MmComp32{}) : run(MmF32{});
    if (A->vtype == TACOGB_F32 && btype == TACOGB_BF16) return run(MmBF16{});
  }
  set_error(TACOGB_ERR_ARG, "SpMM: unsupported value types (A %d, B %d)", A->vtype, btype);
  return TACOGB_ERR_ARG;
}

}  // namespace tacogb
