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

namespace tacogb {

// ------------------------------------------------------------------ vector I/O -----------

template <int VEC>
__device__ __forceinline__ void load_vec(const double* p, double (&o)[VEC]) {
  if constexpr (VEC == 2) {
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    o[0] = v.x;
    o[1] = v.y;
  } else {
    static_assert(VEC == 1, "double vectors are 1 or 2 wide");
    o[0] = __ldg(p);
  }
}

template <int VEC>
__device__ __forceinline__ void load_vec(const float* p, float (&o)[VEC]) {
  if constexpr (VEC == 4) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  } else if constexpr (VEC == 2) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    o[0] = v.x; o[1] = v.y;
  } else {
    static_assert(VEC == 1, "float vectors are 1, 2 or 4 wide");
    o[0] = __ldg(p);
  }
}

__device__ __forceinline__ float bf16_lo(unsigned int w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(unsigned int w) { return __uint_as_float(w & 0xFFFF0000u); }

template <int VEC>
__device__ __forceinline__ void load_vec(const __nv_bfloat16* p, float (&o)[VEC]) {
  if constexpr (VEC == 8) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
    o[0] = bf16_lo(v.x); o[1] = bf16_hi(v.x); o[2] = bf16_lo(v.y); o[3] = bf16_hi(v.y);
    o[4] = bf16_lo(v.z); o[5] = bf16_hi(v.z); o[6] = bf16_lo(v.w); o[7] = bf16_hi(v.w);
  } else if constexpr (VEC == 4) {
    const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
    o[0] = bf16_lo(v.x); o[1] = bf16_hi(v.x); o[2] = bf16_lo(v.y); o[3] = bf16_hi(v.y);
  } else if constexpr (VEC == 2) {
    const unsigned int v = __ldg(reinterpret_cast<const unsigned int*>(p));
    o[0] = bf16_lo(v); o[1] = bf16_hi(v);
  } else {
    static_assert(VEC == 1, "bf16 vectors are 1, 2, 4 or 8 wide");
    o[0] = bf16_lo((unsigned int)__ldg(reinterpret_cast<const unsigned short*>(p)));
  }
}

template <int VEC>
__device__ __forceinline__ void store_vec(double* p, const double (&o)[VEC]) {
  if constexpr (VEC == 2) *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
  else p[0] = o[0];
}

template <int VEC>
__device__ __forceinline__ void store_vec(float* p, const float (&o)[VEC]) {
  if constexpr (VEC == 8) {
    reinterpret_cast<float4*>(p)[0] = make_float4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<float4*>(p)[1] = make_float4(o[4], o[5], o[6], o[7]);
  } else if constexpr (VEC == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
  } else if constexpr (VEC == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(o[0], o[1]);
  } else {
    p[0] = o[0];
  }
}

// ------------------------------------------------------------------ policies -------------

struct MmNative64 {
  using AV = double;  // A value
  using BV = double;  // B element in memory
  using BE = double;  // B element in registers
  using Prep = double;
  using Acc = double;
  using Out = double;
  static constexpr bool kChecked = false;
  __device__ static Prep prep(AV a, bool&) { return a; }
  __device__ static Prep shfl(Prep a, int src) { return __shfl_sync(0xffffffffu, a, src); }
  __device__ static Acc zero() { return 0.0; }
  __device__ static void madd(Acc& acc, Prep a, BE b, bool&) { acc = __fma_rn(a, b, acc); }
  __device__ static Out out(Acc a) { return a; }
  __device__ static double to_double(Acc a) { return a; }
};

struct MmDF64 {
  using AV = double;
  using BV = double;
  using BE = double;
  using Prep = DF;
  using Acc = DF;
  using Out = double;
  static constexpr bool kChecked = true;
  __device__ static Prep prep(AV a, bool& ok) {
    DF p;
    ok &= split_df(a, p.h, p.l);
    return p;
  }
  __device__ static Prep shfl(Prep a, int src) {
    return DF{__shfl_sync(0xffffffffu, a.h, src), __shfl_sync(0xffffffffu, a.l, src)};
  }
  __device__ static Acc zero() { return DF{0.f, 0.f}; }
  __device__ static void madd(Acc& acc, Prep a, BE b, bool& ok) {
    float bh, bl;
    ok &= split_df(b, bh, bl);
    acc = df_add(acc, df_mul(a.h, a.l, bh, bl));
  }
  __device__ static Out out(Acc a) { return df_to_double(a); }
  __device__ static double to_double(Acc a) { return df_to_double(a); }
};

struct MmF32 {
  using AV = float;
  using BV = float;
  using BE = float;
  using Prep = float;
  using Acc = float;
  using Out = float;
  static constexpr bool kChecked = false;
  __device__ static Prep prep(AV a, bool&) { return a; }
  __device__ static Prep shfl(Prep a, int src) { return __shfl_sync(0xffffffffu, a, src); }
  __device__ static Acc zero() { return 0.f; }
  __device__ static void madd(Acc& acc, Prep a, BE b, bool&) { acc = __fmaf_rn(a, b, acc); }
  __device__ static Out out(Acc a) { return a; }
  __device__ static double to_double(Acc a) { return (double)a; }
};

struct MmComp32 : MmF32 {
  using Acc = DF;
  __device__ static Acc zero() { return DF{0.f, 0.f}; }
  __device__ static void madd(Acc& acc, Prep a, BE b, bool&) {
    DF p;
    p.h = __fmul_rn(a, b);
    p.l = __fmaf_rn(a, b, -p.h);
    acc = df_add(acc, p);
  }
  __device__ static Out out(Acc a) { return __fadd_rn(a.h, a.l); }
  __device__ static double to_double(Acc a) { return (double)a.h + (double)a.l; }
};

struct MmBF16 : MmF32 {
  using BV = __nv_bfloat16;
};

// ------------------------------------------------------------------ kernel ---------------

constexpr int kMmBlock = 256;
constexpr int kMmWarps = kMmBlock / 32;
constexpr int kMmUnroll = 4;

// One warp: rows of merge tile `tile`, columns [col0, col0+VEC) per lane.  Returns false when a
// checked policy met an unrepresentable value (the caller then redoes the tile natively).
template <class P, int VEC>
__device__ __forceinline__ bool spmm_tile(const int32_t* __restrict__ pos,
                                          const int32_t* __restrict__ crd,
                                          const typename P::AV* __restrict__ vals,
                                          const typename P::BV* __restrict__ B,
                                          typename P::Out* __restrict__ C, int32_t n, int32_t N,
                                          int2 c0, int2 c1, int tile, int col0, bool active,
                                          int32_t* __restrict__ carry_row,
                                          double* __restrict__ carry_val) {
  using Acc = typename P::Acc;
  using Prep = typename P::Prep;
  using BE = typename P::BE;
  const int lane = threadIdx.x & 31;
  const int r0 = c0.x, k0 = c0.y, r1 = c1.x, k1 = c1.y;
  bool ok = true;
  bool carried = false;
  for (int r = r0; r <= r1 && r < n; r++) {
    const int ps = (r == r0) ? k0 : __ldg(pos + r);
    const int pe = (r < r1) ? __ldg(pos + r + 1) : k1;
    Acc acc[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = P::zero();
    for (int base = ps; base < pe; base += 32) {
      const int cnt = min(32, pe - base);
      int mc = 0;
      Prep ma = Prep();
      if (lane < cnt) {
        mc = ld_stream_i32(crd + base + lane);
        ma = P::prep(vals[base + lane], ok);
      }
      int j = 0;
      for (; j + kMmUnroll <= cnt; j += kMmUnroll) {
        BE b[kMmUnroll][VEC];
#pragma unroll
        for (int u = 0; u < kMmUnroll; u++) {
          const int c = __shfl_sync(0xffffffffu, mc, j + u);
          if (active) load_vec<VEC>(B + (int64_t)c * N + col0, b[u]);
        }
#pragma unroll
        for (int u = 0; u < kMmUnroll; u++) {
          const Prep a = P::shfl(ma, j + u);
          if (active) {
#pragma unroll
            for (int v = 0; v < VEC; v++) P::madd(acc[v], a, b[u][v], ok);
          }
        }
      }
      for (; j < cnt; j++) {
        const int c = __shfl_sync(0xffffffffu, mc, j);
        const Prep a = P::shfl(ma, j);
        if (active) {
          BE b[VEC];
          load_vec<VEC>(B + (int64_t)c * N + col0, b);
#pragma unroll
          for (int v = 0; v < VEC; v++) P::madd(acc[v], a, b[v], ok);
        }
      }
    }
    if (r < r1) {
      if (active) {
        typename P::Out o[VEC];
#pragma unroll
        for (int v = 0; v < VEC; v++) o[v] = P::out(acc[v]);
        store_vec<VEC>(C + (int64_t)r * N + col0, o);
      }
    } else if (pe > ps) {
      carried = true;
      if (active) {
#pragma unroll
        for (int v = 0; v < VEC; v++) carry_val[(int64_t)tile * N + col0 + v] = P::to_double(acc[v]);
      }
    }
  }
  if (lane == 0 && blockIdx.y == 0) carry_row[tile] = carried ? r1 : n;
  return ok;
}

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
