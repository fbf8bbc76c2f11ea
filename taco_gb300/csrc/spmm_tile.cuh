// SpMM building blocks shared by the single-matrix kernel (spmm.cu) and the batched persistent
// kernel (batched.cu): 16-byte lane vectors, accumulation policies and the one-warp merge tile.
#pragma once

#include <climits>
#include <cuda_bf16.h>
#include <type_traits>

#include "common.cuh"
#include "df.cuh"

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

// B pre-split into double-float pairs (8 bytes per element): two pairs per 16-byte load.
template <int VEC>
__device__ __forceinline__ void load_vec(const DF* p, DF (&o)[VEC]) {
  if constexpr (VEC == 2) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = DF{v.x, v.y};
    o[1] = DF{v.z, v.w};
  } else {
    static_assert(VEC == 1, "double-float vectors are 1 or 2 wide");
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    o[0] = DF{v.x, v.y};
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

// Running double-float sum with deferred renormalisation: hi sum s and an unnormalised
// compensation c (the product errors, cross terms and TwoSum errors), renormalised on output
// and once per 32 nonzeros (so that c's own rounding stays at 2^-48 of the sum for long rows).
struct DFAcc {
  float s, c;
};

template <class P>
__device__ __forceinline__ void renorm(typename P::Acc&) {}

// FP32 values and B, compensated: per column the exact TwoProduct and one TwoSum, their errors
// summed into the unnormalised compensation (ten FP32 instructions; renormalised with the
// double-float accumulators, once per 32 nonzeros and on output).
struct MmComp32 : MmF32 {
  using Acc = DFAcc;
  __device__ static Acc zero() { return DFAcc{0.f, 0.f}; }
  __device__ static void madd(Acc& acc, Prep a, BE b, bool&) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    float s1, e;
    two_sum(acc.s, p, s1, e);
    acc.c = __fadd_rn(acc.c, __fadd_rn(pe, e));
    acc.s = s1;
  }
  __device__ static Out out(Acc a) { return __fadd_rn(a.s, a.c); }
  __device__ static double to_double(Acc a) { return (double)a.s + (double)a.c; }
};

template <>
__device__ __forceinline__ void renorm<MmComp32>(DFAcc& a) {
  float s, e;
  two_sum(a.s, a.c, s, e);
  a.s = s;
  a.c = e;
}

struct MmBF16 : MmF32 {
  using BV = __nv_bfloat16;
};


// FP64 values, B pre-split into double-float pairs: per column one exact TwoProduct of the hi
// parts, two cross-term FMAs and one TwoSum (about 12 FP32 instructions); values are split by
// split_df_fast and range-checked (a tile with an out-of-range value is redone natively).
struct MmDFS {
  using AV = double;
  using BV = DF;
  using BE = DF;
  using Prep = DF;
  using Acc = DFAcc;
  using Out = double;
  static constexpr bool kChecked = true;
  __device__ static Prep prep(AV a, bool& ok) {
    DF p;
    split_df_fast(a, p.h, p.l);
    ok &= df_in_range(a);
    return p;
  }
  __device__ static Prep shfl(Prep a, int src) {
    return DF{__shfl_sync(0xffffffffu, a.h, src), __shfl_sync(0xffffffffu, a.l, src)};
  }
  __device__ static Acc zero() { return DFAcc{0.f, 0.f}; }
  __device__ static void madd(Acc& acc, Prep a, BE b, bool&) {
    const float ph = __fmul_rn(a.h, b.h);
    const float pe = __fmaf_rn(a.h, b.h, -ph);
    float c = __fmaf_rn(a.h, b.l, acc.c);
    c = __fmaf_rn(a.l, b.h, c);
    float s1, e;
    two_sum(acc.s, ph, s1, e);
    acc.c = __fadd_rn(c, __fadd_rn(pe, e));
    acc.s = s1;
  }
  __device__ static DF norm(Acc a) {
    DF r;
    two_sum(a.s, a.c, r.h, r.l);
    return r;
  }
  __device__ static Out out(Acc a) { return df_to_double(norm(a)); }
  __device__ static double to_double(Acc a) { return df_to_double(norm(a)); }
};

template <>
__device__ __forceinline__ void renorm<MmDFS>(DFAcc& a) {
  float s, e;
  two_sum(a.s, a.c, s, e);
  a.s = s;
  a.c = e;
}

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
#pragma unroll
      for (int v = 0; v < VEC; v++) renorm<P>(acc[v]);
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

// ------------------------------------------------------------------ streaming warp tile ----
//
// The same merge tile walked as one stream of nonzeros instead of row by row: the warp loads
// crd/vals 32 nonzeros at a time, one chunk ahead of the B-row loads that depend on them,
// whatever the row boundaries; row ends come from a batch of 32 pos entries loaded at once;
// a row is written when the stream passes its end.  A row walk waits for pos, then crd/vals,
// then B for every row; here only the B loads are waited for.  Same contract as spmm_tile.
template <class P, int VEC>
__device__ __forceinline__ bool spmm_tile_stream(const int32_t* __restrict__ pos,
                                                 const int32_t* __restrict__ crd,
                                                 const typename P::AV* __restrict__ vals,
                                                 const typename P::BV* __restrict__ B,
                                                 typename P::Out* __restrict__ C, int32_t n,
                                                 int32_t N, int2 c0, int2 c1, int tile, int col0,
                                                 bool active, int32_t* __restrict__ carry_row,
                                                 double* __restrict__ carry_val) {
  using Acc = typename P::Acc;
  using Prep = typename P::Prep;
  using BE = typename P::BE;
  using AV = typename P::AV;
  constexpr int U = kMmUnroll;
  const int lane = threadIdx.x & 31;
  const int r0 = c0.x, k0 = c0.y, r1 = c1.x, k1 = c1.y;
  bool ok = true;
  // ends (pos[r + 1]) of rows rb .. rb + 31, one per lane; rows r1 and later are open
  int rb = r0;
  int re = (rb + lane < r1) ? __ldg(pos + rb + lane + 1) : INT_MAX;
  int row = r0;
  int next_end = __shfl_sync(0xffffffffu, re, 0);
  bool open_nonempty = false;  // the current row has nonzeros in this tile
  Acc acc[VEC];
#pragma unroll
  for (int v = 0; v < VEC; v++) acc[v] = P::zero();
  auto emit = [&]() {
    if (active) {
      typename P::Out o[VEC];
#pragma unroll
      for (int v = 0; v < VEC; v++) o[v] = P::out(acc[v]);
      store_vec<VEC>(C + (int64_t)row * N + col0, o);
    }
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = P::zero();
    open_nonempty = false;
    row++;
    if (row - rb == 32) {
      rb = row;
      re = (rb + lane < r1) ? __ldg(pos + rb + lane + 1) : INT_MAX;
    }
    next_end = __shfl_sync(0xffffffffu, re, row - rb);
  };
  int mc_n = 0;
  AV mv_n = AV();
  if (k0 + lane < k1) {
    mc_n = __ldg(crd + k0 + lane);
    mv_n = vals[k0 + lane];
  }
  for (int base = k0; base < k1; base += 32) {
    const int cnt = min(32, k1 - base);
    const int mc = mc_n;
    const Prep ma = lane < cnt ? P::prep(mv_n, ok) : Prep();
    if (base + 32 + lane < k1) {
      mc_n = __ldg(crd + base + 32 + lane);
      mv_n = vals[base + 32 + lane];
    }
    int j = 0;
    for (; j + U <= cnt; j += U) {
      BE b[U][VEC];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int c = __shfl_sync(0xffffffffu, mc, j + u);
        if (active) load_vec<VEC>(B + (int64_t)c * N + col0, b[u]);
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        while (next_end <= base + j + u) emit();
        const Prep a = P::shfl(ma, j + u);
        if (active) {
#pragma unroll
          for (int v = 0; v < VEC; v++) P::madd(acc[v], a, b[u][v], ok);
        }
        open_nonempty = true;
      }
    }
    for (; j < cnt; j++) {
      const int c = __shfl_sync(0xffffffffu, mc, j);
      BE b[VEC];
      if (active) load_vec<VEC>(B + (int64_t)c * N + col0, b);
      while (next_end <= base + j) emit();
      const Prep a = P::shfl(ma, j);
      if (active) {
#pragma unroll
        for (int v = 0; v < VEC; v++) P::madd(acc[v], a, b[v], ok);
      }
      open_nonempty = true;
    }
#pragma unroll
    for (int v = 0; v < VEC; v++) renorm<P>(acc[v]);
  }
  while (row < r1) emit();  // rows that end at k1, and empty rows after the last nonzero
  const bool carried = row < n && open_nonempty;
  if (carried && active) {
#pragma unroll
    for (int v = 0; v < VEC; v++) carry_val[(int64_t)tile * N + col0 + v] = P::to_double(acc[v]);
  }
  if (lane == 0 && blockIdx.y == 0) carry_row[tile] = carried ? r1 : n;
  return ok;
}

// ------------------------------------------------------------------ TMA-staged warp tile ---
//
// The streaming warp tile with its B rows staged by bulk copies (cp.async.bulk) instead of
// register loads.  Each warp keeps a ring of S slots in shared memory, one slot per nonzero
// holding the warp's TW = 32 * VEC columns of that nonzero's B row, each completing on its own
// mbarrier.  Lane 0 keeps the copies of the next S nonzeros in flight (re-arming U slots at a
// time after the lanes have read them), so S B rows per warp are in flight without holding any
// registers, where the register-staged tile holds kMmUnroll.  Waits are bounded
// (mbar_wait_or_flag); a wait that gives up records the timeout in the status word and the walk
// goes on, so every copy issued is waited for again before the warp exits.  Needs every lane
// active (N a multiple of TW) and B's row segments 16-byte aligned.

template <class P, int VEC, int S>
struct alignas(16) MmRing {
  alignas(16) typename P::BV row[S][32 * VEC];
  uint64_t bar[S];
};

template <int VEC>
__device__ __forceinline__ void smem_vec(const double* p, double (&o)[VEC]) {
  if constexpr (VEC == 2) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    o[0] = v.x;
    o[1] = v.y;
  } else {
    o[0] = p[0];
  }
}
template <int VEC>
__device__ __forceinline__ void smem_vec(const float* p, float (&o)[VEC]) {
  if constexpr (VEC == 4) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  } else if constexpr (VEC == 2) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    o[0] = v.x; o[1] = v.y;
  } else {
    o[0] = p[0];
  }
}
template <int VEC>
__device__ __forceinline__ void smem_vec(const __nv_bfloat16* p, float (&o)[VEC]) {
  if constexpr (VEC == 8) {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    o[0] = bf16_lo(v.x); o[1] = bf16_hi(v.x); o[2] = bf16_lo(v.y); o[3] = bf16_hi(v.y);
    o[4] = bf16_lo(v.z); o[5] = bf16_hi(v.z); o[6] = bf16_lo(v.w); o[7] = bf16_hi(v.w);
  } else if constexpr (VEC == 4) {
    const uint2 v = *reinterpret_cast<const uint2*>(p);
    o[0] = bf16_lo(v.x); o[1] = bf16_hi(v.x); o[2] = bf16_lo(v.y); o[3] = bf16_hi(v.y);
  } else if constexpr (VEC == 2) {
    const unsigned int v = *reinterpret_cast<const unsigned int*>(p);
    o[0] = bf16_lo(v); o[1] = bf16_hi(v);
  } else {
    o[0] = bf16_lo((unsigned int)*reinterpret_cast<const unsigned short*>(p));
  }
}
template <int VEC>
__device__ __forceinline__ void smem_vec(const DF* p, DF (&o)[VEC]) {
  if constexpr (VEC == 2) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = DF{v.x, v.y};
    o[1] = DF{v.z, v.w};
  } else {
    const float2 v = *reinterpret_cast<const float2*>(p);
    o[0] = DF{v.x, v.y};
  }
}

template <class P, int VEC, int S>
__device__ __forceinline__ bool spmm_tile_tma(MmRing<P, VEC, S>& ring,
                                              const int32_t* __restrict__ pos,
                                              const int32_t* __restrict__ crd,
                                              const typename P::AV* __restrict__ vals,
                                              const typename P::BV* __restrict__ B,
                                              typename P::Out* __restrict__ C, int32_t n,
                                              int32_t N, int2 c0, int2 c1, int tile, int colt,
                                              int* status, int32_t* __restrict__ carry_row,
                                              double* __restrict__ carry_val) {
  using Acc = typename P::Acc;
  using Prep = typename P::Prep;
  using BE = typename P::BE;
  using AV = typename P::AV;
  using BV = typename P::BV;
  constexpr int U = kMmUnroll;
  constexpr uint32_t kRowBytes = 32 * VEC * sizeof(BV);
  static_assert(S >= U && S <= 32, "ring depth");
  static_assert(kRowBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
  const int lane = threadIdx.x & 31;
  const int col0 = colt + lane * VEC;
  const int r0 = c0.x, k0 = c0.y, r1 = c1.x, k1 = c1.y;
  bool ok = true;
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < S; q++) mbar_init(&ring.bar[q], 1);
  }
  __syncwarp();
  auto issue = [&](int g, int c) {  // lane 0: nonzero g's B row segment into its slot
    const int q = (g - k0) % S;
    mbar_arrive_expect_tx(&ring.bar[q], kRowBytes);
    tma_load_bulk(ring.row[q], B + (int64_t)c * N + colt, kRowBytes, &ring.bar[q]);
  };
  int rb = r0;
  int re = (rb + lane < r1) ? __ldg(pos + rb + lane + 1) : INT_MAX;
  int row = r0;
  int next_end = __shfl_sync(0xffffffffu, re, 0);
  bool open_nonempty = false;
  Acc acc[VEC];
#pragma unroll
  for (int v = 0; v < VEC; v++) acc[v] = P::zero();
  auto emit = [&]() {
    typename P::Out o[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) o[v] = P::out(acc[v]);
    store_vec<VEC>(C + (int64_t)row * N + col0, o);
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = P::zero();
    open_nonempty = false;
    row++;
    if (row - rb == 32) {
      rb = row;
      re = (rb + lane < r1) ? __ldg(pos + rb + lane + 1) : INT_MAX;
    }
    next_end = __shfl_sync(0xffffffffu, re, row - rb);
  };
  // crd/vals of the chunk being walked (mc, mv) and of the next one (mc_n, mv_n)
  int mc_n = 0;
  AV mv_n = AV();
  if (k0 + lane < k1) {
    mc_n = __ldg(crd + k0 + lane);
    mv_n = vals[k0 + lane];
  }
  // prologue: the first S nonzeros' rows (their columns are all in the first chunk)
  {
    const int m = min(S, k1 - k0);
    for (int u = 0; u < m; u++) {
      const int c = __shfl_sync(0xffffffffu, mc_n, u);
      if (lane == 0) issue(k0 + u, c);
    }
  }
  for (int base = k0; base < k1; base += 32) {
    const int cnt = min(32, k1 - base);
    const int mc = mc_n;
    const Prep ma = lane < cnt ? P::prep(mv_n, ok) : Prep();
    if (base + 32 + lane < k1) {
      mc_n = __ldg(crd + base + 32 + lane);
      mv_n = vals[base + 32 + lane];
    }
    for (int j = 0; j < cnt; j += U) {
      const int m = min(U, cnt - j);
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (u < m) {
          const int g = base + j + u;
          const int q = g - k0;
          if (!mbar_wait_or_flag(&ring.bar[q % S], (uint32_t)((q / S) & 1), status)) ok = false;
          BE b[VEC];
          smem_vec<VEC>(&ring.row[q % S][lane * VEC], b);
          while (next_end <= g) emit();
          const Prep a = P::shfl(ma, j + u);
#pragma unroll
          for (int v = 0; v < VEC; v++) P::madd(acc[v], a, b[v], ok);
          open_nonempty = true;
        }
      }
      // re-arm the slots just read with the rows S nonzeros ahead (columns from this chunk or
      // the next; S <= 32 keeps them within the two chunks held)
      __syncwarp();
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int jj = j + u + S;
        const int ca = __shfl_sync(0xffffffffu, mc, jj & 31);
        const int cb = __shfl_sync(0xffffffffu, mc_n, jj & 31);
        if (lane == 0 && u < m && base + jj < k1) {
          if (u == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(base + jj, jj < 32 ? ca : cb);
        }
      }
    }
#pragma unroll
    for (int v = 0; v < VEC; v++) renorm<P>(acc[v]);
  }
  while (row < r1) emit();
  const bool carried = row < n && open_nonempty;
  if (carried) {
#pragma unroll
    for (int v = 0; v < VEC; v++) carry_val[(int64_t)tile * N + col0 + v] = P::to_double(acc[v]);
  }
  if (lane == 0 && blockIdx.y == 0) carry_row[tile] = carried ? r1 : n;
  return ok;
}

// ------------------------------------------------------------------ sub-warp tile --------
//
// For narrow dense operands (N*sizeof(B) of 128 bytes or less, N=32 in the batched workload) one
// lane vector per lane covers a B row with LPR = 32/SUB lanes, so the warp splits into SUB
// sub-warps.  Rows of the tile go to sub-warps: SUB consecutive short rows at a time, one per
// sub-warp, while a row segment of kSubLong nonzeros or more is shared by the whole warp (each
// sub-warp takes every SUB-th group of LPR nonzeros, then the sub-warps' sums are added in a
// fixed butterfly).  Each sub-warp issues LPR B-row loads before it multiplies, so up to 32 B
// rows are in flight per warp whatever the row lengths.  Loop trip counts are warp-uniform (the
// longest row of the group), so every shuffle runs on the full warp.

__device__ __forceinline__ double acc_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float acc_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ DF acc_add(DF a, DF b) { return df_add(a, b); }
__device__ __forceinline__ double acc_xor(double a, int o) {
  return __shfl_xor_sync(0xffffffffu, a, o);
}
__device__ __forceinline__ float acc_xor(float a, int o) {
  return __shfl_xor_sync(0xffffffffu, a, o);
}
__device__ __forceinline__ DF acc_xor(DF a, int o) {
  return DF{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}
__device__ __forceinline__ DFAcc acc_add(DFAcc a, DFAcc b) {
  float s, e;
  two_sum(a.s, b.s, s, e);
  return DFAcc{s, __fadd_rn(__fadd_rn(a.c, b.c), e)};
}
__device__ __forceinline__ DFAcc acc_xor(DFAcc a, int o) {
  return DFAcc{__shfl_xor_sync(0xffffffffu, a.s, o), __shfl_xor_sync(0xffffffffu, a.c, o)};
}

constexpr int kSubLong = 64;
#ifndef TACOGB_SUB_BYTES
#define TACOGB_SUB_BYTES 64
#endif
constexpr int kSubBytes = TACOGB_SUB_BYTES;  // register bytes per lane for B rows in flight

// LPR nonzeros of one sub-warp: crd/val sit in the lanes [lb, lb+LPR) of mc/ma; the first cnt
// are valid.  Issues all B-row loads before the multiplies.
template <class P, int VEC, int LPR>
__device__ __forceinline__ void sub_chunk(typename P::Acc (&acc)[VEC], int mc,
                                          typename P::Prep ma, int lb, int cnt,
                                          const typename P::BV* __restrict__ B, int32_t N,
                                          int col0, bool active, bool& ok) {
  using BE = typename P::BE;
  // B-row loads in flight per lane: kSubBytes of registers
  constexpr int UB = kSubBytes / (VEC * (int)sizeof(BE));
  constexpr int U = LPR < UB ? LPR : (UB > 0 ? UB : 1);
#pragma unroll 1
  for (int u0 = 0; u0 < LPR; u0 += U) {
    BE b[U][VEC];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int c = __shfl_sync(0xffffffffu, mc, lb + u0 + u);
      if (active && u0 + u < cnt) load_vec<VEC>(B + (int64_t)c * N + col0, b[u]);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const typename P::Prep a = P::shfl(ma, lb + u0 + u);
      if (active && u0 + u < cnt) {
#pragma unroll
        for (int v = 0; v < VEC; v++) P::madd(acc[v], a, b[u][v], ok);
      }
    }
  }
}

template <class P, int VEC>
__device__ __forceinline__ void sub_emit(const typename P::Acc (&acc)[VEC], int r, int r1,
                                         bool nonempty, typename P::Out* __restrict__ C,
                                         int32_t N, int col0, int tile,
                                         double* __restrict__ carry_val, bool& carried) {
  if (r < r1) {
    typename P::Out o[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) o[v] = P::out(acc[v]);
    store_vec<VEC>(C + (int64_t)r * N + col0, o);
  } else if (nonempty) {
    carried = true;
#pragma unroll
    for (int v = 0; v < VEC; v++) carry_val[(int64_t)tile * N + col0 + v] = P::to_double(acc[v]);
  }
}

// Columns [ct, ct + LPR*VEC) of merge tile `tile`.  Same contract as spmm_tile.  Rows of LONG
// or more nonzeros are shared by the whole warp (sub-warp s takes every SUB-th nonzero, and a
// butterfly joins the sub-warps at the row end); shorter rows get one sub-warp each.  LONG = 0
// shares every row, which keeps all sub-warps busy whatever the row lengths.
template <class P, int VEC, int SUB, int LONG = kSubLong>
__device__ __forceinline__ bool spmm_tile_sub(const int32_t* __restrict__ pos,
                                              const int32_t* __restrict__ crd,
                                              const typename P::AV* __restrict__ vals,
                                              const typename P::BV* __restrict__ B,
                                              typename P::Out* __restrict__ C, int32_t n,
                                              int32_t N, int2 c0, int2 c1, int tile, int ct,
                                              int32_t* __restrict__ carry_row,
                                              double* __restrict__ carry_val) {
  using Acc = typename P::Acc;
  using Prep = typename P::Prep;
  constexpr int LPR = 32 / SUB;
  const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR, lb = sub * LPR;
  const int col0 = ct + sl * VEC;
  const bool active = col0 < N;
  const int r0 = c0.x, k0 = c0.y, r1 = c1.x, k1 = c1.y;
  const int rend = min(r1, n - 1);
  bool ok = true, carried = false;
  int r = r0;
  while (r <= rend) {
    const int myr = r + sub;
    int ps = 0, pe = 0;
    if (myr <= rend) {
      ps = (myr == r0) ? k0 : __ldg(pos + myr);
      pe = (myr < r1) ? __ldg(pos + myr + 1) : k1;
    }
    const int len = pe - ps;
    const unsigned lmask = __ballot_sync(0xffffffffu, sl == 0 && myr <= rend && len >= LONG);
    const int first_long = lmask ? (__ffs(lmask) - 1) / LPR : SUB;
    const int k = min(first_long, rend - r + 1);
    Acc acc[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = P::zero();
    if (k == 0) {
      // row r shared by the whole warp: sub-warp s takes lanes [s*LPR, s*LPR+LPR) of each 32
      const int ps0 = __shfl_sync(0xffffffffu, ps, 0), pe0 = __shfl_sync(0xffffffffu, pe, 0);
      // crd/vals run one chunk ahead of the B-row loads that depend on them
      int mc_n = 0;
      typename P::AV mv_n = typename P::AV();
      if (ps0 + lane < pe0) {
        mc_n = ld_stream_i32(crd + ps0 + lane);
        mv_n = vals[ps0 + lane];
      }
      for (int base = ps0; base < pe0; base += 32) {
        const int cnt = min(32, pe0 - base);
        const int mc = mc_n;
        const Prep ma = lane < cnt ? P::prep(mv_n, ok) : Prep();
        if (base + 32 + lane < pe0) {
          mc_n = ld_stream_i32(crd + base + 32 + lane);
          mv_n = vals[base + 32 + lane];
        }
        sub_chunk<P, VEC, LPR>(acc, mc, ma, lb, cnt - lb, B, N, col0, active, ok);
#pragma unroll
        for (int v = 0; v < VEC; v++) renorm<P>(acc[v]);
      }
#pragma unroll
      for (int o = LPR; o < 32; o <<= 1) {
#pragma unroll
        for (int v = 0; v < VEC; v++) acc[v] = acc_add(acc[v], acc_xor(acc[v], o));
      }
      if (sub == 0 && active)
        sub_emit<P, VEC>(acc, r, r1, pe0 > ps0, C, N, col0, tile, carry_val, carried);
      r += 1;
    } else {
      // rows r .. r+k-1, one per sub-warp
      const bool mine = sub < k;
      int trip = mine ? len : 0;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) trip = max(trip, __shfl_xor_sync(0xffffffffu, trip, o));
      int mc_n = 0;
      typename P::AV mv_n = typename P::AV();
      if (mine && sl < len) {
        mc_n = ld_stream_i32(crd + ps + sl);
        mv_n = vals[ps + sl];
      }
      for (int base = 0; base < trip; base += LPR) {
        const int cnt = mine ? min(LPR, len - base) : 0;
        const int mc = mc_n;
        const Prep ma = sl < cnt ? P::prep(mv_n, ok) : Prep();
        if (mine && base + LPR + sl < len) {
          mc_n = ld_stream_i32(crd + ps + base + LPR + sl);
          mv_n = vals[ps + base + LPR + sl];
        }
        sub_chunk<P, VEC, LPR>(acc, mc, ma, lb, cnt, B, N, col0, active, ok);
#pragma unroll
        for (int v = 0; v < VEC; v++) renorm<P>(acc[v]);
      }
      if (mine && active)
        sub_emit<P, VEC>(acc, myr, r1, len > 0, C, N, col0, tile, carry_val, carried);
      r += k;
    }
  }
  carried = __any_sync(0xffffffffu, carried);
  if (lane == 0 && blockIdx.y == 0) carry_row[tile] = carried ? r1 : n;
  return ok;
}

}  // namespace tacogb
