// CSR SpMV for sm_103a: y(i) = A(i,j) * x(j).
//
// Replaces the compute function taco generates for this statement: a row loop over
// A2_pos/A2_crd with a promoted scalar accumulator (src/lower/lowerer_impl_imperative.cpp:1304,
// src/index_notation/transformations.cpp:1982), and the GPU schedules of
// test/tests-scheduling-eval.cpp:193-247 (thread-per-row, warp-per-row, nnz-split with
// atomics after taco_binarySearchBeforeBlock, src/codegen/codegen_cuda.cpp:110-125).
//
// GB300 facts that shape the kernels (measured on the part): FP64 FMA issues at ~1.6 lanes per
// clock per SM and a DFMA warp instruction costs the same with 1 or 32 lanes active, while FP32
// FMA issues at ~118 lanes per clock per SM.  HBM delivers about two nonzeros (12 bytes each)
// per SM clock, so an FP64 SpMV that spends more than one full-warp FP64 instruction per 32
// nonzeros is FP64-bound, not HBM-bound.
//
// Kernel families:
//
//  wmerge  Merge-path over the sequence (row ends, nonzeros).  A scatter kernel writes the
//          merge coordinate of every CTA tile (one thread per row, no search chains).  A CTA
//          stages its tile's crd, vals and row ends in shared memory with coalesced loads; each
//          lane then walks IPT consecutive merge items, gathers x and accumulates; rows split
//          across lanes are joined by a segmented shuffle scan (all lanes active), rows split
//          across warps by one thread over eight warp carries, rows split across tiles by a
//          fix-up kernel over tile carry-outs.  Row results are staged in shared memory and
//          written coalesced.  No atomics: results are deterministic.
//          Accumulation policies:
//            native  FP64 DFMA (FP64 values), or TwoProduct/TwoSum-compensated FP32 (FP32
//                    values);
//            df      FP64 values evaluated in double-float on the FP32 pipe: each double is
//                    split with integer operations into hi+lo floats (46 significant bits),
//                    products by TwoProduct, sums by TwoSum; a tile whose values fall outside
//                    [2^-40, 2^40) (or are non-finite) is recomputed with native DFMA.  Error
//                    about 1e-14 relative, far inside the 1e-12 parity bar, at FP32-pipe cost.
//  vector  G lanes per row (G = 1 is thread-per-row, G = 32 is warp-per-row); lanes stride the
//          row with coalesced loads and combine with a shuffle butterfly.  Cheapest for short
//          regular rows in FP32; its log2(G) FP64 adds per row cost full warp instructions.

#include <algorithm>
#include <climits>
#include <cstdio>
#include <mutex>
#include <string>
#include <type_traits>
#include <unordered_map>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"
#include "wmerge.cuh"
#include "wtile.cuh"
#include "wspec.cuh"

namespace tacogb {

// x split once per product for the double-float policy; flag set when some entry is outside
// the double-float range (the product then runs every tile natively).
__global__ void spmv_split_x(const double* __restrict__ x, DF* __restrict__ xdf, int32_t n,
                             int* __restrict__ flag) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DF d;
  if (!split_df(__ldg(x + i), d.h, d.l)) *flag = 1;
  xdf[i] = d;
}

// ------------------------------------------------------------------ partition -------------

// Merge coordinate of every tile boundary D = b*T: the (rows ended, nonzeros consumed) point of
// the merge path over (row ends, nonzeros).  Row i owns the diagonals [pos[i]+i, pos[i+1]+i]; a
// boundary D inside them sits at (i, D-i).  One thread per row, so the cost is one coalesced
// read of pos.  part[tiles] = (n, nnz).  Diagonals stay below 2^32 (n and nnz are int32), so
// the division is 32-bit.
// With snap_len > 0 a boundary inside a row shorter than snap_len moves to that row's end
// (i+1, pos[i+1]), so that only rows of snap_len or more nonzeros are split between tiles;
// snap_len < T keeps every short row within one boundary, so coordinates stay monotone.
// Boundary 0 never moves: the first tile starts at (0, 0).
// Unsigned 32-bit division by an invariant divisor T as a multiply and shifts (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994): with
// l = ceil(log2 T) and m = floor(2^32 (2^l - T) / T) + 1, the quotient of any 32-bit v is
// (hi32(m v) + ((v - hi32(m v)) >> min(l, 1))) >> max(l - 1, 0).  Replaces the runtime divide,
// which dominated the partition pass.
struct DivU32 {
  uint32_t T, m, s1, s2;
};

inline DivU32 make_divu32(uint32_t T) {
  uint32_t l = 0;
  while (l < 32 && (1ull << l) < T) l++;
  DivU32 d;
  d.T = T;
  d.m = (uint32_t)(((1ull << 32) * ((1ull << l) - T)) / T + 1);
  d.s1 = l < 1 ? l : 1;
  d.s2 = l > 1 ? l - 1 : 0;
  return d;
}

__device__ __forceinline__ uint32_t divu32(uint32_t v, const DivU32& d) {
  const uint32_t t = __umulhi(d.m, v);
  return (t + ((v - t) >> d.s1)) >> d.s2;
}

__device__ __forceinline__ void partition_row_body(int32_t p0, int32_t p1, const DivU32& dv,
                                                   int32_t tiles, int32_t snap_len,
                                                   int2* __restrict__ part, int64_t i) {
  const uint32_t T = dv.T;
  const uint32_t lo = (uint32_t)p0 + (uint32_t)i;
  const uint32_t hi = (uint32_t)p1 + (uint32_t)i;
  const uint32_t qlo = divu32(lo, dv);
  const uint32_t b0 = qlo + (lo != qlo * T);   // first boundary at or after lo
  const uint32_t b1 = divu32(hi, dv);          // last boundary at or before hi
  const bool snap = (p1 - p0) < snap_len;
  const uint32_t bend = min(b1 + 1, (uint32_t)tiles);
  for (uint32_t b = b0; b < bend; b++)   // b * T <= hi < 2^32
    part[b] = (snap && b > 0) ? make_int2((int)i + 1, p1) : make_int2((int)i, (int)(b * T - (uint32_t)i));
}

// Rows 4g .. 4g+3 (and the end marker when row n falls in the group).  Each thread reads its
// five pos entries at once (one 16-byte load when pos is 16-byte aligned), so the pass needs a
// quarter of the dependent load round trips of one row per thread.
__device__ __forceinline__ void partition_rows4(const int32_t* __restrict__ pos, int32_t n,
                                                int64_t nnz, const DivU32& dv, int32_t tiles,
                                                int32_t snap_len, int2* __restrict__ part,
                                                int64_t g, bool vec) {
  const int64_t i0 = 4 * g;
  if (i0 > n) return;
  int32_t p[5];
  if (vec && i0 + 4 <= n) {
    const int4 v = __ldg(reinterpret_cast<const int4*>(pos + i0));
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
    p[3] = v.w;
    p[4] = __ldg(pos + i0 + 4);
  } else {
#pragma unroll
    for (int j = 0; j < 5; j++) p[j] = (i0 + j <= n) ? __ldg(pos + i0 + j) : 0;
  }
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int64_t i = i0 + j;
    if (i > n) break;
    if (i == n) {
      part[tiles] = make_int2(n, (int)nnz);
      break;
    }
    partition_row_body(p[j], p[j + 1], dv, tiles, snap_len, part, i);
  }
}

__global__ void merge_partition_scatter(const int32_t* __restrict__ pos, int32_t n,
                                        int64_t nnz, DivU32 dv, int32_t tiles,
                                        int32_t snap_len, int2* __restrict__ part) {
  const bool vec = ((uintptr_t)pos & 15) == 0;
  partition_rows4(pos, n, nnz, dv, tiles, snap_len, part,
                  (int64_t)blockIdx.x * blockDim.x + threadIdx.x, vec);
}

// One pass before the double-float SpMV: thread g writes the tile boundaries inside rows
// 4g .. 4g+3 (as merge_partition_scatter) and splits x[4g .. 4g+3] into double-float pairs,
// setting *xflag when an entry lies outside the pairs' range (zeros split exactly).  *xflag is
// cleared by the fix-up kernel at the end of the same product.
__global__ void spmv_prep(const int32_t* __restrict__ pos, int32_t n, int64_t nnz, DivU32 dv,
                          int32_t tiles, int2* __restrict__ part, const double* __restrict__ x,
                          DF* __restrict__ xdf, int32_t cols, int* __restrict__ xflag) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t c0 = 4 * g;
  if (c0 < cols) {
    double v[4];
    if ((((uintptr_t)x | (uintptr_t)xdf) & 15) == 0 && c0 + 4 <= cols) {
      const double2 a = __ldg(reinterpret_cast<const double2*>(x + c0));
      const double2 b = __ldg(reinterpret_cast<const double2*>(x + c0 + 2));
      v[0] = a.x;
      v[1] = a.y;
      v[2] = b.x;
      v[3] = b.y;
    } else {
#pragma unroll
      for (int j = 0; j < 4; j++) v[j] = (c0 + j < cols) ? __ldg(x + c0 + j) : 0.0;
    }
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      DF d;
      ok &= split_df(v[j], d.h, d.l);
      if (c0 + j < cols) xdf[c0 + j] = d;
    }
    if (!ok) *xflag = 1;
  }
  partition_rows4(pos, n, nnz, dv, tiles, 0, part, g, ((uintptr_t)pos & 15) == 0);
}

// Threads needed by the four-rows-per-thread passes over n + 1 pos entries (and cols).
inline int64_t rows4_threads(int64_t n_plus_1, int64_t cols = 0) {
  return (std::max(n_plus_1, cols) + 3) / 4;
}

int merge_partition(const int32_t* pos, int32_t n, int64_t nnz, int64_t tile_items,
                    int32_t tiles, int2* part, cudaStream_t st, int32_t snap_len) {
  TACOGB_CHECK_ARG(tile_items > 0 && tile_items < (1ll << 30), "bad merge tile size");
  const int64_t threads = rows4_threads((int64_t)n + 1);
  TACOGB_LAUNCH("merge_partition_scatter", st,
                merge_partition_scatter<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                    pos, n, nnz, make_divu32((uint32_t)tile_items), tiles, snap_len, part));
  return 0;
}

// xg: x in the policy's gather form (pre-split for the double-float policy); x64: the original
// FP64 x for the native fallback (same as xg for unchecked policies); xflag: non-zero when x
// has entries outside the double-float range.
template <class P, int IPT, bool TMA, int CH = 4>
__global__ void __launch_bounds__(kWmBlock, (IPT <= 11 ? 8 : 4))
spmv_wmerge_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                   const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
                   const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
                   typename P::Out* __restrict__ y, const int2* __restrict__ part, int32_t n,
                   int32_t nnz, int32_t* __restrict__ carry_row, double* __restrict__ carry_val,
                   int* status) {
  using S = WmSmem<P, IPT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const int tile = blockIdx.x;
  const int2 c0 = part[tile], c1 = part[tile + 1];
  double carry_d;
  if constexpr (std::is_same<P, PolGP>::value)
    carry_d = gp_process_tile<P, IPT, TMA>(s, pos, crd, vals, xg, x64, xflag, y, n, nnz, c0.x,
                                           c1.x - c0.x, c0.y, c1.y - c0.y, status);
  else
    carry_d = wm_process_tile<P, IPT, TMA, CH>(s, pos, crd, vals, xg, x64, xflag, y, n, nnz, c0.x,
                                               c1.x - c0.x, c0.y, c1.y - c0.y, status);
  if (threadIdx.x == 0) {
    carry_row[tile] = c1.x;
    carry_val[tile] = carry_d;
  }
}

// ------------------------------------------------------------------ wtile -----------------
//
// Warp-level merge tiles (wtile.cuh): CTA b runs tiles 4b .. 4b+3, one per warp, with no CTA
// barrier; each tile's carry-out goes to the fix-up kernel.

// DIRECT tiles store their rows straight to y (WdSmem, no staging area for row results);
// MINB is the CTAs per SM the register allocation must allow (0: by tile size).
template <class P, int IPT, bool TMA, int CH, bool DIRECT = false, int MINB = 0>
__global__ void __launch_bounds__(kWtWarps * 32,
                                  (MINB ? MINB : IPT <= 7 ? 8 : IPT <= 11 ? 6 : 4))
spmv_wtile_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                  const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
                  const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
                  typename P::Out* __restrict__ y, const int2* __restrict__ part, int32_t n,
                  int32_t nnz, int32_t tiles, int32_t* __restrict__ carry_row,
                  double* __restrict__ carry_val, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  using S = typename std::conditional<DIRECT, WdSmem<P, IPT>, WtSmem<P, IPT>>::type;
  S& s = reinterpret_cast<S*>(smem_raw)[warp];
  const int t = blockIdx.x * kWtWarps + warp;
  if (t >= tiles) return;  // whole warp: nothing below synchronises more than one warp
  const int2 c0 = part[t], c1 = part[t + 1];
  double first_val;
  const double c = wt_process<P, IPT, TMA, CH>(s, pos, crd, vals, xg, x64, xflag, y, n, nnz, c0.x,
                                               c1.x - c0.x, c0.y, c1.y - c0.y, status, first_val);
  // One carry per tile, added by the fix-up kernel.  (Chaining a CTA's four carries before it
  // exits measured slower: any hand-off between warps lengthens the CTA's life.)
  if ((threadIdx.x & 31) == 0) {
    carry_row[t] = c1.x;
    carry_val[t] = c;
  }
}

// Persistent warp pipeline (wtile.cuh, WpSmem): warp w of the grid walks tiles
// [tiles*w/W, tiles*(w+1)/W) with double-buffered staging and chains the open row's carry in a
// register; one carry per warp goes to the fix-up kernel.
template <class P, int IPT, int CH, bool STRIDED>
__global__ void __launch_bounds__(kWtWarps * 32, 6)
spmv_wpipe_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                  const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
                  const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
                  typename P::Out* __restrict__ y, const int2* __restrict__ part, int32_t n,
                  int32_t nnz, int32_t tiles, int32_t* __restrict__ carry_row,
                  double* __restrict__ carry_val, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WpSmem<P, IPT>& s = reinterpret_cast<WpSmem<P, IPT>*>(smem_raw)[warp];
  const int64_t W = (int64_t)gridDim.x * kWtWarps, gw = (int64_t)blockIdx.x * kWtWarps + warp;
  // contiguous runs chain carries; strided assignment (tiles gw, gw + W, ...) keeps the warps
  // of the grid streaming one window of the matrix and writes one carry per tile
  const int tstep = STRIDED ? (int)W : 1;
  const int t0 = STRIDED ? (int)gw : (int)(tiles * gw / W);
  const int t1 = STRIDED ? tiles : (int)(tiles * (gw + 1) / W);
  auto next_t = [&](int t) { return t + tstep; };
  if (lane == 0) {
    mbar_init(&s.bar[0], 1);
    mbar_init(&s.bar[1], 1);
  }
  __syncwarp();
  const bool xok = (xflag == nullptr || *xflag == 0);
  double carry_in = 0.0;
  const int tf = min(t0, tiles);
  int2 c0 = part[tf], c1 = part[t0 < t1 ? tf + 1 : tf];
  int3 off_cur = make_int3(0, 0, 0), off_next = make_int3(0, 0, 0);
  if (t0 < t1)
    off_cur = wp_issue<P, IPT>(s.st[0], &s.bar[0], pos, crd, vals, n, nnz, c0.x, c1.x - c0.x,
                               c0.y, c1.y - c0.y);
  for (int t = t0, i = 0; t < t1; t = next_t(t), i++) {
    const int buf = i & 1;
    const int r0 = c0.x, k0 = c0.y, rn = c1.x - c0.x, kn = c1.y - c0.y;
    int2 nc0 = c1, nc1 = c1;
    const int tn = next_t(t);
    if (tn < t1) {
      nc0 = part[tn];
      nc1 = part[tn + 1];
      off_next = wp_issue<P, IPT>(s.st[buf ^ 1], &s.bar[buf ^ 1], pos, crd, vals, n, nnz, nc0.x,
                                  nc1.x - nc0.x, nc0.y, nc1.y - nc0.y);
    }
    __syncwarp();  // every lane's tail loads of this stage are visible
    mbar_wait_or_flag(&s.bar[buf], (uint32_t)((i >> 1) & 1), status);
    const WpStage<P, IPT>& g = s.st[buf];
    const int32_t* scrd = g.crd + off_cur.x;
    const typename P::Val* sval = g.val + off_cur.y;
    const int32_t* sre = g.re + off_cur.z;
    int row, ks;
    tile_search(sre, rn, kn, k0, min(lane * IPT, rn + kn), row, ks);
    int row_e = __shfl_down_sync(0xffffffffu, row, 1), ke = __shfl_down_sync(0xffffffffu, ks, 1);
    if (lane == 31) {
      row_e = rn;
      ke = kn;
    }
    double c;
    bool native = !P::kChecked;
    if constexpr (P::kChecked) {
      typename P::Acc open, first;
      int first_row;
      bool ok = xok;
      if (__all_sync(0xffffffffu, ok))
        ok = wt_walk<P, IPT, CH>(scrd, sval, sre, xg, row, ks, row_e, ke, k0, SinkSmem{s.y},
                                 open, first, first_row);
      if (__all_sync(0xffffffffu, ok)) {
        const typename P::Acc cc = wt_join<P>(open, row_e, first, first_row, SinkSmem{s.y});
        __syncwarp();
        for (int q = lane; q < rn; q += 32) {
          double v = P::to_double(as_acc<typename P::Acc>(s.y[q]));
          if (q == 0) v = __dadd_rn(v, carry_in);
          y[r0 + q] = (typename P::Out)v;
        }
        c = P::to_double(cc);
      } else {
        native = true;
      }
    }
    if (native) {
      using Q = typename std::conditional<P::kChecked, PolNative64, P>::type;
      typename Q::Acc open, first;
      int first_row;
      wt_walk<Q, IPT, CH>(scrd, (const typename Q::Val*)sval, sre, (const typename Q::XG*)x64,
                          row, ks, row_e, ke, k0, SinkSmem{s.y}, open, first, first_row);
      const typename Q::Acc cc = wt_join<Q>(open, row_e, first, first_row, SinkSmem{s.y});
      __syncwarp();
      for (int q = lane; q < rn; q += 32) {
        double v = Q::to_double(as_acc<typename Q::Acc>(s.y[q]));
        if (q == 0) v = __dadd_rn(v, carry_in);
        y[r0 + q] = (typename P::Out)v;
      }
      c = Q::to_double(cc);
    }
    if constexpr (STRIDED) {
      if (lane == 0) {
        carry_row[t] = c1.x;
        carry_val[t] = c;
      }
    } else {
      carry_in = (rn > 0) ? c : __dadd_rn(carry_in, c);
    }
    __syncwarp();  // this stage and the row staging are free before they are reused
    c0 = nc0;
    c1 = nc1;
    off_cur = off_next;
  }
  if (!STRIDED && lane == 0) {
    // a warp without tiles reports the row at its merge position with a zero carry, so that
    // the carries of a row stay one consecutive run for the fix-up kernel
    carry_row[gw] = part[t1].x;
    carry_val[gw] = carry_in;
  }
}

// ------------------------------------------------------------------ pmerge ----------------
//
// Persistent form of wmerge: CTA b owns the contiguous tile range [tiles*b/G, tiles*(b+1)/G).
// Two shared-memory stages alternate: while the CTA walks tile t from one stage, the bulk copies
// of tile t+1 land in the other, so DRAM latency leaves the critical path.  A row that runs from
// one of the CTA's tiles into the next is chained through a register (carry_in, FP64), so only
// one carry per CTA reaches the fix-up kernel.

template <class P, int IPT>
struct PmStage {
  using Val = typename P::Val;
  static constexpr int ITEMS = kWmBlock * IPT;
  static constexpr int VPAD = 16 / sizeof(Val);
  alignas(16) int32_t crd[ITEMS + 8];
  alignas(16) Val val[ITEMS + 2 * VPAD];
  alignas(16) int32_t re[ITEMS + 8];
};

template <class P, int IPT>
struct PmSmem {
  PmStage<P, IPT> st[2];
  double y[kWmBlock * IPT];
  int2 lane_start[kWmBlock + 1];
  int32_t wkey[kWmWarps];
  double wval[kWmWarps];
  uint64_t bar[2];
};

// Issues the copies of tile (r0, rn, k0, kn) into stage buf: thread 0 the bulk copies over the
// 16-byte-aligned spans, every thread its share of the sub-16-byte tails at the array ends.
// Returns the offsets of the tile's first crd/val/row-end element inside the stage.
template <class P, int IPT>
__device__ __forceinline__ int3 pm_issue(PmSmem<P, IPT>& s, int buf,
                                         const int32_t* __restrict__ pos,
                                         const int32_t* __restrict__ crd,
                                         const typename P::Val* __restrict__ vals, int32_t n,
                                         int32_t nnz, int r0, int rn, int k0, int kn) {
  using Val = typename P::Val;
  constexpr int VP = PmStage<P, IPT>::VPAD;
  PmStage<P, IPT>& g = s.st[buf];
  const int tid = threadIdx.x;
  const int k1 = k0 + kn;
  const int a = k0 & ~3, b = max(a, min((k1 + 3) & ~3, nnz & ~3));
  const int av = k0 & ~(VP - 1), bv = max(av, min((k1 + VP - 1) & ~(VP - 1), nnz & ~(VP - 1)));
  const int q0 = r0 + 1, q1 = r0 + 1 + rn;
  const int ar = q0 & ~3, br = max(ar, min((q1 + 3) & ~3, (n + 1) & ~3));
  if (tid == 0) {
    // generic-proxy reads of this stage (the tile before last) precede the async overwrite
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(&s.bar[buf], (uint32_t)((b - a) * 4 + (bv - av) * (int)sizeof(Val) +
                                                  (br - ar) * 4));
    if (b > a) tma_load_bulk(g.crd, crd + a, (uint32_t)(b - a) * 4, &s.bar[buf]);
    if (bv > av) tma_load_bulk(g.val, vals + av, (uint32_t)(bv - av) * sizeof(Val), &s.bar[buf]);
    if (br > ar) tma_load_bulk(g.re, pos + ar, (uint32_t)(br - ar) * 4, &s.bar[buf]);
  }
  for (int i = max(b, k0) + tid; i < k1; i += kWmBlock) g.crd[i - a] = crd[i];
  for (int i = max(bv, k0) + tid; i < k1; i += kWmBlock) g.val[i - av] = vals[i];
  for (int i = max(br, q0) + tid; i < q1; i += kWmBlock) g.re[i - ar] = __ldg(pos + i);
  return make_int3(k0 - a, k0 - av, q0 - ar);
}

template <class P, int IPT>
__global__ void __launch_bounds__(kWmBlock, 6)
spmv_pmerge_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                   const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
                   const typename P::Val* __restrict__ x64, typename P::Out* __restrict__ y,
                   const int2* __restrict__ part, int32_t n, int32_t nnz, int32_t tiles,
                   int32_t* __restrict__ carry_row, double* __restrict__ carry_val,
                   int* status) {
  using S = PmSmem<P, IPT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const int tid = threadIdx.x;
  const int G = gridDim.x, cb = blockIdx.x;
  const int t0 = (int)((int64_t)tiles * cb / G), t1 = (int)((int64_t)tiles * (cb + 1) / G);
  if (tid == 0) {
    mbar_init(&s.bar[0], 1);
    mbar_init(&s.bar[1], 1);
  }
  __syncthreads();
  double carry_in = 0.0;  // thread 0: part of the open row from this CTA's earlier tiles
  int3 off_cur = make_int3(0, 0, 0), off_next = make_int3(0, 0, 0);
  int2 c0 = part[t0], c1 = part[t0 < t1 ? t0 + 1 : t0];
  if (t0 < t1) off_cur = pm_issue<P, IPT>(s, 0, pos, crd, vals, n, nnz, c0.x, c1.x - c0.x, c0.y,
                                          c1.y - c0.y);
  for (int t = t0, i = 0; t < t1; t++, i++) {
    const int buf = i & 1;
    const int r0 = c0.x, k0 = c0.y, rn = c1.x - c0.x, kn = c1.y - c0.y;
    int2 n1 = c1;
    if (t + 1 < t1) {
      n1 = part[t + 2];
      off_next = pm_issue<P, IPT>(s, buf ^ 1, pos, crd, vals, n, nnz, c1.x, n1.x - c1.x, c1.y,
                                  n1.y - c1.y);
    }
    mbar_wait_or_flag(&s.bar[buf], (uint32_t)((i >> 1) & 1), status);
    __syncthreads();
    const PmStage<P, IPT>& g = s.st[buf];
    const int32_t* scrd = g.crd + off_cur.x;
    const typename P::Val* sval = g.val + off_cur.y;
    const int32_t* sre = g.re + off_cur.z;

    double carry_d = 0.0;
    bool native = !P::kChecked;
    if constexpr (P::kChecked) {
      typename P::Acc carry = P::zero();
      const bool ok = wm_tile<P, IPT>(s, scrd, sval, sre, xg, rn, kn, k0, carry);
      if (__syncthreads_and(ok)) {
        for (int q = tid; q < rn; q += kWmBlock) {
          double v = P::to_double(as_acc<typename P::Acc>(s.y[q]));
          if (q == 0) v += carry_in;
          y[r0 + q] = (typename P::Out)v;
        }
        carry_d = P::to_double(carry);
      } else {
        native = true;
      }
    }
    if (native) {
      using Q = typename std::conditional<P::kChecked, PolNative64, P>::type;
      typename Q::Acc carry = Q::zero();
      wm_tile<Q, IPT>(s, scrd, (const typename Q::Val*)sval, sre, (const typename Q::XG*)x64, rn,
                      kn, k0, carry);
      for (int q = tid; q < rn; q += kWmBlock) {
        double v = Q::to_double(as_acc<typename Q::Acc>(s.y[q]));
        if (q == 0) v += carry_in;
        y[r0 + q] = (typename P::Out)v;
      }
      carry_d = Q::to_double(carry);
    }
    if (tid == 0) carry_in = (rn > 0) ? carry_d : carry_in + carry_d;
    __syncthreads();  // this stage's readers are done before the next iteration reuses it
    c0 = c1;
    c1 = n1;
    off_cur = off_next;
  }
  if (tid == 0) {
    carry_row[cb] = part[t1].x;  // a CTA without tiles keeps the run of carries unbroken
    carry_val[cb] = carry_in;
  }
}

// Adds the tile carry-outs to the rows that continue into later tiles.  Tiles carrying the same
// row are consecutive (carry rows never decrease in tile order); the first tile of each run
// sums the run in tile order, one entry at a time, so the result is that of a serial sum.
// xflag (optional) is the x-range flag of the product, cleared here for the next one.
// Fetching a run 8, 16 or 32 entries at a time shortens the longest run's chain of dependent
// loads but loads past the end of every short run, and measured slower on a power-law matrix
// (4.19M rows, runs up to 57 tiles: 22 us serial, 24-43 us chunked).
template <typename Out>
__global__ void spmv_carry_fixup(const int32_t* __restrict__ carry_row,
                                 const double* __restrict__ carry_val, int32_t tiles,
                                 Out* __restrict__ y, int32_t n, int* __restrict__ xflag = nullptr) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0 && xflag != nullptr) *xflag = 0;
  if (t >= tiles) return;
  // every load the common case needs is issued before any of them is tested: a run of equal
  // carry rows almost always ends at the next tile (only rows longer than a tile span more),
  // so one tile of lookahead, and a loop for the rest
  const int32_t r = carry_row[t];
  const int32_t rp = t > 0 ? carry_row[t - 1] : -1;
  double tot = carry_val[t];
  int32_t u = t + 1;
  int32_t ru = u < tiles ? carry_row[u] : -1;
  if (r >= n || rp == r) return;
  const Out y0 = y[r];
  while (ru == r) {
    tot += carry_val[u];
    u++;
    ru = u < tiles ? carry_row[u] : -1;
  }
  y[r] = (Out)((double)y0 + tot);
}

// ------------------------------------------------------------------ vector ----------------

template <typename V, int G>
__global__ void __launch_bounds__(256)
spmv_vector_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                   const V* __restrict__ vals, const V* __restrict__ x, V* __restrict__ y,
                   int32_t n) {
  using P = typename std::conditional<sizeof(V) == 8, PolNative64, PolComp32>::type;
  const int lane = threadIdx.x & (G - 1);
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t gid = gtid / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  // Every lane of a warp runs the same number of outer iterations so that the shuffles below
  // always see the full warp.
  const int64_t warp_first = (gtid & ~31ll) / G;
  for (int64_t base = warp_first; base < n; base += ngroups) {
    const int64_t row = base + (gid - warp_first);
    typename P::Acc acc = P::zero();
    if (row < n) {
      const int32_t p1 = __ldg(pos + row + 1);
      for (int32_t p = __ldg(pos + row) + lane; p < p1; p += G)
        P::madd(acc, vals[p], __ldg(x + ld_stream_i32(crd + p)));
    }
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) acc = P::add(acc, P::shfl_xor(acc, m));
    if (row < n && lane == 0) y[row] = P::out(acc);
  }
}

// ------------------------------------------------------------------ host side -------------

namespace {

struct SpmvVariant {
  const char* name;
  int family;  // 0 wmerge native, 1 wmerge double-float (x pre-split), 2 vector,
               // 3 wmerge double-float (x split in the walk), 4 pmerge native,
               // 5 pmerge double-float (x split in the walk), 6 wmerge hybrid
               // (DFMA and double-float items interleaved), 7 family 3 with 8-deep gathers,
               // 8 family 3 with four accumulators, 9 both, 10 wmerge PolDFS (x split in the
               // partition pass, eight-instruction value split), 11 family 10, 8-deep gathers,
               // 12 gmerge: product-staged tiles (gathers and products in nonzero order, then
               // a walk over products in shared memory), 13 wtile (warp-level merge tiles)
               // with PolDFS, 14 wtile native, 15 wpipe (persistent double-buffered warp
               // tiles) with PolDFS, 16 wpipe native, 17 wpipe PolDFS with 8-deep gathers
  int param;   // IPT for wmerge, G for vector
};

const SpmvVariant kSpmvVariants[] = {
    {"wmerge_ipt7", 0, 7},       {"wmerge_ipt11", 0, 11},     {"wmerge_df_ipt7", 1, 7},
    {"wmerge_df_ipt11", 1, 11},  {"vector_g1", 2, 1},         {"vector_g2", 2, 2},
    {"vector_g4", 2, 4},         {"vector_g8", 2, 8},         {"vector_g16", 2, 16},
    {"vector_g32", 2, 32},       {"wmerge_dfx_ipt7", 3, 7},   {"wmerge_dfx_ipt11", 3, 11},
    {"pmerge_ipt7", 4, 7},       {"pmerge_dfx_ipt7", 5, 7},   {"pmerge_dfx_ipt11", 5, 11},
    {"wmerge_hyb_ipt7", 6, 7},   {"wmerge_hyb_ipt11", 6, 11},
    {"wmerge_dfx_ipt7_c8", 7, 7}, {"wmerge_dfx4_ipt7", 8, 7}, {"wmerge_dfx_ipt5", 3, 5},
    {"wmerge_dfx_ipt9", 3, 9},   {"wmerge_dfx4_ipt11_c8", 9, 11},
    {"wmerge_dfs_ipt7", 10, 7},  {"wmerge_dfs_ipt11", 10, 11}, {"wmerge_dfs_ipt15", 10, 15},
    {"wmerge_dfs_ipt19", 10, 19}, {"wmerge_dfs_ipt15_c8", 11, 15},
    {"gmerge_ipt5", 12, 5},      {"gmerge_ipt7", 12, 7},      {"gmerge_ipt9", 12, 9},
    {"gmerge_ipt11", 12, 11},    {"gmerge_ipt15", 12, 15},
    {"wtile_dfs_ipt7", 13, 7},   {"wtile_dfs_ipt9", 13, 9},   {"wtile_dfs_ipt11", 13, 11},
    {"wtile_dfs_ipt15", 13, 15}, {"wtile_native_ipt7", 14, 7},
    {"wpipe_dfs_ipt7", 15, 7},   {"wpipe_dfs_ipt9", 15, 9},   {"wpipe_native_ipt7", 16, 7},
    {"wpipe_dfs_ipt7_c8", 17, 7}, {"wpipe_s_dfs_ipt7", 18, 7}, {"wpipe_s_native_ipt7", 19, 7},
    {"wpipe_s_dfs_ipt9", 18, 9},
    // warp tiles storing rows straight to y: param = IPT + 100 * min CTAs per SM (+ 10000 for
    // 8-deep gathers); family 20 native, 21 PolDFS, 22 hybrid
    {"wtile_d_native_ipt7", 20, 807},    {"wtile_d_native_ipt7_b10", 20, 1007},
    {"wtile_d_native_ipt7_b12", 20, 1207}, {"wtile_d_native_ipt9", 20, 809},
    {"wtile_d_native_ipt11", 20, 611},   {"wtile_d_native_ipt7_c8", 20, 10807},
    {"wtile_d_dfs_ipt7", 21, 807},       {"wtile_d_dfs_ipt9", 21, 809},
    {"wtile_d_dfs_ipt11", 21, 611},      {"wtile_d_hyb_ipt7", 22, 807},
    {"wtile_d_hyb_ipt11", 22, 611},      {"wtile_d_native_ipt9_b10", 20, 1009},
    {"wtile_d_native_ipt11_b8", 20, 811}, {"wtile_d_native_ipt15_b6", 20, 615},
    // warp-specialised persistent tiles: param = IPT + 100 * consumers + 10000 * stages;
    // family 23 native, 24 PolDFS
    {"wspec_native_ipt7_c12s20", 23, 201207}, {"wspec_native_ipt7_c24s40", 23, 402407},
    {"wspec_native_ipt9_c12s16", 23, 161209}, {"wspec_native_ipt11_c8s12", 23, 120811},
    {"wspec_native_ipt7_c8s12", 23, 120807}, {"wspec_dfs_ipt9_c12s16", 24, 161209},
    {"wspec_dfs_ipt7_c12s20", 24, 201207},
};
constexpr int kNumSpmvVariants = sizeof(kSpmvVariants) / sizeof(kSpmvVariants[0]);

template <class P, int IPT, int CH = 4>
int launch_wmerge(const tacogb_csr* A, const typename P::Val* x, typename P::Out* y,
                  cudaStream_t st) {
  using S = WmSmem<P, IPT>;
  const int64_t tile_items = S::ITEMS;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + tile_items - 1) / tile_items;
  if (tiles64 == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31), "SpMV: too many merge tiles");
  const int32_t tiles = (int32_t)tiles64;
  // x pre-split into double-float pairs when the policy gathers DF entries; PolDFS fuses the
  // split into the partition pass and keeps its x-range flag in the device status block.
  constexpr bool fused = std::is_same<P, PolDFS>::value || std::is_same<P, PolGP>::value;
  constexpr bool presplit = std::is_same<typename P::XG, DF>::value && !fused;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const size_t crow_bytes = al((size_t)tiles * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)tiles * sizeof(double));
  const size_t xdf_bytes =
      presplit ? al((size_t)A->cols * sizeof(DF)) + 256 : fused ? al((size_t)A->cols * sizeof(DF)) : 0;
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + xdf_bytes, 0);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  int* status = device_status();
  if (!status) return last_code();
  const typename P::XG* xg = (const typename P::XG*)x;
  const int* xflag = nullptr;
  if constexpr (presplit) {
    int* flag = (int*)(ws + part_bytes + crow_bytes + cval_bytes);
    DF* xdf = (DF*)((unsigned char*)flag + 256);
    TACOGB_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    if (A->cols > 0)
      TACOGB_LAUNCH("spmv_split_x", st,
                    spmv_split_x<<<(A->cols + 255) / 256, 256, 0, st>>>((const double*)x, xdf,
                                                                        A->cols, flag));
    xg = (const typename P::XG*)xdf;
    xflag = flag;
  }
  int* fixup_flag = nullptr;
  if constexpr (fused) {
    DF* xdf = (DF*)(ws + part_bytes + crow_bytes + cval_bytes);
    fixup_flag = status + kXFlagWord;
    const int64_t threads = rows4_threads((int64_t)A->rows + 1, A->cols);
    TACOGB_LAUNCH("spmv_prep", st,
                  spmv_prep<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                      A->pos, A->rows, A->nnz, make_divu32((uint32_t)tile_items), tiles, part,
                      (const double*)x, xdf, A->cols, fixup_flag));
    xg = (const typename P::XG*)xdf;
    xflag = fixup_flag;
  } else {
    if (int rc = merge_partition(A->pos, A->rows, A->nnz, tile_items, tiles, part, st)) return rc;
  }
  // Bulk copies need 16-byte aligned sources: true for every allocator the library meets
  // (cudaMalloc, cudaMallocManaged, torch); sliced pointers take the register-staged kernel.
  const bool tma = (((uintptr_t)A->pos | (uintptr_t)A->crd | (uintptr_t)A->vals) & 15) == 0;
  auto kern = tma ? spmv_wmerge_kernel<P, IPT, true, CH> : spmv_wmerge_kernel<P, IPT, false, CH>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(S)));
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, 85));
  TACOGB_LAUNCH("spmv_wmerge_kernel", st,
                kern<<<tiles, kWmBlock, sizeof(S), st>>>(
                    A->pos, A->crd, (const typename P::Val*)A->vals, xg, x, xflag, y, part,
                    A->rows, (int32_t)A->nnz, crow, cval, status));
  TACOGB_LAUNCH("spmv_carry_fixup", st,
                spmv_carry_fixup<typename P::Out><<<(tiles + 255) / 256, 256, 0, st>>>(
                    crow, cval, tiles, y, A->rows, fixup_flag));
  return 0;
}

template <class P, int IPT, int CH = 4, bool DIRECT = false, int MINB = 0>
int launch_wtile(const tacogb_csr* A, const typename P::Val* x, typename P::Out* y,
                 cudaStream_t st) {
  using S = typename std::conditional<DIRECT, WdSmem<P, IPT>, WtSmem<P, IPT>>::type;
  const int64_t tile_items = S::ITEMS;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + tile_items - 1) / tile_items;
  if (tiles64 == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) - 8, "SpMV: too many merge tiles");
  const int32_t tiles = (int32_t)tiles64;
  constexpr bool split = std::is_same<typename P::XG, DF>::value;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const int grid = (tiles + kWtWarps - 1) / kWtWarps;
  const size_t crow_bytes = al((size_t)tiles * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)tiles * sizeof(double));
  const size_t xdf_bytes = split ? al((size_t)A->cols * sizeof(DF)) : 0;
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + xdf_bytes, 0);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  int* status = device_status();
  if (!status) return last_code();
  const typename P::XG* xg = (const typename P::XG*)x;
  int* xflag = nullptr;
  if constexpr (split) {
    DF* xdf = (DF*)(ws + part_bytes + crow_bytes + cval_bytes);
    xflag = status + kXFlagWord;
    const int64_t threads = rows4_threads((int64_t)A->rows + 1, A->cols);
    TACOGB_LAUNCH("spmv_prep", st,
                  spmv_prep<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                      A->pos, A->rows, A->nnz, make_divu32((uint32_t)tile_items), tiles, part,
                      (const double*)x, xdf, A->cols, xflag));
    xg = (const typename P::XG*)xdf;
  } else {
    if (int rc = merge_partition(A->pos, A->rows, A->nnz, tile_items, tiles, part, st)) return rc;
  }
  const bool tma = (((uintptr_t)A->pos | (uintptr_t)A->crd | (uintptr_t)A->vals) & 15) == 0;
  auto kern = tma ? spmv_wtile_kernel<P, IPT, true, CH, DIRECT, MINB>
                  : spmv_wtile_kernel<P, IPT, false, CH, DIRECT, MINB>;
  const int smem = (int)(sizeof(S) * kWtWarps);
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  // carveouts measured best per tile size (random-column gathers want L1 room; the banded
  // matrices run fastest at IPT 9 with the driver's choice)
  // direct tiles: the smallest carveout of 160 KB or 196 KB that holds MINB CTAs
  constexpr int carve = DIRECT ? ((int)sizeof(S) * kWtWarps * MINB > 160 * 1024 ? 86 : 70)
                        : IPT == 7 ? 70 : IPT == 9 ? -1 : 85;
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, carve));
  TACOGB_LAUNCH("spmv_wtile_kernel", st,
                kern<<<grid, kWtWarps * 32, smem, st>>>(
                    A->pos, A->crd, (const typename P::Val*)A->vals, xg, x, xflag, y, part,
                    A->rows, (int32_t)A->nnz, tiles, crow, cval, status));
  TACOGB_LAUNCH("spmv_carry_fixup", st,
                spmv_carry_fixup<typename P::Out><<<(tiles + 255) / 256, 256, 0, st>>>(
                    crow, cval, tiles, y, A->rows, xflag));
  return 0;
}

// Warp-specialised persistent tiles (wspec.cuh): C consumer warps and one producer warp per
// CTA over a ring of S stages, as many CTAs as fit on the GPU at once.
template <class P, int IPT, int C, int S, int CH = 4>
int launch_wspec(const tacogb_csr* A, const typename P::Val* x, typename P::Out* y,
                 cudaStream_t st) {
  static_assert(S <= 32 * (C + 1), "one thread initialises each stage's barriers");
  using SM = WsSmem<P, IPT, S>;
  const int64_t tile_items = 32 * IPT;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + tile_items - 1) / tile_items;
  if (tiles64 == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) - 8, "SpMV: too many merge tiles");
  const int32_t tiles = (int32_t)tiles64;
  // bulk copies need 16-byte aligned sources; otherwise the warp tiles' plain-load form runs
  if ((((uintptr_t)A->pos | (uintptr_t)A->crd | (uintptr_t)A->vals) & 15) != 0)
    return launch_wtile<P, IPT, CH, true, 8>(A, x, y, st);
  auto kern = spmv_wspec_kernel<P, IPT, C, S, CH>;
  const int smem = (int)sizeof(SM);
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  // 160 KB of shared memory (96 KB of L1 for the gathers) unless two CTAs fit only in 196 KB
  const bool two_in_196 = 2 * smem > 160 * 1024 && 2 * smem <= 196 * 1024;
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, two_in_196 ? 86 : 70));
  int per_sm = 0;
  TACOGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (C + 1) * 32,
                                                                smem));
  if (per_sm < 1) per_sm = 1;
  const int grid = (int)std::min<int64_t>(tiles64, (int64_t)sm_count() * per_sm);
  constexpr bool split = std::is_same<typename P::XG, DF>::value;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const size_t crow_bytes = al((size_t)tiles * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)tiles * sizeof(double));
  const size_t xdf_bytes = split ? al((size_t)A->cols * sizeof(DF)) : 0;
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + xdf_bytes, 0);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  int* status = device_status();
  if (!status) return last_code();
  const typename P::XG* xg = (const typename P::XG*)x;
  int* xflag = nullptr;
  if constexpr (split) {
    DF* xdf = (DF*)(ws + part_bytes + crow_bytes + cval_bytes);
    xflag = status + kXFlagWord;
    const int64_t threads = rows4_threads((int64_t)A->rows + 1, A->cols);
    TACOGB_LAUNCH("spmv_prep", st,
                  spmv_prep<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                      A->pos, A->rows, A->nnz, make_divu32((uint32_t)tile_items), tiles, part,
                      (const double*)x, xdf, A->cols, xflag));
    xg = (const typename P::XG*)xdf;
  } else {
    if (int rc = merge_partition(A->pos, A->rows, A->nnz, tile_items, tiles, part, st)) return rc;
  }
  TACOGB_LAUNCH("spmv_wspec_kernel", st,
                kern<<<grid, (C + 1) * 32, smem, st>>>(
                    A->pos, A->crd, (const typename P::Val*)A->vals, xg, x, xflag, y, part,
                    A->rows, (int32_t)A->nnz, tiles, crow, cval, status));
  TACOGB_LAUNCH("spmv_carry_fixup", st,
                spmv_carry_fixup<typename P::Out><<<(tiles + 255) / 256, 256, 0, st>>>(
                    crow, cval, tiles, y, A->rows, xflag));
  return 0;
}

template <class P, int IPT, int CH = 4, bool STRIDED = false>
int launch_wpipe(const tacogb_csr* A, const typename P::Val* x, typename P::Out* y,
                 cudaStream_t st) {
  using S = WpSmem<P, IPT>;
  const int64_t tile_items = 32 * IPT;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + tile_items - 1) / tile_items;
  if (tiles64 == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) - 8, "SpMV: too many merge tiles");
  const int32_t tiles = (int32_t)tiles64;
  // bulk copies need 16-byte aligned sources; otherwise the non-persistent warp tiles run
  if ((((uintptr_t)A->pos | (uintptr_t)A->crd | (uintptr_t)A->vals) & 15) != 0)
    return launch_wtile<P, IPT, CH>(A, x, y, st);
  auto kern = spmv_wpipe_kernel<P, IPT, CH, STRIDED>;
  const int smem = (int)(sizeof(S) * kWtWarps);
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, 85));
  int per_sm = 0;
  TACOGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWtWarps * 32,
                                                                smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t warps64 = std::min<int64_t>(tiles64, (int64_t)sm_count() * per_sm * kWtWarps);
  const int grid = (int)((warps64 + kWtWarps - 1) / kWtWarps);
  const int nw = STRIDED ? tiles : grid * kWtWarps;  // carry entries
  constexpr bool split = std::is_same<typename P::XG, DF>::value;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const size_t crow_bytes = al((size_t)nw * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)nw * sizeof(double));
  const size_t xdf_bytes = split ? al((size_t)A->cols * sizeof(DF)) : 0;
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes + xdf_bytes, 0);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  int* status = device_status();
  if (!status) return last_code();
  const typename P::XG* xg = (const typename P::XG*)x;
  int* xflag = nullptr;
  if constexpr (split) {
    DF* xdf = (DF*)(ws + part_bytes + crow_bytes + cval_bytes);
    xflag = status + kXFlagWord;
    const int64_t threads = rows4_threads((int64_t)A->rows + 1, A->cols);
    TACOGB_LAUNCH("spmv_prep", st,
                  spmv_prep<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                      A->pos, A->rows, A->nnz, make_divu32((uint32_t)tile_items), tiles, part,
                      (const double*)x, xdf, A->cols, xflag));
    xg = (const typename P::XG*)xdf;
  } else {
    if (int rc = merge_partition(A->pos, A->rows, A->nnz, tile_items, tiles, part, st)) return rc;
  }
  TACOGB_LAUNCH("spmv_wpipe_kernel", st,
                kern<<<grid, kWtWarps * 32, smem, st>>>(
                    A->pos, A->crd, (const typename P::Val*)A->vals, xg, x, xflag, y, part,
                    A->rows, (int32_t)A->nnz, tiles, crow, cval, status));
  TACOGB_LAUNCH("spmv_carry_fixup", st,
                spmv_carry_fixup<typename P::Out><<<(nw + 255) / 256, 256, 0, st>>>(
                    crow, cval, nw, y, A->rows, xflag));
  return 0;
}

template <class P, int IPT>
int launch_pmerge(const tacogb_csr* A, const typename P::Val* x, typename P::Out* y,
                  cudaStream_t st) {
  using S = PmSmem<P, IPT>;
  const int64_t tile_items = (int64_t)kWmBlock * IPT;
  const int64_t total = (int64_t)A->rows + A->nnz;
  const int64_t tiles64 = (total + tile_items - 1) / tile_items;
  if (tiles64 == 0) return 0;
  TACOGB_CHECK_ARG(tiles64 < (1ll << 31) - 2, "SpMV: too many merge tiles");
  const int32_t tiles = (int32_t)tiles64;
  auto kern = spmv_pmerge_kernel<P, IPT>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(S)));
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, -1));
  int per_sm = 0;
  TACOGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWmBlock,
                                                                sizeof(S)));
  if (per_sm < 1) per_sm = 1;
  const int64_t grid64 = std::min<int64_t>(tiles64, (int64_t)sm_count() * per_sm);
  const int grid = (int)grid64;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const size_t crow_bytes = al((size_t)grid * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)grid * sizeof(double));
  unsigned char* ws = (unsigned char*)scratch(part_bytes + crow_bytes + cval_bytes, 0);
  if (!ws) return last_code();
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + part_bytes);
  double* cval = (double*)(ws + part_bytes + crow_bytes);
  int* status = device_status();
  if (!status) return last_code();
  if (int rc = merge_partition(A->pos, A->rows, A->nnz, tile_items, tiles, part, st)) return rc;
  TACOGB_LAUNCH("spmv_pmerge_kernel", st,
                kern<<<grid, kWmBlock, sizeof(S), st>>>(
                    A->pos, A->crd, (const typename P::Val*)A->vals,
                    (const typename P::XG*)x, x, y, part, A->rows, (int32_t)A->nnz, tiles, crow,
                    cval, status));
  TACOGB_LAUNCH("spmv_carry_fixup", st,
                spmv_carry_fixup<typename P::Out><<<(grid + 255) / 256, 256, 0, st>>>(
                    crow, cval, grid, y, A->rows));
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
  using Native = typename std::conditional<sizeof(V) == 8, PolNative64, PolComp32>::type;
  using Dbl = typename std::conditional<sizeof(V) == 8, PolDF64, PolComp32>::type;
  if (v.family == 0) {
    if (v.param == 7) return launch_wmerge<Native, 7>(A, x, y, st);
    return launch_wmerge<Native, 11>(A, x, y, st);
  }
  if (v.family == 1) {
    if (v.param == 7) return launch_wmerge<Dbl, 7>(A, x, y, st);
    return launch_wmerge<Dbl, 11>(A, x, y, st);
  }
  using DblX = typename std::conditional<sizeof(V) == 8, PolDF64X, PolComp32>::type;
  if (v.family == 3) {
    switch (v.param) {
      case 5: return launch_wmerge<DblX, 5>(A, x, y, st);
      case 7: return launch_wmerge<DblX, 7>(A, x, y, st);
      case 9: return launch_wmerge<DblX, 9>(A, x, y, st);
      default: return launch_wmerge<DblX, 11>(A, x, y, st);
    }
  }
  using DblX4 = typename std::conditional<sizeof(V) == 8, PolDF64X4, PolComp32>::type;
  if (v.family == 7) return launch_wmerge<DblX, 7, 8>(A, x, y, st);
  if (v.family == 8) return launch_wmerge<DblX4, 7>(A, x, y, st);
  if (v.family == 9) return launch_wmerge<DblX4, 11, 8>(A, x, y, st);
  if (v.family == 10 || v.family == 11) {
    if constexpr (sizeof(V) == 8) {
      if (v.family == 11) return launch_wmerge<PolDFS, 15, 8>(A, x, y, st);
      switch (v.param) {
        case 7: return launch_wmerge<PolDFS, 7>(A, x, y, st);
        case 11: return launch_wmerge<PolDFS, 11>(A, x, y, st);
        case 15: return launch_wmerge<PolDFS, 15>(A, x, y, st);
        default: return launch_wmerge<PolDFS, 19>(A, x, y, st);
      }
    } else {
      return launch_wmerge<PolComp32, 7>(A, x, y, st);
    }
  }
  if (v.family == 12) {
    if constexpr (sizeof(V) == 8) {
      switch (v.param) {
        case 5: return launch_wmerge<PolGP, 5>(A, x, y, st);
        case 7: return launch_wmerge<PolGP, 7>(A, x, y, st);
        case 9: return launch_wmerge<PolGP, 9>(A, x, y, st);
        case 11: return launch_wmerge<PolGP, 11>(A, x, y, st);
        default: return launch_wmerge<PolGP, 15>(A, x, y, st);
      }
    } else {
      return launch_wmerge<PolComp32, 7>(A, x, y, st);
    }
  }
  if (v.family == 13) {
    using Pol = typename std::conditional<sizeof(V) == 8, PolDFS, PolComp32>::type;
    switch (v.param) {
      case 7: return launch_wtile<Pol, 7>(A, x, y, st);
      case 9: return launch_wtile<Pol, 9>(A, x, y, st);
      case 11: return launch_wtile<Pol, 11>(A, x, y, st);
      default: return launch_wtile<Pol, 15>(A, x, y, st);
    }
  }
  if (v.family == 14) return launch_wtile<Native, 7>(A, x, y, st);
  if (v.family == 20) {
    switch (v.param) {
      case 807: return launch_wtile<Native, 7, 4, true, 8>(A, x, y, st);
      case 1007: return launch_wtile<Native, 7, 4, true, 10>(A, x, y, st);
      case 1207: return launch_wtile<Native, 7, 4, true, 12>(A, x, y, st);
      case 809: return launch_wtile<Native, 9, 4, true, 8>(A, x, y, st);
      case 611: return launch_wtile<Native, 11, 4, true, 6>(A, x, y, st);
      case 1009: return launch_wtile<Native, 9, 4, true, 10>(A, x, y, st);
      case 811: return launch_wtile<Native, 11, 4, true, 8>(A, x, y, st);
      case 615: return launch_wtile<Native, 15, 4, true, 6>(A, x, y, st);
      default: return launch_wtile<Native, 7, 8, true, 8>(A, x, y, st);
    }
  }
  if (v.family == 23) {
    switch (v.param) {
      case 201207: return launch_wspec<Native, 7, 12, 20>(A, x, y, st);
      case 402407: return launch_wspec<Native, 7, 24, 40>(A, x, y, st);
      case 161209: return launch_wspec<Native, 9, 12, 16>(A, x, y, st);
      case 120811: return launch_wspec<Native, 11, 8, 12>(A, x, y, st);
      default: return launch_wspec<Native, 7, 8, 12>(A, x, y, st);
    }
  }
  if (v.family == 24) {
    using Pol = typename std::conditional<sizeof(V) == 8, PolDFS, PolComp32>::type;
    if (v.param == 161209) return launch_wspec<Pol, 9, 12, 16>(A, x, y, st);
    return launch_wspec<Pol, 7, 12, 20>(A, x, y, st);
  }
  if (v.family == 21) {
    using Pol = typename std::conditional<sizeof(V) == 8, PolDFS, PolComp32>::type;
    switch (v.param) {
      case 807: return launch_wtile<Pol, 7, 4, true, 8>(A, x, y, st);
      case 809: return launch_wtile<Pol, 9, 4, true, 8>(A, x, y, st);
      default: return launch_wtile<Pol, 11, 4, true, 6>(A, x, y, st);
    }
  }
  if (v.family == 22) {
    using Hyb = typename std::conditional<sizeof(V) == 8, PolHybrid, PolComp32>::type;
    if (v.param == 807) return launch_wtile<Hyb, 7, 4, true, 8>(A, x, y, st);
    return launch_wtile<Hyb, 11, 4, true, 6>(A, x, y, st);
  }
  if (v.family == 15 || v.family == 17) {
    using Pol = typename std::conditional<sizeof(V) == 8, PolDFS, PolComp32>::type;
    if (v.family == 17) return launch_wpipe<Pol, 7, 8>(A, x, y, st);
    if (v.param == 9) return launch_wpipe<Pol, 9>(A, x, y, st);
    return launch_wpipe<Pol, 7>(A, x, y, st);
  }
  if (v.family == 16) return launch_wpipe<Native, 7>(A, x, y, st);
  if (v.family == 18) {
    using Pol = typename std::conditional<sizeof(V) == 8, PolDFS, PolComp32>::type;
    if (v.param == 9) return launch_wpipe<Pol, 9, 4, true>(A, x, y, st);
    return launch_wpipe<Pol, 7, 4, true>(A, x, y, st);
  }
  if (v.family == 19) return launch_wpipe<Native, 7, 4, true>(A, x, y, st);
  if (v.family == 4) return launch_pmerge<Native, 7>(A, x, y, st);
  if (v.family == 6) {
    using Hyb = typename std::conditional<sizeof(V) == 8, PolHybrid, PolComp32>::type;
    if (v.param == 7) return launch_wmerge<Hyb, 7>(A, x, y, st);
    return launch_wmerge<Hyb, 11>(A, x, y, st);
  }
  if (v.family == 5) {
    if (v.param == 7) return launch_pmerge<DblX, 7>(A, x, y, st);
    return launch_pmerge<DblX, 11>(A, x, y, st);
  }
  switch (v.param) {
    case 1: return launch_vector<V, 1>(A, x, y, st);
    case 2: return launch_vector<V, 2>(A, x, y, st);
    case 4: return launch_vector<V, 4>(A, x, y, st);
    case 8: return launch_vector<V, 8>(A, x, y, st);
    case 16: return launch_vector<V, 16>(A, x, y, st);
    case 32: return launch_vector<V, 32>(A, x, y, st);
  }
  set_error(TACOGB_ERR_ARG, "SpMV: bad variant %d", variant);
  return TACOGB_ERR_ARG;
}

}  // namespace

int spmv_variant_count() { return kNumSpmvVariants; }
const char* spmv_variant_name(int v) {
  return (v >= 0 && v < kNumSpmvVariants) ? kSpmvVariants[v].name : "";
}

// ---- the library's choice of variant (TACOGB_VARIANT_AUTO) ----
//
// Measured on GB300 (FP64 and compensated FP32): warp tiles that store their rows straight to y
// are fastest on every workload, but the best tile shape depends on where the x gathers go.
// Scattered columns (the power-law matrix) need the L1 for the gathers: 11 items per lane with
// 160 KB of shared memory (96 KB of L1) — 0.433 ms per 1.0e8 nonzeros in FP64.  Local columns
// (the banded matrix) gather from few lines: 9 items per lane with ten CTAs per SM in 196 KB of
// shared memory — 0.413 ms per 1.34e8 nonzeros, where the scattered choice takes 0.494 ms and
// the local choice on the power-law matrix 0.664 ms.  A matrix is local when most gaps between
// consecutive stored columns are short: one small kernel counts, over 4096 evenly spaced
// nonzeros, how many have |crd[p+1] - crd[p]| < 64 (one or a few x lines).  The decision is
// cached per matrix (pos and crd pointers, rows, nonzeros), so an iterated SpMV pays for the
// count once; a call made while its stream is being captured uses the scattered choice
// without counting.
// Matrices of fewer than 2^21 nonzeros are launch-bound rather than gather-bound: there one
// launch beats three (partition, tiles, fix-up) when no row is long.  One small kernel finds the
// longest row (cached the same way), and rows of at most 32 nonzeros run vector_g4 (four lanes
// per row, one launch): 8.1 us against 11.8 us for the warp tiles on the 65,536-row uniform
// matrix (1.0e6 nonzeros, rows of 4-28), both timed as CUDA-graph replays.

namespace {

constexpr int kLocalSamples = 4096;
constexpr int kLocalGap = 64;

__global__ void spmv_locality_kernel(const int32_t* __restrict__ crd, int64_t nnz,
                                     volatile unsigned long long* out) {
  __shared__ int warp_count[8];
  int c = 0;
  for (int i = threadIdx.x; i < kLocalSamples; i += blockDim.x) {
    const int64_t p = (nnz - 1) * (int64_t)i / kLocalSamples;  // p + 1 < nnz
    c += abs(__ldg(crd + p + 1) - __ldg(crd + p)) < kLocalGap;
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) warp_count[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += warp_count[w];
    *out = (unsigned long long)t;  // mapped host memory
    __threadfence_system();
  }
}

// Longest row of a matrix (one block) into mapped host memory.
__global__ void spmv_rowlen_kernel(const int32_t* __restrict__ pos, int32_t n,
                                   volatile unsigned long long* out) {
  __shared__ int warp_max[32];
  int m = 0;
  for (int32_t i = threadIdx.x; i < n; i += blockDim.x)
    m = max(m, __ldg(pos + i + 1) - __ldg(pos + i));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = max(t, warp_max[w]);
    *out = (unsigned long long)t;
    __threadfence_system();
  }
}

// Below this many nonzeros the choice is between one launch and the warp tiles (longest row);
// from it on, between the two tile shapes (locality count).
constexpr int64_t kLocalMinNnz = (int64_t)1 << 21;
constexpr int kVectorMaxRow = 32;

struct AutoEntry {
  const void* pos;
  int32_t rows;
  int64_t nnz;
  int variant;
};
std::mutex g_auto_mu;
std::unordered_map<const void*, AutoEntry> g_auto;  // keyed by crd

int variant_index(const char* name) {
  for (int i = 0; i < kNumSpmvVariants; i++)
    if (std::string(kSpmvVariants[i].name) == name) return i;
  return 0;
}

}  // namespace

int spmv_default_variant(const tacogb_csr* A) {
  (void)A;
  static const int v = variant_index("wtile_d_native_ipt11");
  return v;  // the scattered-column choice: DFMA for FP64 values, compensated FP32 for FP32
}

// The variant TACOGB_VARIANT_AUTO runs for A on stream st (see above).
int spmv_auto_variant(const tacogb_csr* A, cudaStream_t st) {
  static const int scattered = variant_index("wtile_d_native_ipt11");
  static const int local = variant_index("wtile_d_native_ipt9_b10");
  static const int vector = variant_index("vector_g4");
  const bool small = A->nnz < kLocalMinNnz;
  if (A->rows == 0 || A->nnz == 0) return scattered;
  {
    std::lock_guard<std::mutex> lk(g_auto_mu);
    const auto it = g_auto.find(A->crd);
    if (it != g_auto.end() && it->second.pos == A->pos && it->second.rows == A->rows &&
        it->second.nnz == A->nnz)
      return it->second.variant;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return scattered;
  }
  // the count goes straight to the host mailbox: no copy that could queue behind large copies
  // on the copy engines (the pipelined products run this on chunks while copies are in flight)
  unsigned long long* box = host_mailbox();
  if (!box) return scattered;
  volatile unsigned long long* word = box + (small ? kMailboxRowLen : kMailboxLocality);
  count_launch();
  if (small)
    spmv_rowlen_kernel<<<1, 1024, 0, st>>>(A->pos, A->rows, word);
  else
    spmv_locality_kernel<<<1, 256, 0, st>>>(A->crd, A->nnz, word);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
    return scattered;
  const int64_t h = (int64_t)*word;
  const int v = small ? (h <= kVectorMaxRow ? vector : scattered)
                      : (2 * h > kLocalSamples ? local : scattered);
  std::lock_guard<std::mutex> lk(g_auto_mu);
  if (g_auto.size() >= 65536) g_auto.clear();  // bounded: a long-running caller starts over
  g_auto[A->crd] = AutoEntry{A->pos, A->rows, A->nnz, v};
  return v;
}

int spmv_run(const tacogb_csr* A, const void* x, void* y, int variant, cudaStream_t st) {
  TACOGB_CHECK_ARG(A != nullptr, "SpMV: null matrix");
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->nnz >= 0, "SpMV: negative size");
  TACOGB_CHECK_ARG(A->rows == 0 || y != nullptr, "SpMV: null y");
  TACOGB_CHECK_ARG(A->nnz == 0 || x != nullptr, "SpMV: null x");
  TACOGB_CHECK_ARG(A->nnz <= INT32_MAX, "SpMV: nnz exceeds int32 positions");
  TACOGB_CHECK_ARG(A->rows == 0 || A->pos != nullptr, "SpMV: null pos");
  TACOGB_CHECK_ARG(A->nnz == 0 || (A->crd != nullptr && A->vals != nullptr),
                   "SpMV: null crd/vals");
  if (variant < 0) variant = spmv_auto_variant(A, st);
  TACOGB_CHECK_ARG(variant < kNumSpmvVariants, "SpMV: variant %d out of range", variant);
  if (A->vtype == TACOGB_F64)
    return spmv_typed<double>(A, (const double*)x, (double*)y, variant, st);
  if (A->vtype == TACOGB_F32)
    return spmv_typed<float>(A, (const float*)x, (float*)y, variant, st);
  set_error(TACOGB_ERR_ARG, "SpMV: unsupported value type %d", A->vtype);
  return TACOGB_ERR_ARG;
}

// ------------------------------------------------------------ allocation-free SpMV --------
//
// Some callers cannot call cudaMalloc when they multiply: code that runs inside another
// framework's memory pool or allocator hooks (where a foreign allocation breaks its accounting),
// latency-critical or real-time paths (cudaMalloc and cudaFree can synchronise the device), and
// deployments that fix their GPU memory budget up front.  For them, tacogb_spmv_noalloc runs the
// merge-path SpMV with its temporary global memory (the tile partition and the tile carry-outs)
// in a file-scope device array of kNoAllocScratchBytes, reserved on every GPU that loads this
// library for as long as the process lives, instead of the library's grow-on-demand arena.

namespace {
constexpr size_t kNoAllocScratchBytes = (size_t)4 << 20;  // 4 MiB: ~2.9e8 merge items (rows + nnz)
}  // namespace

static __device__ __align__(256) unsigned char g_spmv_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_base[64];  // device address of g_spmv_noalloc_scratch, per device

// Device address of the static scratch on the current device.  In host code the array's name
// is only a host-side stand-in, so the address is looked up once per device, with that device
// current, and cached.
int noalloc_base(void** out) {
  int dev = 0;
  TACOGB_CUDA_TRY(cudaGetDevice(&dev));
  TACOGB_CHECK_ARG(dev >= 0 && dev < 64, "SpMV (no-alloc): device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_spmv_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error(TACOGB_ERR_CUDA, "SpMV (no-alloc): cudaGetSymbolAddress failed: %s",
                cudaGetErrorString(e));
      return TACOGB_ERR_CUDA;
    }
    g_noalloc_base[dev] = p;
  }
  *out = g_noalloc_base[dev];
  return 0;
}

constexpr int kNoAllocIpt = 11;
constexpr int64_t kNoAllocTileItems = (int64_t)kWmBlock * kNoAllocIpt;

// Bytes of scratch a call needs: tile partition, carry rows, carry values.
struct NoAllocLayout {
  int64_t tiles;
  size_t part_bytes, crow_bytes, need;
};

NoAllocLayout noalloc_layout(const tacogb_csr* A) {
  NoAllocLayout l;
  l.tiles = ((int64_t)A->rows + A->nnz + kNoAllocTileItems - 1) / kNoAllocTileItems;
  l.part_bytes = (((size_t)l.tiles + 1) * sizeof(int2) + 255) & ~(size_t)255;
  l.crow_bytes = ((size_t)l.tiles * sizeof(int32_t) + 255) & ~(size_t)255;
  l.need = l.part_bytes + l.crow_bytes + (size_t)l.tiles * sizeof(double);
  return l;
}

template <class P>
int launch_wmerge_noalloc(const tacogb_csr* A, const typename P::Val* x, typename P::Out* y,
                          const NoAllocLayout& l, cudaStream_t st) {
  using S = WmSmem<P, kNoAllocIpt>;
  static_assert(S::ITEMS == kNoAllocTileItems, "tile size");
  if (l.tiles == 0) return 0;
  void* base = nullptr;
  if (int rc = noalloc_base(&base)) return rc;
  const int32_t tiles = (int32_t)l.tiles;
  unsigned char* ws = (unsigned char*)base;
  int2* part = (int2*)ws;
  int32_t* crow = (int32_t*)(ws + l.part_bytes);
  double* cval = (double*)(ws + l.part_bytes + l.crow_bytes);
  // Every entry of part, crow and cval is written before it is read, so the contents left by
  // an earlier call need no clearing.
  const int64_t threads = rows4_threads((int64_t)A->rows + 1);
  count_launch();
  merge_partition_scatter<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
      A->pos, A->rows, A->nnz, make_divu32((uint32_t)kNoAllocTileItems), tiles, 0, part);
  if (int rc = launch_check("merge_partition_scatter")) return rc;
  auto kern = spmv_wmerge_kernel<P, kNoAllocIpt, false>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(S)));
  TACOGB_CUDA_TRY(set_gather_carveout((const void*)kern, -1));
  count_launch();
  kern<<<tiles, kWmBlock, sizeof(S), st>>>(A->pos, A->crd, (const typename P::Val*)A->vals,
                                          (const typename P::XG*)x, x, nullptr, y, part, A->rows,
                                          (int32_t)A->nnz, crow, cval, nullptr);
  if (int rc = launch_check("spmv_wmerge_kernel")) return rc;
  count_launch();
  spmv_carry_fixup<typename P::Out><<<(tiles + 255) / 256, 256, 0, st>>>(crow, cval, tiles, y,
                                                                          A->rows);
  return launch_check("spmv_carry_fixup");
}

}  // namespace

}  // namespace tacogb

extern "C" int tacogb_spmv_noalloc(const tacogb_csr* A, const void* x, void* y, void* stream) {
  using namespace tacogb;
  TACOGB_CHECK_ARG(A != nullptr, "SpMV (no-alloc): null matrix");
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->nnz >= 0, "SpMV (no-alloc): negative size");
  TACOGB_CHECK_ARG(A->nnz <= INT32_MAX, "SpMV (no-alloc): nnz exceeds int32 positions");
  const NoAllocLayout l = noalloc_layout(A);
  if (l.need > kNoAllocScratchBytes) {
    set_error(TACOGB_ERR_ARG,
              "SpMV (no-alloc): %lld rows + %lld nonzeros need %zu bytes of scratch but the "
              "static scratch holds %zu (about %lld rows + nonzeros at most); use tacogb_spmv",
              (long long)A->rows, (long long)A->nnz, l.need, kNoAllocScratchBytes,
              (long long)(kNoAllocScratchBytes / 20 * kNoAllocTileItems));
    return TACOGB_ERR_ARG;
  }
  TACOGB_CHECK_ARG(A->vtype == TACOGB_F64 || A->vtype == TACOGB_F32,
                   "SpMV (no-alloc): unsupported value type %d", A->vtype);
  TACOGB_CHECK_ARG(A->rows == 0 || (A->pos != nullptr && y != nullptr),
                   "SpMV (no-alloc): null pos or y");
  TACOGB_CHECK_ARG(A->nnz == 0 || (A->crd != nullptr && A->vals != nullptr && x != nullptr),
                   "SpMV (no-alloc): null crd, vals or x");
  const cudaStream_t st = (cudaStream_t)stream;
  if (A->vtype == TACOGB_F64)
    return launch_wmerge_noalloc<PolDF64X>(A, (const double*)x, (double*)y, l, st);
  return launch_wmerge_noalloc<PolComp32>(A, (const float*)x, (float*)y, l, st);
}
