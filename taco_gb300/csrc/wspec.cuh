// Warp-specialised persistent merge tiles for CSR SpMV.
//
// The warp tiles of wtile.cuh each stage their own tile and then wait for it: every tile pays
// one DRAM round trip of latency before its gathers start, and while a warp waits it has
// neither copies nor gathers in flight.  Here one producer warp per CTA runs ahead through a
// ring of S shared-memory stages, issuing the bulk copies (crd, values, row ends) of the CTA's
// next tiles as soon as a stage is released, and C consumer warps take the filled stages in
// turn: search, walk with x gathers, release the stage, join the lanes, store the rows.  The
// CTA's tiles are t = blockIdx.x + k * gridDim.x (k = 0, 1, ...); tile k sits in stage k mod S
// and is walked by consumer k mod C.
//
// Synchronisation is per stage: a `full` mbarrier (the producer's arrival plus the copies'
// bytes) and an `empty` mbarrier (the consumer's arrival once it no longer reads the stage).
// Every wait is bounded (mbar_wait_or_flag): on timeout the warp records TACOGB_DEV_TIMEOUT and
// leaves its loop, and the producer, before it exits, waits (bounded) for the copies it issued,
// so no copy writes the shared memory of an exited CTA.
#pragma once

#include "wtile.cuh"

namespace tacogb {

// One stage: a tile's staged arrays and its coordinates.
template <class P, int IPT>
struct alignas(16) WsStage {
  using Val = typename P::Val;
  static constexpr int ITEMS = 32 * IPT;
  static constexpr int VPAD = 16 / sizeof(Val);
  alignas(16) int32_t crd[ITEMS + 8];
  alignas(16) Val val[ITEMS + 2 * VPAD];
  alignas(16) int32_t re[ITEMS + 8];
  int4 tile;  // r0, rn, k0, kn
  int4 off;   // offsets of the first crd, value and row end inside the stage; tile index
};

template <class P, int IPT, int S>
struct alignas(16) WsSmem {
  WsStage<P, IPT> st[S];
  uint64_t full[S];
  uint64_t empty[S];
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Producer: fills stage s with tile (r0, rn, k0, kn).  Lanes load the few entries past the
// last 16-byte boundary of an array (only the tiles at the arrays' ends have any); lane 0 then
// arrives once, announcing the bytes, and issues the bulk copies of the aligned spans (rounded
// outwards).  One arrival per tile: 32 lanes arriving on one mbarrier serialise.
template <class P, int IPT>
__device__ __forceinline__ void ws_fill(WsStage<P, IPT>& g, uint64_t* full,
                                        const int32_t* __restrict__ pos,
                                        const int32_t* __restrict__ crd,
                                        const typename P::Val* __restrict__ vals, int32_t n,
                                        int32_t nnz, int r0, int rn, int k0, int kn, int t) {
  using Val = typename P::Val;
  constexpr int VP = WsStage<P, IPT>::VPAD;
  const int lane = threadIdx.x & 31;
  const int k1 = k0 + kn;
  const int q0 = r0 + 1, q1 = r0 + 1 + rn;
  const int a = k0 & ~3, b = max(a, min((k1 + 3) & ~3, nnz & ~3));
  const int av = k0 & ~(VP - 1), bv = max(av, min((k1 + VP - 1) & ~(VP - 1), nnz & ~(VP - 1)));
  const int ar = q0 & ~3, br = max(ar, min((q1 + 3) & ~3, (n + 1) & ~3));
  const bool tail = b < k1 || bv < k1 || br < q1;  // warp-uniform
  if (tail) {
    for (int i = max(b, k0) + lane; i < k1; i += 32) g.crd[i - a] = crd[i];
    for (int i = max(bv, k0) + lane; i < k1; i += 32) g.val[i - av] = vals[i];
    for (int i = max(br, q0) + lane; i < q1; i += 32) g.re[i - ar] = __ldg(pos + i);
    __syncwarp();  // the lanes' stores precede lane 0's arrival
  }
  if (lane == 0) {
    g.tile = make_int4(r0, rn, k0, kn);
    g.off = make_int4(k0 - a, k0 - av, q0 - ar, t);
    if (tail) __threadfence_block();
    // the consumer's reads of this stage's previous tile are ordered before these copies by
    // the empty barrier (its release arrival, this warp's acquiring wait), as in a TMA load
    // pipeline; no proxy fence is needed for a write-after-read through the barrier
    mbar_arrive_expect_tx(full, (uint32_t)((b - a) * 4 + (bv - av) * (int)sizeof(Val) +
                                           (br - ar) * 4));
    if (b > a) tma_load_bulk(g.crd, crd + a, (uint32_t)(b - a) * 4, full);
    if (bv > av) tma_load_bulk(g.val, vals + av, (uint32_t)(bv - av) * sizeof(Val), full);
    if (br > ar) tma_load_bulk(g.re, pos + ar, (uint32_t)(br - ar) * 4, full);
  }
}

// Consumer: one staged tile with policy P (native redo for checked policies).  The stage is
// released (empty barrier) as soon as no lane reads it any more; rows go straight to y; returns
// the FP64 carry-out (every lane) and, in end_row, the row it belongs to.
template <class P, int IPT, int CH>
__device__ __forceinline__ double ws_consume(const WsStage<P, IPT>& g, uint64_t* empty,
                                             const typename P::XG* __restrict__ xg,
                                             const typename P::Val* __restrict__ x64,
                                             const int* __restrict__ xflag,
                                             typename P::Out* __restrict__ y, int& end_row) {
  const int lane = threadIdx.x & 31;
  const int4 tl = g.tile, of = g.off;
  const int r0 = tl.x, rn = tl.y, k0 = tl.z, kn = tl.w;
  end_row = r0 + rn;
  const int32_t* scrd = g.crd + of.x;
  const typename P::Val* sval = g.val + of.y;
  const int32_t* sre = g.re + of.z;
  int row, ks;
  tile_search(sre, rn, kn, k0, min(lane * IPT, rn + kn), row, ks);
  int row_e = __shfl_down_sync(0xffffffffu, row, 1), ke = __shfl_down_sync(0xffffffffu, ks, 1);
  if (lane == 31) {
    row_e = rn;
    ke = kn;
  }
  const SinkDirect<typename P::Out> sink{y + r0};
  auto release = [&] {
    __syncwarp();
    if (lane == 0) mbar_arrive(empty);
  };
  if constexpr (P::kChecked) {
    typename P::Acc open, first;
    int first_row;
    bool ok = (xflag == nullptr || *xflag == 0);
    if (__all_sync(0xffffffffu, ok))
      ok = wt_walk<P, IPT, CH>(scrd, sval, sre, xg, row, ks, row_e, ke, k0, sink, open, first,
                               first_row);
    if (__all_sync(0xffffffffu, ok)) {
      release();
      return P::to_double(wt_join<P>(open, row_e, first, first_row, sink));
    }
    // a value outside the double-float range: the whole tile again in native FP64 (rows the
    // first pass stored are stored again)
    typename PolNative64::Acc nopen, nfirst;
    wt_walk<PolNative64, IPT, CH>(scrd, (const double*)sval, sre, (const double*)x64, row, ks,
                                  row_e, ke, k0, sink, nopen, nfirst, first_row);
    release();
    return wt_join<PolNative64>(nopen, row_e, nfirst, first_row, sink);
  } else {
    typename P::Acc open, first;
    int first_row;
    wt_walk<P, IPT, CH>(scrd, sval, sre, xg, row, ks, row_e, ke, k0, sink, open, first,
                        first_row);
    release();
    return P::to_double(wt_join<P>(open, row_e, first, first_row, sink));
  }
}

// The persistent kernel: warp 0 produces, warps 1..C consume.  One carry per tile goes to the
// fix-up kernel, as for the warp tiles.
template <class P, int IPT, int C, int S, int CH>
__global__ void __launch_bounds__((C + 1) * 32)
spmv_wspec_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                  const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
                  const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
                  typename P::Out* __restrict__ y, const int2* __restrict__ part, int32_t n,
                  int32_t nnz, int32_t tiles, int32_t* __restrict__ carry_row,
                  double* __restrict__ carry_val, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WsSmem<P, IPT, S>& sm = *reinterpret_cast<WsSmem<P, IPT, S>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < S) {
    mbar_init(&sm.full[threadIdx.x], 1);
    mbar_init(&sm.empty[threadIdx.x], 1);
  }
  __syncthreads();
  const int G = gridDim.x;
  // tiles of this CTA: t_k = blockIdx.x + k * G
  const int my_tiles = tiles > (int)blockIdx.x ? (tiles - 1 - (int)blockIdx.x) / G + 1 : 0;
  if (warp == 0) {
    int issued = 0;
    bool alive = true;
    for (int k = 0; k < my_tiles && alive; k += 32) {
      // the coordinates of the next 32 tiles, one per lane (two L2 loads in flight per lane)
      const int kk = k + lane;
      const int t = (int)blockIdx.x + kk * G;
      int2 c0 = make_int2(0, 0), c1 = make_int2(0, 0);
      if (kk < my_tiles) {
        c0 = part[t];
        c1 = part[t + 1];
      }
      const int m = min(32, my_tiles - k);
      for (int j = 0; j < m; j++) {
        const int kj = k + j;
        const int s = kj % S;
        if (kj >= S && !mbar_wait_or_flag(&sm.empty[s], (uint32_t)(((kj / S) - 1) & 1), status)) {
          alive = false;
          break;
        }
        const int r0 = __shfl_sync(0xffffffffu, c0.x, j), k0 = __shfl_sync(0xffffffffu, c0.y, j);
        const int r1 = __shfl_sync(0xffffffffu, c1.x, j), k1 = __shfl_sync(0xffffffffu, c1.y, j);
        ws_fill<P, IPT>(sm.st[s], &sm.full[s], pos, crd, vals, n, nnz, r0, r1 - r0, k0, k1 - k0,
                        (int)blockIdx.x + kj * G);
        issued = kj + 1;
      }
    }
    // every copy this warp issued has landed before the CTA may exit (bounded)
    for (int kj = max(0, issued - S); kj < issued; kj++)
      mbar_wait_bounded(&sm.full[kj % S], (uint32_t)((kj / S) & 1));
    return;
  }
  const int c = warp - 1;
  for (int k = c; k < my_tiles; k += C) {
    const int s = k % S;
    if (!mbar_wait_or_flag(&sm.full[s], (uint32_t)((k / S) & 1), status)) break;
    int end_row;
    const double carry =
        ws_consume<P, IPT, CH>(sm.st[s], &sm.empty[s], xg, x64, xflag, y, end_row);
    if (lane == 0) {
      const int t = (int)blockIdx.x + k * G;
      carry_row[t] = end_row;
      carry_val[t] = carry;
    }
  }
}

}  // namespace tacogb
