// Warp-level merge tiles for CSR SpMV.
//
// The merge path over (row ends, nonzeros) is cut into tiles of 32 * IPT items, one per warp.
// A warp stages its tile's crd, vals and row ends in its own shared-memory region with bulk
// copies completing on its own mbarrier, finds each lane's start on the merge path by binary
// search over the staged row ends, walks IPT items per lane, joins the lanes' open rows with a
// segmented shuffle scan, and writes the rows that end in the tile with one coalesced pass.
// Warps never wait for one another (no CTA barrier, no cross-warp join), so one warp's
// staging and search overlap other warps' gathers.  The row still open at the end of a tile is
// returned as a carry-out and added by the fix-up kernel, in tile order (deterministic).
#pragma once

#include "wmerge.cuh"

namespace tacogb {

constexpr int kWtWarps = 4;  // warps (tiles) per CTA

template <class P, int IPT>
struct alignas(16) WtSmem {
  using Val = typename P::Val;
  static constexpr int ITEMS = 32 * IPT;
  static constexpr int VPAD = 16 / sizeof(Val);
  alignas(16) int32_t crd[ITEMS + 8];
  alignas(16) Val val[ITEMS + 2 * VPAD];
  alignas(16) int32_t re[ITEMS + 8];  // global nonzero index of each row end (pos entries)
  alignas(16) double y[ITEMS];        // row results (policy accumulator, 8 bytes)
  uint64_t bar;
};

// The same staging area without the row-result array, for tiles whose rows go straight to y
// (3.7 KB per warp at IPT 7 instead of 5.5 KB, so more warps fit on an SM).
template <class P, int IPT>
struct alignas(16) WdSmem {
  using Val = typename P::Val;
  static constexpr int ITEMS = 32 * IPT;
  static constexpr int VPAD = 16 / sizeof(Val);
  alignas(16) int32_t crd[ITEMS + 8];
  alignas(16) Val val[ITEMS + 2 * VPAD];
  alignas(16) int32_t re[ITEMS + 8];
  uint64_t bar;
};

// Where a warp tile puts the sums of the rows that end in it: staged in shared memory (written
// to y by one coalesced pass after the join) or stored straight to y (y + the tile's first row).
struct SinkSmem {
  double* ys;
  template <class P>
  __device__ __forceinline__ void put(int r, typename P::Acc v) const {
    as_acc<typename P::Acc>(ys[r]) = v;
  }
};
template <class Out>
struct SinkDirect {
  Out* yg;
  template <class P>
  __device__ __forceinline__ void put(int r, typename P::Acc v) const {
    yg[r] = (Out)P::out(v);
  }
};

// Stages one warp tile: lane 0 issues bulk copies over the 16-byte-aligned spans of crd, vals
// and pos; every lane loads its share of the sub-16-byte tails; every lane then waits (bounded)
// on the warp's mbarrier.  Without TMA (unaligned bases) the lanes load everything.
template <bool TMA, class P, int IPT, class S>
__device__ __forceinline__ void wt_stage(S& s, const int32_t* __restrict__ pos,
                                         const int32_t* __restrict__ crd,
                                         const typename P::Val* __restrict__ vals, int32_t n,
                                         int32_t nnz, int r0, int rn, int k0, int kn, int* status,
                                         const int32_t*& scrd, const typename P::Val*& sval,
                                         const int32_t*& sre) {
  using Val = typename P::Val;
  constexpr int VP = S::VPAD;
  const int lane = threadIdx.x & 31;
  const int k1 = k0 + kn;
  const int q0 = r0 + 1, q1 = r0 + 1 + rn;  // pos indices of the row ends
  if constexpr (TMA) {
    const int a = k0 & ~3, b = max(a, min((k1 + 3) & ~3, nnz & ~3));
    const int av = k0 & ~(VP - 1), bv = max(av, min((k1 + VP - 1) & ~(VP - 1), nnz & ~(VP - 1)));
    const int ar = q0 & ~3, br = max(ar, min((q1 + 3) & ~3, (n + 1) & ~3));
    if (lane == 0) {
      mbar_init(&s.bar, 1);
      mbar_arrive_expect_tx(&s.bar, (uint32_t)((b - a) * 4 + (bv - av) * (int)sizeof(Val) +
                                               (br - ar) * 4));
      if (b > a) tma_load_bulk(s.crd, crd + a, (uint32_t)(b - a) * 4, &s.bar);
      if (bv > av) tma_load_bulk(s.val, vals + av, (uint32_t)(bv - av) * sizeof(Val), &s.bar);
      if (br > ar) tma_load_bulk(s.re, pos + ar, (uint32_t)(br - ar) * 4, &s.bar);
    }
    for (int i = max(b, k0) + lane; i < k1; i += 32) s.crd[i - a] = crd[i];
    for (int i = max(bv, k0) + lane; i < k1; i += 32) s.val[i - av] = vals[i];
    for (int i = max(br, q0) + lane; i < q1; i += 32) s.re[i - ar] = __ldg(pos + i);
    __syncwarp();  // lane 0's mbarrier initialisation and the tails precede every wait and read
    mbar_wait_or_flag(&s.bar, 0, status);
    scrd = s.crd + (k0 - a);
    sval = s.val + (k0 - av);
    sre = s.re + (q0 - ar);
  } else {
    for (int i = lane; i < kn; i += 32) {
      s.crd[i] = ld_stream_i32(crd + k0 + i);
      s.val[i] = vals[k0 + i];
    }
    for (int i = lane; i < rn; i += 32) s.re[i] = __ldg(pos + q0 + i);
    __syncwarp();
    scrd = s.crd;
    sval = s.val;
    sre = s.re;
  }
}

// Walks this lane's merge items [(row, ks), (row_e, ke)) over the staged tile with policy P,
// gathering x in chunks of CH independent loads.  Rows that end inside the lane's range go to
// the sink, except the first one (which may have begun in an earlier lane): its sum is
// returned in `first` (first_row = its tile-local index, -1 if none).  Returns the sum of the
// open row at the lane's end in `open`, and false when a checked policy met an out-of-range
// value.
template <class P, int IPT, int CH, class Sink>
__device__ __forceinline__ bool wt_walk(const int32_t* scrd, const typename P::Val* sval,
                                        const int32_t* sre, const typename P::XG* __restrict__ x,
                                        int row, int ks, int row_e, int ke, int k0,
                                        const Sink& sink, typename P::Acc& open,
                                        typename P::Acc& first, int& first_row) {
  using Acc = typename P::Acc;
  using Val = typename P::Val;
  using XG = typename P::XG;
  using Wk = typename P::W;
  const int cnt = ke - ks;
  const int base = k0 + ks;
  int next_end = row < row_e ? sre[row] - base : INT_MAX;  // lane-local index of the next end
  bool ok = true;
  typename Wk::State st = Wk::init();
  first = P::zero();
  first_row = -1;
  auto emit = [&](int r) {
    const Acc v = Wk::take(st);
    if (first_row < 0) {
      first_row = r;
      first = v;
    } else {
      sink.template put<P>(r, v);
    }
    row = r + 1;
    next_end = row < row_e ? sre[row] - base : INT_MAX;
  };
  static_assert(CH % 2 == 0, "item parity within a chunk must equal the parity of j");
#pragma unroll 1
  for (int c = 0; c < IPT; c += CH) {
    Val vv[CH];
    XG xv[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) {
      if (c + j < cnt) {
        vv[j] = sval[ks + c + j];
        xv[j] = ldg_xg(x + scrd[ks + c + j]);
      }
    }
#pragma unroll
    for (int j = 0; j < CH; j++) {
      if (c + j < IPT) {
        while (next_end <= c + j) emit(row);
        if (c + j < cnt)
          ok &= (j & 1) ? Wk::template step<1>(st, vv[j], xv[j])
                        : Wk::template step<0>(st, vv[j], xv[j]);
      }
    }
  }
  while (row < row_e) emit(row);
  open = Wk::take(st);
  return ok;
}

// Joins the lanes of one warp tile: segmented inclusive shuffle scan of the open-row sums keyed
// by the open row (non-decreasing along the lanes), then each lane adds the preceding lanes'
// part to its first ended row.  Returns (every lane) the sum of the row still open at the
// tile's end, which is lane 31's key.
template <class P, class Sink>
__device__ __forceinline__ typename P::Acc wt_join(typename P::Acc open, int key,
                                                   typename P::Acc first, int first_row,
                                                   const Sink& sink) {
  using Acc = typename P::Acc;
  const int lane = threadIdx.x & 31;
  Acc sc = open;
  // A step whose distance no run of equal keys spans is skipped, and so are the longer ones
  // (keys never decrease along the lanes): on GB300 an FP64 add costs the FP64 pipe the same
  // with one lane active as with 32, and short rows need one or two steps, not five.
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int ko = __shfl_up_sync(0xffffffffu, key, d);
    const bool need = lane >= d && ko == key;
    if (!__any_sync(0xffffffffu, need)) break;
    const Acc o = P::shfl_up(sc, d);
    if (need) sc = P::add(o, sc);
  }
  const Acc prev = P::shfl_up(sc, 1);
  const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
  if (first_row >= 0) {
    Acc tot = first;
    if (lane > 0 && kprev == first_row) tot = P::add(prev, first);
    sink.template put<P>(first_row, tot);
  }
  Acc out;
  if constexpr (sizeof(Acc) == 8 && std::is_same<Acc, double>::value) {
    out = __shfl_sync(0xffffffffu, sc, 31);
  } else {
    out = DF{__shfl_sync(0xffffffffu, sc.h, 31), __shfl_sync(0xffffffffu, sc.l, 31)};
  }
  return out;
}

// One warp tile with policy P (native redo for checked policies); writes the rows ending in the
// tile and returns the FP64 carry-out (every lane).  first_val (lane 0, when rn > 0) is the FP64
// value written for the tile's first row.
template <class P, int IPT, bool TMA, int CH, class S>
__device__ __forceinline__ double wt_process(
    S& s, const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
    const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
    const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
    typename P::Out* __restrict__ y, int32_t n, int32_t nnz, int r0, int rn, int k0, int kn,
    int* status, double& first_val) {
  const int lane = threadIdx.x & 31;
  const int32_t* scrd;
  const typename P::Val* sval;
  const int32_t* sre;
  // direct tiles (no y staging area) store their rows straight to y
  constexpr bool kDirect = std::is_same<S, WdSmem<P, IPT>>::value;
  wt_stage<TMA, P, IPT>(s, pos, crd, vals, n, nnz, r0, rn, k0, kn, status, scrd, sval, sre);
  // lane starts on the merge path; lane 31 ends at the tile end (rn, kn)
  int row, ks;
  tile_search(sre, rn, kn, k0, min(lane * IPT, rn + kn), row, ks);
  int row_e = __shfl_down_sync(0xffffffffu, row, 1), ke = __shfl_down_sync(0xffffffffu, ks, 1);
  if (lane == 31) {
    row_e = rn;
    ke = kn;
  }
  double carry;
  bool native = !P::kChecked;
  if constexpr (P::kChecked) {
    typename P::Acc open, first;
    int first_row;
    bool ok = (xflag == nullptr || *xflag == 0);
    if constexpr (kDirect) {
      const SinkDirect<typename P::Out> sink{y + r0};
      if (__all_sync(0xffffffffu, ok))
        ok = wt_walk<P, IPT, CH>(scrd, sval, sre, xg, row, ks, row_e, ke, k0, sink, open, first,
                                 first_row);
      if (__all_sync(0xffffffffu, ok)) {
        carry = P::to_double(wt_join<P>(open, row_e, first, first_row, sink));
      } else {
        native = true;
      }
    } else {
      const SinkSmem sink{s.y};
      if (__all_sync(0xffffffffu, ok))
        ok = wt_walk<P, IPT, CH>(scrd, sval, sre, xg, row, ks, row_e, ke, k0, sink, open, first,
                                 first_row);
      if (__all_sync(0xffffffffu, ok)) {
        const typename P::Acc c = wt_join<P>(open, row_e, first, first_row, sink);
        __syncwarp();
        for (int i = lane; i < rn; i += 32) y[r0 + i] = P::out(as_acc<typename P::Acc>(s.y[i]));
        if (lane == 0 && rn > 0) first_val = P::to_double(as_acc<typename P::Acc>(s.y[0]));
        carry = P::to_double(c);
      } else {
        native = true;
      }
    }
  }
  if (native) {
    using Q = typename std::conditional<P::kChecked, PolNative64, P>::type;
    typename Q::Acc open, first;
    int first_row;
    if constexpr (kDirect) {
      // rows a checked first pass stored are stored again here
      const SinkDirect<typename P::Out> sink{y + r0};
      wt_walk<Q, IPT, CH>(scrd, (const typename Q::Val*)sval, sre, (const typename Q::XG*)x64,
                          row, ks, row_e, ke, k0, sink, open, first, first_row);
      carry = Q::to_double(wt_join<Q>(open, row_e, first, first_row, sink));
    } else {
      const SinkSmem sink{s.y};
      wt_walk<Q, IPT, CH>(scrd, (const typename Q::Val*)sval, sre, (const typename Q::XG*)x64,
                          row, ks, row_e, ke, k0, sink, open, first, first_row);
      const typename Q::Acc c = wt_join<Q>(open, row_e, first, first_row, sink);
      __syncwarp();
      for (int i = lane; i < rn; i += 32)
        y[r0 + i] = (typename P::Out)Q::out(as_acc<typename Q::Acc>(s.y[i]));
      if (lane == 0 && rn > 0) first_val = Q::to_double(as_acc<typename Q::Acc>(s.y[0]));
      carry = Q::to_double(c);
    }
  }
  return carry;
}

}  // namespace tacogb

namespace tacogb {

// ------------------------------------------------------------------ persistent warp pipeline
//
// Each warp owns a contiguous run of tiles and keeps two staging buffers: the bulk copies of
// tile t+1 are in flight while the warp walks tile t, so the DRAM latency of staging leaves
// the critical path.  The row still open at the end of a tile is the first row of the next
// tile, so the warp chains it in a register (carry_in) and only the last one reaches the
// fix-up kernel.

template <class P, int IPT>
struct alignas(16) WpStage {
  using Val = typename P::Val;
  static constexpr int ITEMS = 32 * IPT;
  static constexpr int VPAD = 16 / sizeof(Val);
  alignas(16) int32_t crd[ITEMS + 8];
  alignas(16) Val val[ITEMS + 2 * VPAD];
  alignas(16) int32_t re[ITEMS + 8];
};

template <class P, int IPT>
struct alignas(16) WpSmem {
  WpStage<P, IPT> st[2];
  alignas(16) double y[32 * IPT];
  uint64_t bar[2];
};

// Issues the copies of tile (r0, rn, k0, kn) into stage g completing on bar (lane 0: bulk copies
// of the 16-byte-aligned spans; every lane: its share of the sub-16-byte tails).  Returns the
// offsets of the tile's first crd / value / row end inside the stage.
template <class P, int IPT>
__device__ __forceinline__ int3 wp_issue(WpStage<P, IPT>& g, uint64_t* bar,
                                         const int32_t* __restrict__ pos,
                                         const int32_t* __restrict__ crd,
                                         const typename P::Val* __restrict__ vals, int32_t n,
                                         int32_t nnz, int r0, int rn, int k0, int kn) {
  using Val = typename P::Val;
  constexpr int VP = WpStage<P, IPT>::VPAD;
  const int lane = threadIdx.x & 31;
  const int k1 = k0 + kn;
  const int q0 = r0 + 1, q1 = r0 + 1 + rn;
  const int a = k0 & ~3, b = max(a, min((k1 + 3) & ~3, nnz & ~3));
  const int av = k0 & ~(VP - 1), bv = max(av, min((k1 + VP - 1) & ~(VP - 1), nnz & ~(VP - 1)));
  const int ar = q0 & ~3, br = max(ar, min((q1 + 3) & ~3, (n + 1) & ~3));
  if (lane == 0) {
    // the lanes' earlier reads of this stage precede the asynchronous overwrite
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(bar, (uint32_t)((b - a) * 4 + (bv - av) * (int)sizeof(Val) +
                                          (br - ar) * 4));
    if (b > a) tma_load_bulk(g.crd, crd + a, (uint32_t)(b - a) * 4, bar);
    if (bv > av) tma_load_bulk(g.val, vals + av, (uint32_t)(bv - av) * sizeof(Val), bar);
    if (br > ar) tma_load_bulk(g.re, pos + ar, (uint32_t)(br - ar) * 4, bar);
  }
  for (int i = max(b, k0) + lane; i < k1; i += 32) g.crd[i - a] = crd[i];
  for (int i = max(bv, k0) + lane; i < k1; i += 32) g.val[i - av] = vals[i];
  for (int i = max(br, q0) + lane; i < q1; i += 32) g.re[i - ar] = __ldg(pos + i);
  return make_int3(k0 - a, k0 - av, q0 - ar);
}

}  // namespace tacogb
