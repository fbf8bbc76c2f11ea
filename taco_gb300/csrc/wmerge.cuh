// Merge-path tile machinery shared by the single-matrix SpMV kernels (spmv.cu) and the batched
// persistent launch (batched.cu): accumulation policies, the shared-memory tile layout, the
// bulk-copy staging of one tile, and the per-lane walk with its lane, warp and tile joins.
#pragma once

#include <climits>
#include <type_traits>

#include "common.cuh"
#include "df.cuh"

namespace tacogb {

// ------------------------------------------------------------------ policies -------------

// Accumulation policies.  Val is the stored value type; XG is the element type of the x array
// the kernel gathers from (pre-split double-float pairs for PolDF64).

// Walk state.  A lane's items go through step<J> (J = item parity, a compile-time constant
// after unrolling); take() returns the row's sum in the policy's accumulator type and resets.
// The default keeps kAcc interleaved accumulators of type Acc, which shortens the dependency
// chain of each one.
template <class P, class AccT, int NA>
struct InterleavedWalk {
  struct State {
    AccT a[NA];
  };
  __device__ static State init() {
    State s;
#pragma unroll
    for (int i = 0; i < NA; i++) s.a[i] = P::zero();
    return s;
  }
  template <int J>
  __device__ static bool step(State& s, typename P::Val a, typename P::XG x) {
    return P::madd(s.a[J % NA], a, x);
  }
  __device__ static AccT take(State& s) {
    AccT v = s.a[0];
    s.a[0] = P::zero();
#pragma unroll
    for (int i = 1; i < NA; i++) {
      v = P::add(v, s.a[i]);
      s.a[i] = P::zero();
    }
    return v;
  }
};

// FP64 values, FP64 accumulation (DFMA).
struct PolNative64 {
  using Val = double;
  using Out = double;
  using Acc = double;
  using XG = double;
  static constexpr bool kChecked = false;
  static constexpr int kAcc = 1;  // joining accumulators at a row end would cost an FP64 add
  __device__ static Acc zero() { return 0.0; }
  __device__ static bool madd(Acc& acc, Val a, XG x) {
    acc = __fma_rn(a, x, acc);
    return true;
  }
  __device__ static Acc add(Acc a, Acc b) { return __dadd_rn(a, b); }
  __device__ static Acc shfl_up(Acc a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
  __device__ static Acc shfl_xor(Acc a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
  __device__ static Out out(Acc a) { return a; }
  __device__ static double to_double(Acc a) { return a; }
  using W = InterleavedWalk<PolNative64, Acc, kAcc>;
};

// FP64 values evaluated in double-float on the FP32 pipe; x arrives pre-split (DF per entry).
struct PolDF64 {
  using Val = double;
  using Out = double;
  using Acc = DF;
  using XG = DF;
  static constexpr bool kChecked = true;
  static constexpr int kAcc = 2;  // interleaved accumulators halve the TwoSum dependency chain
  __device__ static Acc zero() { return DF{0.f, 0.f}; }
  __device__ static bool madd(Acc& acc, Val a, XG x) {
    float ah, al;
    const bool ok = split_df(a, ah, al);
    acc = df_add(acc, df_mul(ah, al, x.h, x.l));
    return ok;
  }
  __device__ static Acc add(Acc a, Acc b) { return df_add(a, b); }
  __device__ static Acc shfl_up(Acc a, int d) {
    return DF{__shfl_up_sync(0xffffffffu, a.h, d), __shfl_up_sync(0xffffffffu, a.l, d)};
  }
  __device__ static Acc shfl_xor(Acc a, int m) {
    return DF{__shfl_xor_sync(0xffffffffu, a.h, m), __shfl_xor_sync(0xffffffffu, a.l, m)};
  }
  __device__ static Out out(Acc a) { return df_to_double(a); }
  __device__ static double to_double(Acc a) { return df_to_double(a); }
  using W = InterleavedWalk<PolDF64, Acc, kAcc>;
};

// FP32 values, TwoProduct/TwoSum-compensated FP32 accumulation.
struct PolComp32 {
  using Val = float;
  using Out = float;
  using Acc = DF;
  using XG = float;
  static constexpr bool kChecked = false;
  static constexpr int kAcc = 2;
  __device__ static Acc zero() { return DF{0.f, 0.f}; }
  __device__ static bool madd(Acc& acc, Val a, XG x) {
    DF p;
    p.h = __fmul_rn(a, x);
    p.l = __fmaf_rn(a, x, -p.h);
    acc = df_add(acc, p);
    return true;
  }
  __device__ static Acc add(Acc a, Acc b) { return df_add(a, b); }
  __device__ static Acc shfl_up(Acc a, int d) {
    return DF{__shfl_up_sync(0xffffffffu, a.h, d), __shfl_up_sync(0xffffffffu, a.l, d)};
  }
  __device__ static Acc shfl_xor(Acc a, int m) {
    return DF{__shfl_xor_sync(0xffffffffu, a.h, m), __shfl_xor_sync(0xffffffffu, a.l, m)};
  }
  __device__ static Out out(Acc a) { return __fadd_rn(a.h, a.l); }
  __device__ static double to_double(Acc a) { return (double)a.h + (double)a.l; }
  using W = InterleavedWalk<PolComp32, Acc, kAcc>;
};

// Double-float policy that gathers the FP64 x and splits each gathered entry while staging
// (no pre-split buffer; more integer work per nonzero).
struct PolDF64X : PolDF64 {
  using XG = double;
  __device__ static bool madd(Acc& acc, Val a, XG x) {
    float ah, al, xh, xl;
    const bool ok = split_df(a, ah, al) & split_df(x, xh, xl);
    acc = df_add(acc, df_mul(ah, al, xh, xl));
    return ok;
  }
  using W = InterleavedWalk<PolDF64X, Acc, kAcc>;
};

// PolDF64X with four interleaved accumulators (shorter TwoSum chains, one more join per row).
struct PolDF64X4 : PolDF64X {
  static constexpr int kAcc = 4;
  using W = InterleavedWalk<PolDF64X, Acc, kAcc>;
};

// FP64 values, both pipes at once: even items of a lane accumulate with DFMA on the FP64 pipe,
// odd items in double-float on the FP32 pipe (x split on the fly); a row's two partial sums
// join in FP64 at the row end, and the lane/warp/tile joins run in FP64.  Error is bounded by
// the double-float half (about 2^-46 per product).
struct PolHybrid {
  using Val = double;
  using Out = double;
  using Acc = double;
  using XG = double;
  static constexpr bool kChecked = true;
  __device__ static Acc zero() { return 0.0; }
  __device__ static Acc add(Acc a, Acc b) { return __dadd_rn(a, b); }
  __device__ static Acc shfl_up(Acc a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
  __device__ static Acc shfl_xor(Acc a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
  __device__ static Out out(Acc a) { return a; }
  __device__ static double to_double(Acc a) { return a; }
  __device__ static bool madd(Acc& acc, Val a, XG x) {  // used by the vector family only
    acc = __fma_rn(a, x, acc);
    return true;
  }
  struct W {
    struct State {
      double n;
      DF d;
    };
    __device__ static State init() { return State{0.0, DF{0.f, 0.f}}; }
    template <int J>
    __device__ static bool step(State& s, double a, double x) {
      if (J == 0) {
        s.n = __fma_rn(a, x, s.n);
        return true;
      }
      float ah, al, xh, xl;
      const bool ok = split_df(a, ah, al) & split_df(x, xh, xl);
      s.d = df_add(s.d, df_mul(ah, al, xh, xl));
      return ok;
    }
    __device__ static double take(State& s) {
      const double v = __dadd_rn(s.n, df_to_double(s.d));
      s.n = 0.0;
      s.d = DF{0.f, 0.f};
      return v;
    }
  };
};

// FP64 values in double-float with the fewest FP32-pipe instructions per nonzero (about 22):
// x arrives pre-split; each value is split by split_df_fast and range-checked from its high
// word; the walk keeps a running hi sum s and an unnormalised compensation c, so each product
// costs one exact TwoProduct of the hi parts, two cross-term FMAs into c and one TwoSum into
// s, and the renormalisation to a double-float pair happens once per row end.  |c| stays near
// 2^-24 of the partial sums it collects, so the row error stays about 2^-46 of sum |a x|.
struct PolDFS : PolDF64 {
  struct W {
    struct State {
      float s, c;
    };
    __device__ static State init() { return State{0.f, 0.f}; }
    template <int J>
    __device__ static bool step(State& st, double a, DF x) {
      float ah, al;
      split_df_fast(a, ah, al);
      const float ph = __fmul_rn(ah, x.h);
      const float pe = __fmaf_rn(ah, x.h, -ph);
      float c = __fmaf_rn(ah, x.l, st.c);
      c = __fmaf_rn(al, x.h, c);
      float s1, e;
      two_sum(st.s, ph, s1, e);
      st.c = __fadd_rn(c, __fadd_rn(pe, e));
      st.s = s1;
      return df_in_range(a);
    }
    __device__ static DF take(State& st) {
      DF r;
      float e;
      two_sum(st.s, st.c, r.h, e);
      r.l = e;
      st.s = 0.f;
      st.c = 0.f;
      return r;
    }
  };
};

// Tag policy selecting the product-staged tile (gp_process_tile) for FP64 values.
struct PolGP : PolDFS {};

// ------------------------------------------------------------------ wmerge ----------------

// 128-thread CTAs with a small shared-memory footprint, so that many tiles are in flight per
// SM and the hardware overlaps one tile's staging with another's arithmetic.  IPT is odd: a
// lane's items start about IPT elements after its neighbour's, and an odd stride spreads the
// lanes' shared-memory reads over all banks.
constexpr int kWmBlock = 128;
constexpr int kWmWarps = kWmBlock / 32;

template <class P, int IPT>
struct WmSmem {
  using Val = typename P::Val;
  static constexpr int ITEMS = kWmBlock * IPT;
  static constexpr int VPAD = 16 / sizeof(Val);  // values per 16 bytes
  // Staged arrays keep room for the 16-byte alignment slack of the bulk copies.
  alignas(16) int32_t crd[ITEMS + 8];
  alignas(16) Val val[ITEMS + 2 * VPAD];
  alignas(16) int32_t re[ITEMS + 8];  // global nonzero index of each row end (pos entries)
  double y[ITEMS];                    // row results (policy accumulator, 8 bytes)
  int2 lane_start[kWmBlock + 1];      // merge coordinate where each lane's walk starts
  int32_t wkey[kWmWarps];
  double wval[kWmWarps];  // warp carries (policy accumulator)
  uint64_t bar;
};

// Stages a tile's crd[k0,k1), vals[k0,k1) and row ends pos[r0+1, r0+1+rn) in shared memory.
// With TMA, one thread issues three bulk copies over the 16-byte-aligned spans inside the
// arrays and every thread waits on the mbarrier (bounded); the sub-16-byte tails at the array
// ends are loaded by plain loads.  Without TMA (unaligned base pointers), each thread issues
// its IPT loads before storing any of them.  Sets the shared-memory base pointers for
// tile-local indices.
template <bool TMA, class P, int IPT>
__device__ __forceinline__ void wm_stage(WmSmem<P, IPT>& s, const int32_t* __restrict__ pos,
                                         const int32_t* __restrict__ crd,
                                         const typename P::Val* __restrict__ vals, int32_t n,
                                         int32_t nnz, int r0, int rn, int k0, int kn,
                                         int* status, int32_t*& scrd, typename P::Val*& sval,
                                         const int32_t*& sre) {
  using Val = typename P::Val;
  using S = WmSmem<P, IPT>;
  const int tid = threadIdx.x;
  const int k1 = k0 + kn;
  if constexpr (TMA) {
    constexpr int VP = S::VPAD;
    const int a = k0 & ~3, b = max(a, min((k1 + 3) & ~3, nnz & ~3));
    const int av = k0 & ~(VP - 1), bv = max(av, min((k1 + VP - 1) & ~(VP - 1), nnz & ~(VP - 1)));
    const int q0 = r0 + 1, q1 = r0 + 1 + rn;  // pos indices of the row ends
    const int ar = q0 & ~3, br = max(ar, min((q1 + 3) & ~3, (n + 1) & ~3));
    if (tid == 0) mbar_init(&s.bar, 1);
    __syncthreads();
    if (tid == 0) {
      // a persistent caller reuses this memory: earlier generic-proxy reads precede the copies
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive_expect_tx(&s.bar, (uint32_t)((b - a) * 4 + (bv - av) * (int)sizeof(Val) +
                                               (br - ar) * 4));
      if (b > a) tma_load_bulk(s.crd, crd + a, (uint32_t)(b - a) * 4, &s.bar);
      if (bv > av) tma_load_bulk(s.val, vals + av, (uint32_t)(bv - av) * sizeof(Val), &s.bar);
      if (br > ar) tma_load_bulk(s.re, pos + ar, (uint32_t)(br - ar) * 4, &s.bar);
    }
    for (int i = max(b, k0) + tid; i < k1; i += kWmBlock) s.crd[i - a] = crd[i];
    for (int i = max(bv, k0) + tid; i < k1; i += kWmBlock) s.val[i - av] = vals[i];
    for (int i = max(br, q0) + tid; i < q1; i += kWmBlock) s.re[i - ar] = __ldg(pos + i);
    mbar_wait_or_flag(&s.bar, 0, status);
    scrd = s.crd + (k0 - a);
    sval = s.val + (k0 - av);
    sre = s.re + (q0 - ar);
  } else {
    int32_t cc[IPT];
    Val vv[IPT];
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      const int i = tid + j * kWmBlock;
      if (i < kn) {
        cc[j] = ld_stream_i32(crd + k0 + i);
        vv[j] = vals[k0 + i];
      }
    }
#pragma unroll
    for (int j = 0; j < IPT; j++) {
      const int i = tid + j * kWmBlock;
      if (i < kn) {
        s.crd[i] = cc[j];
        s.val[i] = vv[j];
      }
    }
    for (int i = tid; i < rn; i += kWmBlock) s.re[i] = __ldg(pos + r0 + 1 + i);
    scrd = s.crd;
    sval = s.val;
    sre = s.re;
  }
  __syncthreads();
  if constexpr (TMA) {
    if (tid == 0) mbar_inval(&s.bar);  // every thread is past its wait
  }
}

template <typename T>
__device__ __forceinline__ T ldg_xg(const T* p);
// Gathers of x use ld.global.cg: on GB300 random 8-byte gathers through it run at up to ~0.88
// per clock per SM against ~0.79 for ld.global.nc (measured with a 60 KB L1).
template <>
__device__ __forceinline__ double ldg_xg<double>(const double* p) {
  double v;
  asm("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
template <>
__device__ __forceinline__ float ldg_xg<float>(const float* p) {
  float v;
  asm("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
template <>
__device__ __forceinline__ DF ldg_xg<DF>(const DF* p) {
  DF v;
  asm("ld.global.cg.v2.f32 {%0, %1}, [%2];" : "=f"(v.h), "=f"(v.l) : "l"(p));
  return v;
}

// Tile-local merge coordinate of diagonal d (rows ended, nonzeros consumed).
__device__ __forceinline__ void tile_search(const int32_t* s_re, int rn, int kn, int k0, int d,
                                            int& row, int& k) {
  int lo = max(d - kn, 0), hi = min(d, rn);
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (s_re[mid] <= k0 + d - mid - 1) lo = mid + 1; else hi = mid;
  }
  row = lo;
  k = d - lo;
}

template <class A>
__device__ __forceinline__ A& as_acc(double& slot) {
  static_assert(sizeof(A) == sizeof(double), "accumulator must be 8 bytes");
  return *reinterpret_cast<A*>(&slot);
}

template <class P, class S>
__device__ __forceinline__ void wm_join(S& s, typename P::Acc accv, int key, typename P::Acc first,
                                        int first_row, int rn, typename P::Acc& carry);

// Walks this lane's IPT merge items over the staged tile with policy P, gathering x in chunks
// of CH independent loads inside the walk (other warps' arithmetic hides their latency), joins
// lanes and warps, and leaves every row result of the tile in s.y; the part of the row still
// open at the tile end is returned in `carry` (thread 0).  Returns false when a checked policy
// met a value it cannot represent.
template <class P, int IPT, class S, int CH = 4>
__device__ __forceinline__ bool wm_tile(S& s, const int32_t* scrd, const typename P::Val* sval,
                                        const int32_t* sre, const typename P::XG* __restrict__ x,
                                        int rn, int kn, int k0, typename P::Acc& carry) {
  using Acc = typename P::Acc;
  using Val = typename P::Val;
  using XG = typename P::XG;
  const int tid = threadIdx.x;
  const int items = rn + kn;
  // One merge-path search per thread: a lane's walk ends where the next lane's begins.
  int row, ks;
  tile_search(sre, rn, kn, k0, min(tid * IPT, items), row, ks);
  s.lane_start[tid] = make_int2(row, ks);
  if (tid == 0) {
    int r, k;
    tile_search(sre, rn, kn, k0, min(kWmBlock * IPT, items), r, k);
    s.lane_start[kWmBlock] = make_int2(r, k);
  }
  __syncthreads();
  const int row_e = s.lane_start[tid + 1].x, ke = s.lane_start[tid + 1].y;
  const int cnt = ke - ks;
  // global nonzero index of the next row end (kept in a register; reloaded only at row ends)
  int next_end = row < row_e ? sre[row] : INT_MAX;

  bool ok = true;
  using Wk = typename P::W;
  typename Wk::State st = Wk::init();
  Acc first = P::zero();
  int first_row = -1;
  auto emit = [&](int r) {
    const Acc v = Wk::take(st);
    if (first_row < 0) {
      first_row = r;
      first = v;
    } else {
      as_acc<Acc>(s.y[r]) = v;
    }
    row = r + 1;
    next_end = row < row_e ? sre[row] : INT_MAX;
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
        while (next_end <= k0 + ks + c + j) emit(row);
        if (c + j < cnt)
          ok &= (j & 1) ? Wk::template step<1>(st, vv[j], xv[j])
                        : Wk::template step<0>(st, vv[j], xv[j]);
      }
    }
  }
  while (row < row_e) emit(row);
  wm_join<P>(s, Wk::take(st), row_e, first, first_row, rn, carry);
  return ok;
}

// Joins the lanes' open rows: `accv` is this lane's sum for row `key` (its last, still open
// row), `first` its sum for `first_row` (the first row it ended, -1 if none), which may have
// begun in earlier lanes.  Leaves every row result of the tile in s.y and the part of the row
// still open at the tile end in `carry` (thread 0).
template <class P, class S>
__device__ __forceinline__ void wm_join(S& s, typename P::Acc accv, int key, typename P::Acc first,
                                        int first_row, int rn, typename P::Acc& carry) {
  using Acc = typename P::Acc;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // Segmented inclusive scan of lane carries keyed by the open row (keys are non-decreasing
  // along the lanes, so equal keys are contiguous).
  Acc sc = accv;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const Acc o = P::shfl_up(sc, d);
    const int ko = __shfl_up_sync(0xffffffffu, key, d);
    if (lane >= d && ko == key) sc = P::add(o, sc);
  }
  const Acc prev = P::shfl_up(sc, 1);
  const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
  if (first_row >= 0) {
    Acc tot = first;
    if (lane > 0 && kprev == first_row) tot = P::add(prev, first);
    as_acc<Acc>(s.y[first_row]) = tot;
  }
  if (lane == 31) {
    s.wkey[warp] = key;
    as_acc<Acc>(s.wval[warp]) = sc;
  }
  __syncthreads();
  // Warps in order: a run of equal open-row keys adds into the row where it ends (a later
  // warp's first row) or, for the final run, becomes the tile carry-out.
  if (tid == 0) {
    int rk = s.wkey[0];
    Acc rv = as_acc<Acc>(s.wval[0]);
    for (int w = 1; w <= kWmWarps; w++) {
      if (w < kWmWarps && s.wkey[w] == rk) {
        rv = P::add(rv, as_acc<Acc>(s.wval[w]));
        continue;
      }
      if (rk < rn) as_acc<Acc>(s.y[rk]) = P::add(rv, as_acc<Acc>(s.y[rk]));
      else carry = rv;
      if (w < kWmWarps) {
        rk = s.wkey[w];
        rv = as_acc<Acc>(s.wval[w]);
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ product-staged tile ---
//
// The same merge tile in two phases.  Phase 1 takes the tile's nonzeros in order, thread tid
// owning items tid, tid + 128, ...: it reads the staged columns (consecutive, so free of bank
// conflicts), issues all of its IPT gathers of x at once (no dependence between them, so they
// overlap one another and the merge-path search that follows), then forms each product as a
// double-float pair and stores it over the staged value.  Phase 2 is the merge walk, which now
// reads products from shared memory only and sums them with TwoSum: no global load waits
// inside the walk.  FP64 values only (a product pair fills a value's 8-byte slot).

// Product of one FP64 value with a pre-split x entry as an unevaluated pair; false when the
// value lies outside the double-float range.
__device__ __forceinline__ bool gp_product(double a, DF x, DF& p) {
  float ah, al;
  split_df_fast(a, ah, al);
  p.h = __fmul_rn(ah, x.h);
  const float pe = __fmaf_rn(ah, x.h, -p.h);
  p.l = __fmaf_rn(ah, x.l, __fmaf_rn(al, x.h, pe));
  return df_in_range(a);
}

// Phase 1 (see above).  Also runs the lanes' merge-path search between the gathers and their
// use.  Returns false (every thread) when some value of the tile is out of range.
template <int IPT, class S>
__device__ __forceinline__ bool gp_products(S& s, const int32_t* scrd, double* sval,
                                            const int32_t* sre, const DF* __restrict__ x, int rn,
                                            int kn, int k0) {
  const int tid = threadIdx.x;
  DF xv[IPT];
#pragma unroll
  for (int j = 0; j < IPT; j++) {
    const int i = tid + j * kWmBlock;
    if (i < kn) {
      const float2 v = __ldg(reinterpret_cast<const float2*>(x + scrd[i]));
      xv[j] = DF{v.x, v.y};
    }
  }
  const int items = rn + kn;
  int row, ks;
  tile_search(sre, rn, kn, k0, min(tid * IPT, items), row, ks);
  s.lane_start[tid] = make_int2(row, ks);
  if (tid == 0) {
    int r, k;
    tile_search(sre, rn, kn, k0, min(kWmBlock * IPT, items), r, k);
    s.lane_start[kWmBlock] = make_int2(r, k);
  }
  bool ok = true;
#pragma unroll
  for (int j = 0; j < IPT; j++) {
    const int i = tid + j * kWmBlock;
    if (i < kn) {
      DF p;
      ok &= gp_product(sval[i], xv[j], p);
      as_acc<DF>(sval[i]) = p;
    }
  }
  return __syncthreads_and(ok);
}

// Phase 2: the lane walks its merge items over the staged products; rows are joined as in
// wm_tile.  The open row's sum is kept as a running hi part s and an unnormalised
// compensation c; each product costs one TwoSum.
template <class P, int IPT, class S>
__device__ __forceinline__ void gp_walk(S& s, const DF* sprod, const int32_t* sre, int rn, int k0,
                                        DF& carry) {
  const int tid = threadIdx.x;
  int row = s.lane_start[tid].x;
  const int ks = s.lane_start[tid].y;
  const int row_e = s.lane_start[tid + 1].x, ke = s.lane_start[tid + 1].y;
  const int cnt = ke - ks;
  const int base = k0 + ks;
  int next_end = row < row_e ? sre[row] - base : INT_MAX;  // lane-local index of the next row end
  DF pv[IPT];
#pragma unroll
  for (int j = 0; j < IPT; j++)
    if (j < cnt) pv[j] = sprod[ks + j];
  float hs = 0.f, hc = 0.f;
  DF first = DF{0.f, 0.f};
  int first_row = -1;
  auto emit = [&](int r) {
    DF v;
    two_sum(hs, hc, v.h, v.l);
    hs = 0.f;
    hc = 0.f;
    if (first_row < 0) {
      first_row = r;
      first = v;
    } else {
      as_acc<DF>(s.y[r]) = v;
    }
    row = r + 1;
    next_end = row < row_e ? sre[row] - base : INT_MAX;
  };
#pragma unroll
  for (int j = 0; j < IPT; j++) {
    while (next_end <= j) emit(row);
    if (j < cnt) {
      float s1, e;
      two_sum(hs, pv[j].h, s1, e);
      hc = __fadd_rn(hc, __fadd_rn(e, pv[j].l));
      hs = s1;
    }
  }
  while (row < row_e) emit(row);
  DF acc;
  two_sum(hs, hc, acc.h, acc.l);
  wm_join<P>(s, acc, row_e, first, first_row, rn, carry);
}

// One product-staged tile with native FP64 redo: stage, products (+ search), walk, write y;
// when a value or x entry is outside the double-float range the tile is staged again and
// walked with DFMA.  Returns the FP64 carry-out (thread 0).
template <class P, int IPT, bool TMA>
__device__ __forceinline__ double gp_process_tile(
    WmSmem<P, IPT>& s, const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
    const double* __restrict__ vals, const DF* __restrict__ xg, const double* __restrict__ x64,
    const int* __restrict__ xflag, double* __restrict__ y, int32_t n, int32_t nnz, int r0, int rn,
    int k0, int kn, int* status) {
  static_assert(std::is_same<typename P::Val, double>::value, "FP64 values only");
  using S = WmSmem<P, IPT>;
  const int tid = threadIdx.x;
  int32_t* scrd;
  double* sval;
  const int32_t* sre;
  wm_stage<TMA, P, IPT>(s, pos, crd, vals, n, nnz, r0, rn, k0, kn, status, scrd, sval, sre);
  double carry_d = 0.0;
  if ((xflag == nullptr || *xflag == 0) &&
      gp_products<IPT>(s, scrd, sval, sre, xg, rn, kn, k0)) {
    DF carry = DF{0.f, 0.f};
    gp_walk<PolDF64, IPT>(s, reinterpret_cast<const DF*>(sval), sre, rn, k0, carry);
    for (int i = tid; i < rn; i += kWmBlock) y[r0 + i] = df_to_double(as_acc<DF>(s.y[i]));
    carry_d = df_to_double(carry);
  } else {
    // products may have overwritten staged values: every thread orders its shared-memory
    // writes before the copies that stage the tile again
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    wm_stage<TMA, P, IPT>(s, pos, crd, vals, n, nnz, r0, rn, k0, kn, status, scrd, sval, sre);
    double carry = 0.0;
    wm_tile<PolNative64, IPT, S>(s, scrd, sval, sre, x64, rn, kn, k0, carry);
    for (int i = tid; i < rn; i += kWmBlock) y[r0 + i] = s.y[i];
    carry_d = carry;
  }
  return carry_d;
}

// One tile of rows r0..r0+rn (ends) and nonzeros k0..k0+kn: stage, walk (checked policies first
// try their fast form and redo the tile natively when a value is out of range), write every row
// that ends in the tile to y, and return the FP64 part of the row still open at the tile end.
// xg: x in the policy's gather form; x64: the FP64 x for the native redo; xflag (optional):
// non-zero when x has entries the checked policy cannot represent.
template <class P, int IPT, bool TMA, int CH = 4>
__device__ __forceinline__ double wm_process_tile(
    WmSmem<P, IPT>& s, const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
    const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
    const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
    typename P::Out* __restrict__ y, int32_t n, int32_t nnz, int r0, int rn, int k0, int kn,
    int* status) {
  using S = WmSmem<P, IPT>;
  const int tid = threadIdx.x;
  int32_t* scrd;
  typename P::Val* sval;
  const int32_t* sre;
  wm_stage<TMA, P, IPT>(s, pos, crd, vals, n, nnz, r0, rn, k0, kn, status, scrd, sval, sre);

  double carry_d = 0.0;
  bool native = !P::kChecked;
  if constexpr (P::kChecked) {
    bool ok = (xflag == nullptr || *xflag == 0);
    typename P::Acc carry = P::zero();
    if (__syncthreads_and(ok)) ok = wm_tile<P, IPT, S, CH>(s, scrd, sval, sre, xg, rn, kn, k0, carry);
    if (__syncthreads_and(ok)) {
      for (int i = tid; i < rn; i += kWmBlock) y[r0 + i] = P::out(as_acc<typename P::Acc>(s.y[i]));
      carry_d = P::to_double(carry);
    } else {
      native = true;
    }
  }
  if (native) {
    using Q = typename std::conditional<P::kChecked, PolNative64, P>::type;
    typename Q::Acc carry = Q::zero();
    wm_tile<Q, IPT, S, CH>(s, scrd, (const typename Q::Val*)sval, sre, (const typename Q::XG*)x64,
                           rn, kn, k0, carry);
    for (int i = tid; i < rn; i += kWmBlock)
      y[r0 + i] = (typename P::Out)Q::out(as_acc<typename Q::Acc>(s.y[i]));
    carry_d = Q::to_double(carry);
  }
  return carry_d;  // meaningful in thread 0
}

}  // namespace tacogb
