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
#include <type_traits>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

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
__global__ void merge_partition_scatter(const int32_t* __restrict__ pos, int32_t n,
                                        int64_t nnz, uint32_t T, int32_t tiles,
                                        int32_t snap_len, int2* __restrict__ part) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == n) {
    part[tiles] = make_int2(n, (int)nnz);
    return;
  }
  const int32_t p0 = __ldg(pos + i), p1 = __ldg(pos + i + 1);
  const uint32_t lo = (uint32_t)p0 + (uint32_t)i;
  const uint32_t hi = (uint32_t)p1 + (uint32_t)i;
  const bool snap = (p1 - p0) < snap_len;
  for (uint32_t b = lo / T + (lo % T != 0); (uint64_t)b * T <= hi && (int32_t)b < tiles; b++)
    part[b] = (snap && b > 0) ? make_int2((int)i + 1, p1)
                              : make_int2((int)i, (int)((uint64_t)b * T - (uint64_t)i));
}

int merge_partition(const int32_t* pos, int32_t n, int64_t nnz, int64_t tile_items,
                    int32_t tiles, int2* part, cudaStream_t st, int32_t snap_len) {
  TACOGB_CHECK_ARG(tile_items > 0 && tile_items < (1ll << 30), "bad merge tile size");
  const int64_t threads = (int64_t)n + 1;
  TACOGB_LAUNCH("merge_partition_scatter", st,
                merge_partition_scatter<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                    pos, n, nnz, (uint32_t)tile_items, tiles, snap_len, part));
  return 0;
}

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
}

template <typename T>
__device__ __forceinline__ T ldg_xg(const T* p) { return __ldg(p); }
template <>
__device__ __forceinline__ DF ldg_xg<DF>(const DF* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return DF{v.x, v.y};
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
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
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
  const Acc accv = Wk::take(st);

  // Segmented inclusive scan of lane carries keyed by the open row (keys are non-decreasing
  // along the lanes, so equal keys are contiguous).
  const int key = row_e;
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
  return ok;
}

// xg: x in the policy's gather form (pre-split for the double-float policy); x64: the original
// FP64 x for the native fallback (same as xg for unchecked policies); xflag: non-zero when x
// has entries outside the double-float range.
template <class P, int IPT, bool TMA, int CH = 4>
__global__ void __launch_bounds__(kWmBlock, 8)
spmv_wmerge_kernel(const int32_t* __restrict__ pos, const int32_t* __restrict__ crd,
                   const typename P::Val* __restrict__ vals, const typename P::XG* __restrict__ xg,
                   const typename P::Val* __restrict__ x64, const int* __restrict__ xflag,
                   typename P::Out* __restrict__ y, const int2* __restrict__ part, int32_t n,
                   int32_t nnz, int32_t* __restrict__ carry_row, double* __restrict__ carry_val,
                   int* status) {
  using S = WmSmem<P, IPT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const int tid = threadIdx.x;
  const int tile = blockIdx.x;
  const int2 c0 = part[tile], c1 = part[tile + 1];
  const int r0 = c0.x, k0 = c0.y;
  const int rn = c1.x - c0.x, kn = c1.y - c0.y;

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
  if (tid == 0) {
    carry_row[tile] = r0 + rn;
    carry_val[tile] = carry_d;
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
    carry_row[cb] = (t0 < t1) ? part[t1].x : n;
    carry_val[cb] = carry_in;
  }
}

// Adds the tile carry-outs to the rows that continue into later tiles.  Tiles carrying the same
// row are consecutive; the first tile of each run sums the run in tile order.
template <typename Out>
__global__ void spmv_carry_fixup(const int32_t* __restrict__ carry_row,
                                 const double* __restrict__ carry_val, int32_t tiles,
                                 Out* __restrict__ y, int32_t n) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tiles) return;
  const int32_t r = carry_row[t];
  if (r >= n) return;
  if (t > 0 && carry_row[t - 1] == r) return;
  double tot = carry_val[t];
  for (int32_t u = t + 1; u < tiles && carry_row[u] == r; u++) tot += carry_val[u];
  y[r] = (Out)((double)y[r] + tot);
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
               // 8 family 3 with four accumulators, 9 both
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
  // x pre-split into double-float pairs when the policy gathers DF entries
  constexpr bool presplit = std::is_same<typename P::XG, DF>::value;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t part_bytes = al(((size_t)tiles + 1) * sizeof(int2));
  const size_t crow_bytes = al((size_t)tiles * sizeof(int32_t));
  const size_t cval_bytes = al((size_t)tiles * sizeof(double));
  const size_t xdf_bytes = presplit ? al((size_t)A->cols * sizeof(DF)) + 256 : 0;
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
  if (int rc = merge_partition(A->pos, A->rows, A->nnz, tile_items, tiles, part, st)) return rc;
  // Bulk copies need 16-byte aligned sources: true for every allocator the library meets
  // (cudaMalloc, cudaMallocManaged, torch); sliced pointers take the register-staged kernel.
  const bool tma = (((uintptr_t)A->pos | (uintptr_t)A->crd | (uintptr_t)A->vals) & 15) == 0;
  auto kern = tma ? spmv_wmerge_kernel<P, IPT, true, CH> : spmv_wmerge_kernel<P, IPT, false, CH>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(S)));
  TACOGB_LAUNCH("spmv_wmerge_kernel", st,
                kern<<<tiles, kWmBlock, sizeof(S), st>>>(
                    A->pos, A->crd, (const typename P::Val*)A->vals, xg, x, xflag, y, part,
                    A->rows, (int32_t)A->nnz, crow, cval, status));
  TACOGB_LAUNCH("spmv_carry_fixup", st,
                spmv_carry_fixup<typename P::Out><<<(tiles + 255) / 256, 256, 0, st>>>(
                    crow, cval, tiles, y, A->rows));
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

// Structural rule used when neither a tuning record nor the cost model gives a choice: the
// merge family is robust to any skew, and for FP64 values the double-float policy keeps the
// kernel off GB300's narrow FP64 pipe (IPT 7 measured fastest on the power-law workload).
int spmv_default_variant(const tacogb_csr* A) {
  (void)A;
  return 10;  // wmerge_dfx_ipt7: double-float for FP64 values, compensated FP32 for FP32
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
  if (variant < 0) variant = spmv_default_variant(A);
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
  const int64_t threads = (int64_t)A->rows + 1;
  count_launch();
  merge_partition_scatter<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
      A->pos, A->rows, A->nnz, (uint32_t)kNoAllocTileItems, tiles, 0, part);
  if (int rc = launch_check("merge_partition_scatter")) return rc;
  auto kern = spmv_wmerge_kernel<P, kNoAllocIpt, false>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sizeof(S)));
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
