// Two-phase CSR x CSR SpGEMM for sm_103a: C(i,k) = A(i,j) * B(j,k), all operands CSR.
//
// Replaces the assemble and compute functions taco generates for this statement through the
// workspace form forall(i, where(forall(k, C(i,k) = w(k)), forall(j,k, w(k) += A(i,j)*B(j,k))))
// (src/index_notation/transformations.cpp:2083, dense accelerator arrays from
// src/lower/lowerer_impl_imperative.cpp:2197, compressed appends from
// src/lower/mode_format_compressed.cpp:107-213) and its parallel two-pass form
// (test/tests-scheduling-eval.cpp:68-94 -> lowerAssemble,
// src/lower/lowerer_impl_imperative.cpp:2616-2781).  taco has no GPU schedule for SpGEMM.
//
// Semantics kept exactly: every structural product is kept (no numerical-zero dropping), the
// columns of each row are sorted ascending, and each output value is the sum of its products in
// A-row order, the first product initialising it — the order of taco's serial loop.  Products
// and sums are separately rounded (no FMA), so values are bit-identical to taco's generated
// code when that code is compiled without FMA contraction.
//
// Work decomposition: per row, the product count P_i = sum of B-row lengths over A's row.  Rows
// are binned by P_i; each bin runs expand-sort-compress (ESC) on (column, sequence) keys:
//   bin 1  P <= 32     one warp per row, keys in registers, warp bitonic sort by shuffles
//   bin 2  P <= 256    one warp per row, bitonic sort in registers (P <= 128: two or four keys
//                      per lane, shuffles) or in the warp's shared-memory slice
//   bin 3  P <= 4096   one CTA per row, bitonic sort in shared memory
//   bin 4  P >  4096   one CTA per row over a dense per-CTA accumulator in global scratch
//                      (column bitmap for the pattern, stamp + value arrays for the numbers)
// Phases: symbolic count -> device exclusive scan -> (caller allocates) -> crd fill; numeric.
// One-pass form (taco's assemble-while-compute, used by evaluate): the rows' products go to
// slots sized by P_i (an exclusive scan of the product counts); one ESC pass sorts keys and
// values together and writes each row's sorted columns, summed values and count into its slot;
// a scan of the counts gives pos and a compaction moves the slots into C.  One sort per row
// where the three-phase form sorts three times.
// Bin lists are built with per-bin atomic counters; the order of rows inside a list does not
// affect any result.

#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "kernels.h"

namespace tacogb {

namespace {

constexpr int kBins = 5;  // 0: empty rows, 1..4 as above
constexpr int kBin1 = 32, kBin2 = 256, kBin3 = 4096;
constexpr int kDenseSlots = 64;  // concurrent CTAs of the dense (bin 4) path

__device__ __forceinline__ int bin_of(int64_t p) {
  return p == 0 ? 0 : p <= kBin1 ? 1 : p <= kBin2 ? 2 : p <= kBin3 ? 3 : 4;
}

// P_i per row, and the row appended to its bin's list (warp-aggregated atomics per bin).
__global__ void spgemm_bin_rows(const int32_t* __restrict__ Apos, const int32_t* __restrict__ Acrd,
                                const int32_t* __restrict__ Bpos, int32_t n,
                                int64_t* __restrict__ prod, int32_t* __restrict__ bin_cnt,
                                int32_t* __restrict__ bin_rows) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int b = -1;
  if (i < n) {
    int64_t p = 0;
    for (int32_t q = __ldg(Apos + i); q < __ldg(Apos + i + 1); q++) {
      const int32_t j = __ldg(Acrd + q);
      p += __ldg(Bpos + j + 1) - __ldg(Bpos + j);
    }
    prod[i] = p;
    b = bin_of(p);
  }
  const int lane = threadIdx.x & 31;
  for (int bb = 0; bb < kBins; bb++) {
    const unsigned m = __ballot_sync(0xffffffffu, b == bb);
    if (!m) continue;
    int base = 0;
    const int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(bin_cnt + bb, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (b == bb) bin_rows[(int64_t)bb * n + base + __popc(m & ((1u << lane) - 1))] = (int32_t)i;
  }
}

// Sorts 64-bit keys (and payloads) of one warp, one per lane, ascending; invalid lanes hold
// UINT64_MAX.
template <typename V>
__device__ __forceinline__ void warp_bitonic(uint64_t& key, V& val) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const uint64_t ok = __shfl_xor_sync(0xffffffffu, key, j);
      const V ov = __shfl_xor_sync(0xffffffffu, val, j);
      // keys are distinct but for the empty slots', whose payloads are all zero
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      const bool take = (ok < key) == keep_min;
      key = take ? ok : key;
      val = take ? ov : val;
    }
  }
}

// warp_bitonic / reg_bitonic on narrow keys without payloads.
__device__ __forceinline__ void warp_bitonic32(uint32_t& key) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const uint32_t ok = __shfl_xor_sync(0xffffffffu, key, j);
      // the lower lane of an ascending pair (or the upper of a descending one) keeps the min
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      key = keep_min ? min(ok, key) : max(ok, key);
    }
  }
}

template <int R>
__device__ __forceinline__ void reg_bitonic32(uint32_t (&key)[R]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int jr = j >> 5;
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (r & jr) continue;
          const bool up = ((r * 32) & k) == 0;  // k >= 64 here: the lane's bits do not matter
          const uint32_t lo = min(key[r], key[r | jr]), hi = max(key[r], key[r | jr]);
          key[r] = up ? lo : hi;
          key[r | jr] = up ? hi : lo;
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) {
          const uint32_t ok = __shfl_xor_sync(0xffffffffu, key[r], j);
          const bool keep_min = ((lane & j) == 0) == (((r * 32 + lane) & k) == 0);
          key[r] = keep_min ? min(ok, key[r]) : max(ok, key[r]);
        }
      }
    }
  }
}

// The values of sorted narrow keys: slot (r, lane) takes the value of product key[r] & 0xFF
// from the registers val[] of the lane that computed it.
template <int R, typename V>
__device__ __forceinline__ void gather_sorted_vals(const uint32_t (&key)[R], V (&val)[R]) {
  V out[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int e = (int)(key[r] & 0xFFu);
    V g = V();
#pragma unroll
    for (int rr = 0; rr < R; rr++) {
      const V t = __shfl_sync(0xffffffffu, val[rr], e & 31);
      if ((e >> 5) == rr) g = t;
    }
    out[r] = g;
  }
#pragma unroll
  for (int r = 0; r < R; r++) val[r] = out[r];
}

// Bitonic sort of cap (power of two) keys/payloads in shared memory by `nthreads` threads
// starting at thread index `t0`; `sync` synchronises those threads.
template <typename V, typename Sync>
__device__ __forceinline__ void smem_bitonic(uint64_t* key, V* val, int cap, int t, int nthreads,
                                             Sync sync) {
  for (int k = 2; k <= cap; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int idx = t; idx < cap / 2; idx += nthreads) {
        const int i = 2 * idx - (idx & (j - 1));
        const int p = i + j;
        const bool up = (i & k) == 0;
        const uint64_t a = key[i], b = key[p];
        if ((a > b) == up) {
          key[i] = b;
          key[p] = a;
          const V tv = val[i];
          val[i] = val[p];
          val[p] = tv;
        }
      }
      sync();
    }
  }
}

template <typename V> __device__ __forceinline__ V mul_rn(V a, V b);
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <typename V> __device__ __forceinline__ V add_rn(V a, V b);
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ uint64_t esc_key(int32_t col, int32_t seq) {
  return ((uint64_t)(uint32_t)col << 32) | (uint32_t)seq;
}
__device__ __forceinline__ int32_t key_col(uint64_t k) { return (int32_t)(k >> 32); }

// Narrow keys for the register sorts when B has fewer than 2^24 columns: column << 8 | the
// product's sequence number (< 256 in bins 1 and 2), with 0xFFFFFFFF for empty slots (above
// every key, since columns stay below 2^24 - 1).  Only the keys move through the sorting
// network; each value is fetched once afterwards from the lane and register that computed it
// (sequence number e lives in lane e % 32, register e / 32).  The order is that of the wide
// keys (column, then sequence), so the sums are the same bit for bit.
constexpr int64_t kNarrowKeyCols = (1 << 24) - 1;
__device__ __forceinline__ uint32_t narrow_key(uint64_t k) {
  return k == ~0ull ? 0xFFFFFFFFu : ((uint32_t)key_col(k) << 8) | ((uint32_t)k & 0xFFu);
}
__device__ __forceinline__ uint64_t wide_key(uint32_t k) {
  return k == 0xFFFFFFFFu ? ~0ull : esc_key((int32_t)(k >> 8), (int32_t)(k & 0xFFu));
}

// What a pass computes and writes: MODE 0 counts (cnt), 1 writes columns at Cpos, 2 writes
// values at Cpos, 3 (one pass) writes columns and values at the row's product slot (Cpos holds
// the slot offsets) and counts.
template <int MODE> constexpr bool mode_vals() { return MODE == 2 || MODE == 3; }
template <int MODE> constexpr bool mode_crd() { return MODE == 1 || MODE == 3; }
template <int MODE> constexpr bool mode_count() { return MODE == 0 || MODE == 3; }

// MODE 0: count unique columns -> cnt[row]; 1: write sorted columns at Cpos[row];
// 2: write values (sum of products in sequence order) at Cpos[row].
template <int MODE, typename V>
__device__ __forceinline__ void esc_emit_warp(const uint64_t* key, const V* val, int P, int row,
                                              const int32_t* __restrict__ Cpos,
                                              int32_t* __restrict__ cnt,
                                              int32_t* __restrict__ Ccrd, V* __restrict__ Cvals) {
  const int lane = threadIdx.x & 31;
  int base = 0;
  const int out0 = (MODE == 0) ? 0 : Cpos[row];
  for (int c = 0; c < P; c += 32) {
    const int e = c + lane;
    const bool head = e < P && (e == 0 || key_col(key[e]) != key_col(key[e - 1]));
    const unsigned m = __ballot_sync(0xffffffffu, head);
    if (MODE != 0 && head) {
      const int rank = base + __popc(m & ((1u << lane) - 1));
      if (mode_crd<MODE>()) Ccrd[out0 + rank] = key_col(key[e]);
      if (mode_vals<MODE>()) {
        V s = val[e];
        for (int f = e + 1; f < P && key_col(key[f]) == key_col(key[e]); f++) s = add_rn(s, val[f]);
        Cvals[out0 + rank] = s;
      }
    }
    base += __popc(m);
  }
  if (mode_count<MODE>() && lane == 0) cnt[row] = base;
}

// Expands row `row`'s products into (key, value) slots [0, P) of a buffer, strided over
// `nthreads` threads starting at `t`.
template <bool VALS, typename V>
__device__ __forceinline__ void esc_expand(const int32_t* __restrict__ Apos,
                                           const int32_t* __restrict__ Acrd,
                                           const V* __restrict__ Avals,
                                           const int32_t* __restrict__ Bpos,
                                           const int32_t* __restrict__ Bcrd,
                                           const V* __restrict__ Bvals, int row, uint64_t* key,
                                           V* val, int t, int nthreads) {
  // Walk A's row; each thread handles products strided over the concatenated B rows.
  int seq0 = 0;
  for (int32_t q = __ldg(Apos + row); q < __ldg(Apos + row + 1); q++) {
    const int32_t j = __ldg(Acrd + q);
    const int32_t b0 = __ldg(Bpos + j), len = __ldg(Bpos + j + 1) - b0;
    V a = V();
    if (VALS) a = Avals[q];
    for (int u = t; u < len; u += nthreads) {
      key[seq0 + u] = esc_key(__ldg(Bcrd + b0 + u), seq0 + u);
      if (VALS) val[seq0 + u] = mul_rn(a, Bvals[b0 + u]);
    }
    seq0 += len;
  }
}

// Expands row `row`'s products into a warp's registers: product e = r * 32 + lane, in sequence
// order (A's entries in order, each B row in order), gets key esc_key(column, e) and, with
// VALS, the value A(row, j) * B(j, column); slots past the row's P products are left alone.
// The lanes load up to 32 of A's entries and their B row bounds at once, and a scan of the B
// row lengths places every product (the source entry of slot e is the number of entries whose
// inclusive end is at most e, found by a five-step shuffle search), so a row costs four rounds
// of dependent loads instead of three per A entry.  P <= 32 * R.  Returns P.
template <int R, bool VALS, typename V>
__device__ __forceinline__ int warp_expand_regs(const int32_t* __restrict__ Apos,
                                                const int32_t* __restrict__ Acrd,
                                                const V* __restrict__ Avals,
                                                const int32_t* __restrict__ Bpos,
                                                const int32_t* __restrict__ Bcrd,
                                                const V* __restrict__ Bvals, int row,
                                                uint64_t (&key)[R], V (&val)[R]) {
  const int lane = threadIdx.x & 31;
  const int32_t a0 = __ldg(Apos + row), na = __ldg(Apos + row + 1) - a0;
  int seq0 = 0;
  for (int c = 0; c < na; c += 32) {
    int32_t b0 = 0, len = 0;
    V av = V();
    if (c + lane < na) {
      const int32_t j = __ldg(Acrd + a0 + c + lane);
      if (VALS) av = Avals[a0 + c + lane];
      b0 = __ldg(Bpos + j);
      len = __ldg(Bpos + j + 1) - b0;
    }
    int inc = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += t;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    const int exc = inc - len;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int e = r * 32 + lane - seq0;  // this chunk's product index of slot (r, lane)
      const int ec = min(max(e, 0), max(total - 1, 0));
      int src = 0;
#pragma unroll
      for (int step = 16; step >= 1; step >>= 1) {
        const int t = __shfl_sync(0xffffffffu, inc, src + step - 1);
        if (t <= ec) src += step;
      }
      const int sb = __shfl_sync(0xffffffffu, b0, src);
      const int sx = __shfl_sync(0xffffffffu, exc, src);
      V sa = V();
      if (VALS) sa = __shfl_sync(0xffffffffu, av, src);
      if (e >= 0 && e < total) {
        const int u = e - sx;
        key[r] = esc_key(__ldg(Bcrd + sb + u), r * 32 + lane);
        if (VALS) val[r] = mul_rn(sa, Bvals[sb + u]);
      }
    }
    seq0 += total;
  }
  return seq0;
}

// ---- bin 1: P <= 32, one warp per row, registers -----------------------------------------

template <int MODE, typename V, bool K32>
__global__ void __launch_bounds__(256)
spgemm_bin1(const int32_t* __restrict__ Apos, const int32_t* __restrict__ Acrd,
            const V* __restrict__ Avals, const int32_t* __restrict__ Bpos,
            const int32_t* __restrict__ Bcrd, const V* __restrict__ Bvals,
            const int32_t* __restrict__ rows, const int32_t* __restrict__ count,
            const int32_t* __restrict__ Cpos, int32_t* __restrict__ cnt,
            int32_t* __restrict__ Ccrd, V* __restrict__ Cvals) {
  const int lane = threadIdx.x & 31;
  const int nr = *count;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nr;
       w += (gridDim.x * blockDim.x) >> 5) {
    const int row = rows[w];
    // lane l takes product l (<= 32 products)
    uint64_t k1[1] = {~0ull};
    V v1[1] = {V()};
    const int P = warp_expand_regs<1, mode_vals<MODE>()>(Apos, Acrd, Avals, Bpos, Bcrd, Bvals,
                                                         row, k1, v1);
    uint64_t key = k1[0];
    V val = v1[0];
    if constexpr (K32) {
      uint32_t k32[1] = {narrow_key(key)};
      warp_bitonic32(k32[0]);
      if (mode_vals<MODE>()) gather_sorted_vals<1>(k32, v1);
      key = wide_key(k32[0]);
      val = v1[0];
    } else {
      warp_bitonic(key, val);
    }
    const uint64_t prevk = __shfl_up_sync(0xffffffffu, key, 1);
    const bool valid = lane < P;
    const bool head = valid && (lane == 0 || key_col(prevk) != key_col(key));
    const unsigned m = __ballot_sync(0xffffffffu, head);
    if (mode_count<MODE>() && lane == 0) cnt[row] = __popc(m);
    if (MODE != 0) {
      // run sums in sequence order: lane-serial accumulation along each run
      V s = val;
      if (mode_vals<MODE>()) {
        // walk forward within the run from each head
        for (int d = 1; d < 32; d++) {
          const uint64_t kd = __shfl_down_sync(0xffffffffu, key, d);
          const V vd = __shfl_down_sync(0xffffffffu, val, d);
          const bool same = (lane + d < P) && key_col(kd) == key_col(key);
          const bool any = __any_sync(0xffffffffu, head && same);
          if (!any) break;
          if (head && same) s = add_rn(s, vd);
        }
      }
      if (head) {
        const int rank = __popc(m & ((1u << lane) - 1));
        const int o = Cpos[row] + rank;
        if (mode_crd<MODE>()) Ccrd[o] = key_col(key);
        if (mode_vals<MODE>()) Cvals[o] = s;
      }
    }
  }
}

// ---- bin 2: P <= 256, one warp per row, shared memory -------------------------------------

// Bitonic sort of a warp's 32*R keys (and payloads) held in registers, element r*32 + lane in
// key[r]: strides of 32 and more swap registers within a lane, shorter ones exchange by shuffle.
// Ascending; no shared memory, so the sort does not occupy the shared-memory pipe.  Without
// VALS (the symbolic and fill phases) the payloads are left alone.
template <int R, bool VALS, typename V>
__device__ __forceinline__ void reg_bitonic(uint64_t (&key)[R], V (&val)[R]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int jr = j >> 5;
#pragma unroll
        for (int r = 0; r < R; r++) {
          if (r & jr) continue;
          const bool up = ((r * 32) & k) == 0;  // k >= 64 here: the lane's bits do not matter
          const uint64_t a = key[r], b = key[r | jr];
          const bool sw = (a > b) == up;
          key[r] = sw ? b : a;
          key[r | jr] = sw ? a : b;
          if (VALS) {
            const V va = val[r], vb = val[r | jr];
            val[r] = sw ? vb : va;
            val[r | jr] = sw ? va : vb;
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) {
          const uint64_t ok = __shfl_xor_sync(0xffffffffu, key[r], j);
          V ov = V();
          if (VALS) ov = __shfl_xor_sync(0xffffffffu, val[r], j);
          const bool keep_min = ((lane & j) == 0) == (((r * 32 + lane) & k) == 0);
          const bool take = (ok < key[r]) == keep_min;
          key[r] = take ? ok : key[r];
          if (VALS) val[r] = take ? ov : val[r];
        }
      }
    }
  }
}

// Rows of at most 32*R products: each lane computes products lane, lane + 32, ...
// (warp_expand_regs), sorts them in registers, then leaves them in the warp's shared slice for
// the run detection and emission of esc_emit_warp.
template <int R, int MODE, bool K32, typename V>
__device__ __forceinline__ void bin2_row_regs(const int32_t* __restrict__ Apos,
                                              const int32_t* __restrict__ Acrd,
                                              const V* __restrict__ Avals,
                                              const int32_t* __restrict__ Bpos,
                                              const int32_t* __restrict__ Bcrd,
                                              const V* __restrict__ Bvals, int row, uint64_t* skey,
                                              V* sval) {
  const int lane = threadIdx.x & 31;
  uint64_t key[R];
  V val[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    key[r] = ~0ull;
    val[r] = V();
  }
  warp_expand_regs<R, mode_vals<MODE>()>(Apos, Acrd, Avals, Bpos, Bcrd, Bvals, row, key, val);
  if constexpr (K32) {
    uint32_t k32[R];
#pragma unroll
    for (int r = 0; r < R; r++) k32[r] = narrow_key(key[r]);
    reg_bitonic32<R>(k32);
    if (mode_vals<MODE>()) gather_sorted_vals<R>(k32, val);
#pragma unroll
    for (int r = 0; r < R; r++) key[r] = wide_key(k32[r]);
  } else {
    reg_bitonic<R, mode_vals<MODE>()>(key, val);
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    skey[r * 32 + lane] = key[r];
    if (mode_vals<MODE>()) sval[r * 32 + lane] = val[r];
  }
  __syncwarp();
}

template <int MODE, typename V, bool K32>
__global__ void __launch_bounds__(256)
spgemm_bin2(const int32_t* __restrict__ Apos, const int32_t* __restrict__ Acrd,
            const V* __restrict__ Avals, const int32_t* __restrict__ Bpos,
            const int32_t* __restrict__ Bcrd, const V* __restrict__ Bvals,
            const int32_t* __restrict__ rows, const int32_t* __restrict__ count,
            const int64_t* __restrict__ prod, const int32_t* __restrict__ Cpos,
            int32_t* __restrict__ cnt, int32_t* __restrict__ Ccrd, V* __restrict__ Cvals) {
  __shared__ uint64_t s_key[8][kBin2];
  __shared__ V s_val[8][kBin2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* key = s_key[warp];
  V* val = s_val[warp];
  const int nr = *count;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nr;
       w += (gridDim.x * blockDim.x) >> 5) {
    const int row = rows[w];
    const int P = (int)prod[row];
    int cap = 32;
    while (cap < P) cap <<= 1;
    if (cap <= 64) {
      bin2_row_regs<2, MODE, K32>(Apos, Acrd, Avals, Bpos, Bcrd, Bvals, row, key, val);
    } else if (cap <= 128) {
      bin2_row_regs<4, MODE, K32>(Apos, Acrd, Avals, Bpos, Bcrd, Bvals, row, key, val);
    } else {
      esc_expand<mode_vals<MODE>()>(Apos, Acrd, Avals, Bpos, Bcrd, Bvals, row, key, val, lane,
                                    32);
      for (int e = P + lane; e < cap; e += 32) key[e] = ~0ull;
      __syncwarp();
      smem_bitonic(key, val, cap, lane, 32, [] __device__() { __syncwarp(); });
    }
    esc_emit_warp<MODE>(key, val, P, row, Cpos, cnt, Ccrd, Cvals);
    __syncwarp();
  }
}

// ---- bin 3: P <= 4096, one CTA per row, shared memory -------------------------------------

template <int MODE, typename V>
__global__ void __launch_bounds__(256)
spgemm_bin3(const int32_t* __restrict__ Apos, const int32_t* __restrict__ Acrd,
            const V* __restrict__ Avals, const int32_t* __restrict__ Bpos,
            const int32_t* __restrict__ Bcrd, const V* __restrict__ Bvals,
            const int32_t* __restrict__ rows, const int32_t* __restrict__ count,
            const int64_t* __restrict__ prod, const int32_t* __restrict__ Cpos,
            int32_t* __restrict__ cnt, int32_t* __restrict__ Ccrd, V* __restrict__ Cvals) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* key = reinterpret_cast<uint64_t*>(smem_raw);
  V* val = reinterpret_cast<V*>(key + kBin3);
  __shared__ int32_t s_wcount[8];
  const int nr = *count;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int w = blockIdx.x; w < nr; w += gridDim.x) {
    const int row = rows[w];
    const int P = (int)prod[row];
    int cap = 32;
    while (cap < P) cap <<= 1;
    esc_expand<mode_vals<MODE>()>(Apos, Acrd, Avals, Bpos, Bcrd, Bvals, row, key, val, tid,
                                  256);
    for (int e = P + tid; e < cap; e += 256) key[e] = ~0ull;
    __syncthreads();
    smem_bitonic(key, val, cap, tid, 256, [] __device__() { __syncthreads(); });
    // heads: per-thread chunks of ELEMS consecutive slots, block prefix over chunk counts
    constexpr int ELEMS = kBin3 / 256;
    const int e0 = tid * ELEMS;
    int local = 0;
    for (int e = e0; e < e0 + ELEMS && e < P; e++)
      local += (e == 0 || key_col(key[e]) != key_col(key[e - 1]));
    // block exclusive scan of `local`
    int incl = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int o = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += o;
    }
    if (lane == 31) s_wcount[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int x = 0; x < warp; x++) wbase += s_wcount[x];
    int rank = wbase + incl - local;
    if (mode_count<MODE>() && tid == 255) cnt[row] = wbase + incl;
    if (MODE != 0) {
      const int o0 = Cpos[row];
      for (int e = e0; e < e0 + ELEMS && e < P; e++) {
        if (e == 0 || key_col(key[e]) != key_col(key[e - 1])) {
          if (mode_crd<MODE>()) Ccrd[o0 + rank] = key_col(key[e]);
          if (mode_vals<MODE>()) {
            V s = val[e];
            for (int f = e + 1; f < P && key_col(key[f]) == key_col(key[e]); f++) s = add_rn(s, val[f]);
            Cvals[o0 + rank] = s;
          }
          rank++;
        }
      }
    }
    __syncthreads();
  }
}

// ---- bin 4: P > 4096, one CTA per row, dense accumulator in global scratch -----------------
//
// Per CTA slot: a column bitmap (K bits) and, for values, a stamp (int32 per column, the row
// that last touched it) and an accumulator (V per column).  A's row is walked in order; the
// threads split each B row, whose columns are distinct, so every column's products are added
// in A-row order without atomics.  The pattern is read back by scanning the bitmap words in
// column order, which yields sorted columns directly.

template <int MODE, typename V>
__global__ void __launch_bounds__(256)
spgemm_bin4(const int32_t* __restrict__ Apos, const int32_t* __restrict__ Acrd,
            const V* __restrict__ Avals, const int32_t* __restrict__ Bpos,
            const int32_t* __restrict__ Bcrd, const V* __restrict__ Bvals,
            const int32_t* __restrict__ rows, const int32_t* __restrict__ count, int32_t K,
            uint32_t* __restrict__ bitmap_all, int32_t* __restrict__ stamp_all,
            V* __restrict__ acc_all, const int32_t* __restrict__ Cpos,
            int32_t* __restrict__ cnt, int32_t* __restrict__ Ccrd, V* __restrict__ Cvals) {
  const int nr = *count;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int words = (K + 31) >> 5;
  uint32_t* bitmap = bitmap_all + (int64_t)blockIdx.x * words;
  int32_t* stamp = stamp_all + (int64_t)blockIdx.x * K;
  V* acc = acc_all + (int64_t)blockIdx.x * K;
  __shared__ int32_t s_wcount[8];
  __shared__ int32_t s_base;
  for (int w = blockIdx.x; w < nr; w += gridDim.x) {
    const int row = rows[w];
    for (int32_t q = __ldg(Apos + row); q < __ldg(Apos + row + 1); q++) {
      const int32_t j = __ldg(Acrd + q);
      const int32_t b0 = __ldg(Bpos + j), b1 = __ldg(Bpos + j + 1);
      V a = V();
      if (mode_vals<MODE>()) a = Avals[q];
      for (int32_t u = b0 + tid; u < b1; u += 256) {
        const int32_t k = __ldg(Bcrd + u);
        if (mode_vals<MODE>()) {
          const V pr = mul_rn(a, Bvals[u]);
          if (stamp[k] != row) {
            stamp[k] = row;
            acc[k] = pr;
          } else {
            acc[k] = add_rn(acc[k], pr);
          }
        }
        if (MODE != 2) atomicOr(bitmap + (k >> 5), 1u << (k & 31));
      }
      __syncthreads();  // B rows of later A nonzeros may hit the same columns
    }
    if (MODE == 2) {
      // the pattern is known: gather accumulated values in column order
      for (int32_t t = Cpos[row] + tid; t < Cpos[row + 1]; t += 256) Cvals[t] = acc[Ccrd[t]];
      __syncthreads();
      continue;
    }
    // scan the bitmap in column order (chunks of 256 words)
    if (tid == 0) s_base = 0;
    __syncthreads();
    for (int c = 0; c < words; c += 256) {
      const int wi = c + tid;
      const uint32_t bits = wi < words ? bitmap[wi] : 0u;
      const int pc = __popc(bits);
      int incl = pc;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += o;
      }
      if (lane == 31) s_wcount[warp] = incl;
      __syncthreads();
      int wbase = 0, total = 0;
      for (int x = 0; x < 8; x++) {
        if (x < warp) wbase += s_wcount[x];
        total += s_wcount[x];
      }
      if (mode_crd<MODE>() && bits) {
        int r = s_base + wbase + incl - pc;
        const int o0 = Cpos[row];
        uint32_t bb = bits;
        while (bb) {
          const int bit = __ffs(bb) - 1;
          const int col = (wi << 5) + bit;
          Ccrd[o0 + r] = col;
          if (mode_vals<MODE>()) Cvals[o0 + r] = acc[col];
          r++;
          bb &= bb - 1;
        }
      }
      if (wi < words) bitmap[wi] = 0u;  // leave the slot clean for the next row
      __syncthreads();
      if (tid == 0) s_base += total;
      __syncthreads();
    }
    if (mode_count<MODE>() && tid == 0) cnt[row] = s_base;
    __syncthreads();
  }
}

// ---- exclusive scan of row counts into pos (int32, overflow-checked) -----------------------

constexpr int kScanChunk = 4096;

__global__ void scan_block_sums(const int32_t* __restrict__ cnt, int32_t n,
                                int64_t* __restrict__ sums) {
  __shared__ int64_t s[256];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  int64_t t = 0;
  for (int e = threadIdx.x; e < kScanChunk; e += 256)
    if (base + e < n) t += cnt[base + e];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) s[threadIdx.x] += s[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = s[0];
}

// Exclusive scan of the block sums by one warp, 32 at a time; sums[nblocks] = the total.
__global__ void scan_sums_exclusive(int64_t* __restrict__ sums, int32_t nblocks,
                                    int32_t* __restrict__ total_overflow) {
  const int lane = threadIdx.x & 31;
  int64_t carry = 0;
  for (int32_t b0 = 0; b0 < nblocks; b0 += 32) {
    const int32_t b = b0 + lane;
    const int64_t v = b < nblocks ? sums[b] : 0;
    int64_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += t;
    }
    if (b < nblocks) sums[b] = carry + inc - v;
    carry += __shfl_sync(0xffffffffu, inc, 31);
  }
  if (lane == 0) {
    sums[nblocks] = carry;
    *total_overflow = carry > INT32_MAX ? 1 : 0;
  }
}

// Small results into the host mailbox from kMailboxSpgemm on: nb bin sizes, then a total and
// an overflow flag (plain stores to mapped host memory).
__global__ void spgemm_publish(const int32_t* __restrict__ bin_cnt, int nb,
                               const int64_t* __restrict__ total, const int32_t* __restrict__ flag,
                               volatile unsigned long long* box) {
  const int t = threadIdx.x;
  if (t < nb) box[t] = (unsigned long long)(uint32_t)bin_cnt[t];
  if (t == nb && total) box[t] = (unsigned long long)*total;
  if (t == nb + 1 && flag) box[t] = (unsigned long long)(uint32_t)*flag;
  __threadfence_system();
}

__global__ void scan_write_pos(const int32_t* __restrict__ cnt, int32_t n,
                               const int64_t* __restrict__ sums, int32_t* __restrict__ pos) {
  __shared__ int64_t s_warp[8];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int PER = kScanChunk / 256;
  const int64_t e0 = base + (int64_t)threadIdx.x * PER;
  int64_t local[PER];
  int64_t t = 0;
#pragma unroll
  for (int e = 0; e < PER; e++) {
    local[e] = t;
    t += (e0 + e < n) ? cnt[e0 + e] : 0;
  }
  int64_t incl = t;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int64_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  int64_t wb = 0;
  for (int x = 0; x < warp; x++) wb += s_warp[x];
  const int64_t off = sums[blockIdx.x] + wb + incl - t;
#pragma unroll
  for (int e = 0; e < PER; e++)
    if (e0 + e < n) pos[e0 + e] = (int32_t)(off + local[e]);
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) pos[n] = (int32_t)sums[gridDim.x];
}

// ---- host orchestration -------------------------------------------------------------------

struct Plan {
  int64_t* prod;
  int32_t* bin_cnt;   // kBins counters
  int32_t* bin_rows;  // kBins * n
  int32_t* cnt;       // per-row unique counts (symbolic)
  int64_t* sums;      // scan block sums
  int32_t* flag;      // overflow flag
  int32_t h_cnt[kBins];
};

// The mailbox words SpGEMM publishes into, or null (the error is set).
volatile unsigned long long* spgemm_box() {
  unsigned long long* box = host_mailbox();
  return box ? box + kMailboxSpgemm : nullptr;
}

// Publishes (nb bin sizes, total, flag) into the mailbox, waits for st, and reads them back.
int publish_and_wait(const int32_t* bin_cnt, int nb, const int64_t* total, const int32_t* flag,
                     int32_t* h_cnt, int64_t* h_total, bool* h_overflow, cudaStream_t st) {
  volatile unsigned long long* box = spgemm_box();
  if (!box) return last_code();
  TACOGB_LAUNCH("spgemm_publish", st,
                spgemm_publish<<<1, 32, 0, st>>>(bin_cnt, nb, total, flag,
                                                 (unsigned long long*)box));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  for (int b = 0; b < nb; b++) h_cnt[b] = (int32_t)box[b];
  if (h_total) *h_total = (int64_t)box[nb];
  if (h_overflow) *h_overflow = box[nb + 1] != 0;
  return 0;
}

// Bins the rows of A*B; with `wait`, reads the bin sizes back (one synchronisation).
int make_plan(const tacogb_csr* A, const tacogb_csr* B, Plan& pl, cudaStream_t st,
              bool wait = true) {
  const int64_t n = A->rows;
  const int64_t nblocks = (n + kScanChunk - 1) / kScanChunk;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t off = 0;
  const size_t o_prod = off; off += al(sizeof(int64_t) * (n + 1));
  const size_t o_bc = off; off += al(sizeof(int32_t) * kBins);
  const size_t o_br = off; off += al(sizeof(int32_t) * kBins * (n + 1));
  const size_t o_cnt = off; off += al(sizeof(int32_t) * (n + 1));
  const size_t o_sums = off; off += al(sizeof(int64_t) * (nblocks + 2));
  const size_t o_flag = off; off += al(sizeof(int32_t) * 4);
  unsigned char* ws = (unsigned char*)scratch(off, 2);
  if (!ws) return last_code();
  pl.prod = (int64_t*)(ws + o_prod);
  pl.bin_cnt = (int32_t*)(ws + o_bc);
  pl.bin_rows = (int32_t*)(ws + o_br);
  pl.cnt = (int32_t*)(ws + o_cnt);
  pl.sums = (int64_t*)(ws + o_sums);
  pl.flag = (int32_t*)(ws + o_flag);
  TACOGB_CUDA_TRY(cudaMemsetAsync(pl.bin_cnt, 0, sizeof(int32_t) * kBins, st));
  TACOGB_CUDA_TRY(cudaMemsetAsync(pl.cnt, 0, sizeof(int32_t) * (n + 1), st));
  if (n > 0)
    TACOGB_LAUNCH("spgemm_bin_rows", st,
                  spgemm_bin_rows<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                      A->pos, A->crd, B->pos, (int32_t)n, pl.prod, pl.bin_cnt, pl.bin_rows));
  if (!wait) return 0;
  return publish_and_wait(pl.bin_cnt, kBins, nullptr, nullptr, pl.h_cnt, nullptr, nullptr, st);
}

template <int MODE, typename V>
int run_bins(const tacogb_csr* A, const tacogb_csr* B, const Plan& pl, const int32_t* Cpos,
             int32_t* Ccrd, V* Cvals, cudaStream_t st) {
  const int64_t n = A->rows;
  const V* Av = (const V*)A->vals;
  const V* Bv = (const V*)B->vals;
  const int sms = sm_count();
  auto rows_of = [&](int b) { return pl.bin_rows + (int64_t)b * n; };
  auto grid = [](int64_t items, int64_t cap) { return (unsigned)(items < cap ? items : cap); };
  const bool k32 = B->cols <= kNarrowKeyCols;
  if (pl.h_cnt[1] > 0) {
    auto kern = k32 ? spgemm_bin1<MODE, V, true> : spgemm_bin1<MODE, V, false>;
    TACOGB_LAUNCH("spgemm_bin1", st,
                  (kern<<<grid((pl.h_cnt[1] + 7) / 8, sms * 8), 256, 0, st>>>(
                      A->pos, A->crd, Av, B->pos, B->crd, Bv, rows_of(1), pl.bin_cnt + 1, Cpos,
                      pl.cnt, Ccrd, Cvals)));
  }
  if (pl.h_cnt[2] > 0) {
    auto kern = k32 ? spgemm_bin2<MODE, V, true> : spgemm_bin2<MODE, V, false>;
    TACOGB_LAUNCH("spgemm_bin2", st,
                  (kern<<<grid((pl.h_cnt[2] + 7) / 8, sms * 5), 256, 0, st>>>(
                      A->pos, A->crd, Av, B->pos, B->crd, Bv, rows_of(2), pl.bin_cnt + 2, pl.prod,
                      Cpos, pl.cnt, Ccrd, Cvals)));
  }
  if (pl.h_cnt[3] > 0) {
    const size_t smem3 = (size_t)kBin3 * (sizeof(uint64_t) + sizeof(V));
    TACOGB_CUDA_TRY(cudaFuncSetAttribute(spgemm_bin3<MODE, V>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3));
    TACOGB_LAUNCH("spgemm_bin3", st,
                  (spgemm_bin3<MODE, V><<<grid(pl.h_cnt[3], sms * 2), 256, smem3, st>>>(
                      A->pos, A->crd, Av, B->pos, B->crd, Bv, rows_of(3), pl.bin_cnt + 3, pl.prod,
                      Cpos, pl.cnt, Ccrd, Cvals)));
  }
  if (pl.h_cnt[4] > 0) {
    // dense per-slot scratch: bitmap for the pattern, stamps + accumulators for values
    const int64_t K = B->cols;
    const int slots = (int)(pl.h_cnt[4] < kDenseSlots ? pl.h_cnt[4] : kDenseSlots);
    const size_t words = (size_t)((K + 31) / 32);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t bm_bytes = al(sizeof(uint32_t) * words * slots);
    const size_t st_bytes = mode_vals<MODE>() ? al(sizeof(int32_t) * K * slots) : 0;
    const size_t acc_bytes = mode_vals<MODE>() ? al(sizeof(V) * K * slots) : 0;
    unsigned char* ws = (unsigned char*)scratch(bm_bytes + st_bytes + acc_bytes, 3);
    if (!ws) return last_code();
    uint32_t* bitmap = (uint32_t*)ws;
    int32_t* stamp = (int32_t*)(ws + bm_bytes);
    V* acc = (V*)(ws + bm_bytes + st_bytes);
    TACOGB_CUDA_TRY(cudaMemsetAsync(bitmap, 0, bm_bytes, st));
    if (mode_vals<MODE>()) TACOGB_CUDA_TRY(cudaMemsetAsync(stamp, 0xFF, st_bytes, st));
    TACOGB_LAUNCH("spgemm_bin4", st,
                  (spgemm_bin4<MODE, V><<<slots, 256, 0, st>>>(
                      A->pos, A->crd, Av, B->pos, B->crd, Bv, rows_of(4), pl.bin_cnt + 4,
                      (int32_t)K, bitmap, mode_vals<MODE>() ? stamp : nullptr,
                      mode_vals<MODE>() ? acc : nullptr,
                      Cpos, pl.cnt, Ccrd, Cvals)));
  }
  return 0;
}

// Product counts (int64) as int32 for the scan of the one-pass slot offsets (values beyond
// int32 are clamped; the scan then flags the overflow).
__global__ void spgemm_prod32(const int64_t* __restrict__ prod, int32_t n, int32_t* __restrict__ p32) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p32[i] = (int32_t)min(prod[i], (int64_t)INT32_MAX);
}

// Moves row i's slot [off[i], off[i] + cnt[i]) to [Cpos[i], Cpos[i+1]) of C; one warp per row.
template <typename V>
__global__ void spgemm_compact(const int32_t* __restrict__ off, const int32_t* __restrict__ Cpos,
                               int32_t n, const int32_t* __restrict__ scrd,
                               const V* __restrict__ svals, int32_t* __restrict__ Ccrd,
                               V* __restrict__ Cvals) {
  const int lane = threadIdx.x & 31;
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int32_t s0 = __ldg(off + row), d0 = __ldg(Cpos + row);
    const int32_t len = __ldg(Cpos + row + 1) - d0;
    for (int32_t e = lane; e < len; e += 32) {
      Ccrd[d0 + e] = scrd[s0 + e];
      Cvals[d0 + e] = svals[s0 + e];
    }
  }
}

// Exclusive scan of cnt[0..n) into pos[0..n] (pos[n] = total); *total and the overflow flag
// are read back (synchronises).
// Exclusive scan of cnt[0, n) into pos[0, n] (pos[n] = the total) on st, without waiting; the
// total is left at sums[nblocks] and its int32 overflow flag at *flag.
int scan_counts_launch(const int32_t* cnt, int64_t n, int64_t* sums, int32_t* flag, int32_t* pos,
                       cudaStream_t st, int64_t* nblocks_out) {
  const int64_t nblocks = (n + kScanChunk - 1) / kScanChunk;
  *nblocks_out = nblocks;
  TACOGB_LAUNCH("spgemm_scan_sums", st,
                scan_block_sums<<<(unsigned)nblocks, 256, 0, st>>>(cnt, (int32_t)n, sums));
  TACOGB_LAUNCH("spgemm_scan_top", st,
                scan_sums_exclusive<<<1, 32, 0, st>>>(sums, (int32_t)nblocks, flag));
  TACOGB_LAUNCH("spgemm_scan_pos", st,
                scan_write_pos<<<(unsigned)nblocks, 256, 0, st>>>(cnt, (int32_t)n, sums, pos));
  return 0;
}

// The same, then waits and reads the total and the overflow flag.
int scan_counts(const int32_t* cnt, int64_t n, int64_t* sums, int32_t* flag, int32_t* pos,
                int64_t* total, bool* overflow, cudaStream_t st) {
  int64_t nblocks = 0;
  if (int rc = scan_counts_launch(cnt, n, sums, flag, pos, st, &nblocks)) return rc;
  return publish_and_wait(nullptr, 0, sums + nblocks, flag, nullptr, total, overflow, st);
}

// State of the last one-pass product on this device, between spgemm_onepass and
// spgemm_onepass_finish (library scratch slots 12: offsets, 13: slots; the counts live in the
// plan's scratch, slot 2).
struct OnePassState {
  int32_t* off = nullptr;   // slot offsets, n + 1
  int32_t* cnt = nullptr;   // unique columns per row, n + 1
  int32_t* scrd = nullptr;  // slot columns, total products
  void* svals = nullptr;    // slot values, total products
  int64_t n = -1;
  int vtype = 0;
};
OnePassState g_onepass[64];

int check_pair(const tacogb_csr* A, const tacogb_csr* B) {
  TACOGB_CHECK_ARG(A != nullptr && B != nullptr, "SpGEMM: null matrix");
  TACOGB_CHECK_ARG(A->cols == B->rows, "SpGEMM: A has %d columns, B has %d rows", A->cols,
                   B->rows);
  TACOGB_CHECK_ARG(A->rows >= 0 && B->cols >= 0, "SpGEMM: negative size");
  TACOGB_CHECK_ARG(A->rows == 0 || A->pos != nullptr, "SpGEMM: null A pos");
  TACOGB_CHECK_ARG(B->rows == 0 || B->pos != nullptr, "SpGEMM: null B pos");
  TACOGB_CHECK_ARG(A->nnz <= INT32_MAX && B->nnz <= INT32_MAX, "SpGEMM: nnz exceeds int32");
  return 0;
}

}  // namespace

int spgemm_symbolic(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos, int64_t* nnzC,
                    cudaStream_t st) {
  if (int rc = check_pair(A, B)) return rc;
  TACOGB_CHECK_ARG(Cpos != nullptr && nnzC != nullptr, "SpGEMM: null output");
  const int64_t n = A->rows;
  if (n == 0) {
    TACOGB_CUDA_TRY(cudaMemsetAsync(Cpos, 0, sizeof(int32_t), st));
    TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
    *nnzC = 0;
    return 0;
  }
  Plan pl;
  if (int rc = make_plan(A, B, pl, st)) return rc;
  if (int rc = run_bins<0, double>(A, B, pl, nullptr, nullptr, nullptr, st)) return rc;
  const int64_t nblocks = (n + kScanChunk - 1) / kScanChunk;
  TACOGB_LAUNCH("spgemm_scan_sums", st,
                scan_block_sums<<<(unsigned)nblocks, 256, 0, st>>>(pl.cnt, (int32_t)n, pl.sums));
  TACOGB_LAUNCH("spgemm_scan_top", st,
                scan_sums_exclusive<<<1, 32, 0, st>>>(pl.sums, (int32_t)nblocks, pl.flag));
  TACOGB_LAUNCH("spgemm_scan_pos", st,
                scan_write_pos<<<(unsigned)nblocks, 256, 0, st>>>(pl.cnt, (int32_t)n, pl.sums,
                                                                  Cpos));
  int64_t total = 0;
  int32_t flag = 0;
  TACOGB_CUDA_TRY(cudaMemcpyAsync(&total, pl.sums + nblocks, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaMemcpyAsync(&flag, pl.flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (flag) {
    set_error(TACOGB_ERR_OVERFLOW, "SpGEMM: nnz(C) = %lld exceeds int32 positions",
              (long long)total);
    return TACOGB_ERR_OVERFLOW;
  }
  *nnzC = total;
  return 0;
}

int spgemm_onepass(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos, int64_t* nnzC,
                   cudaStream_t st) {
  if (int rc = check_pair(A, B)) return rc;
  TACOGB_CHECK_ARG(Cpos != nullptr && nnzC != nullptr, "SpGEMM: null output");
  TACOGB_CHECK_ARG(A->vtype == B->vtype && (A->vtype == TACOGB_F64 || A->vtype == TACOGB_F32),
                   "SpGEMM: A and B need the same value type (F64 or F32)");
  TACOGB_CHECK_ARG(A->nnz == 0 || A->vals != nullptr, "SpGEMM: null A values");
  TACOGB_CHECK_ARG(B->nnz == 0 || B->vals != nullptr, "SpGEMM: null B values");
  int dev = 0;
  TACOGB_CUDA_TRY(cudaGetDevice(&dev));
  TACOGB_CHECK_ARG(dev >= 0 && dev < 64, "SpGEMM: device %d out of range", dev);
  OnePassState& os = g_onepass[dev];
  const int64_t n = A->rows;
  os.n = n;
  os.vtype = A->vtype;
  if (n == 0) {
    TACOGB_CUDA_TRY(cudaMemsetAsync(Cpos, 0, sizeof(int32_t), st));
    TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
    *nnzC = 0;
    return 0;
  }
  Plan pl;
  if (int rc = make_plan(A, B, pl, st, false)) return rc;
  // slot offsets: exclusive scan of the product counts, read back with the bin sizes (one wait)
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t vb = A->vtype == TACOGB_F64 ? 8 : 4;
  const size_t head = 2 * al(sizeof(int32_t) * (n + 1));
  unsigned char* ws = (unsigned char*)scratch(head, 12);
  if (!ws) return last_code();
  int32_t* p32 = (int32_t*)ws;
  int32_t* off = (int32_t*)(ws + al(sizeof(int32_t) * (n + 1)));
  TACOGB_LAUNCH("spgemm_prod32", st,
                spgemm_prod32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pl.prod, (int32_t)n,
                                                                            p32));
  int64_t products = 0, nblocks = 0;
  bool overflow = false;
  if (int rc = scan_counts_launch(p32, n, pl.sums, pl.flag, off, st, &nblocks)) return rc;
  if (int rc = publish_and_wait(pl.bin_cnt, kBins, pl.sums + nblocks, pl.flag, pl.h_cnt,
                                &products, &overflow, st))
    return rc;
  TACOGB_CHECK_ARG(!overflow, "SpGEMM: %lld products exceed the one-pass slots' int32 offsets; "
                   "use the symbolic/fill/numeric phases", (long long)products);
  // the slots, in a scratch slot of their own (growing it leaves the offsets alone)
  unsigned char* sl = (unsigned char*)scratch(al(4 * (size_t)products) + al(vb * (size_t)products),
                                              13);
  if (!sl) return last_code();
  os.off = off;
  os.cnt = pl.cnt;
  os.scrd = (int32_t*)sl;
  os.svals = sl + al(4 * (size_t)products);
  if (A->vtype == TACOGB_F64) {
    if (int rc = run_bins<3, double>(A, B, pl, os.off, os.scrd, (double*)os.svals, st)) return rc;
  } else {
    if (int rc = run_bins<3, float>(A, B, pl, os.off, os.scrd, (float*)os.svals, st)) return rc;
  }
  int64_t total = 0;
  if (int rc = scan_counts(pl.cnt, n, pl.sums, pl.flag, Cpos, &total, &overflow, st)) return rc;
  if (overflow) {
    set_error(TACOGB_ERR_OVERFLOW, "SpGEMM: nnz(C) = %lld exceeds int32 positions",
              (long long)total);
    return TACOGB_ERR_OVERFLOW;
  }
  *nnzC = total;
  return 0;
}

int spgemm_onepass_finish(const int32_t* Cpos, int32_t* Ccrd, void* Cvals, cudaStream_t st) {
  int dev = 0;
  TACOGB_CUDA_TRY(cudaGetDevice(&dev));
  TACOGB_CHECK_ARG(dev >= 0 && dev < 64 && g_onepass[dev].n >= 0,
                   "SpGEMM: no one-pass product to finish on this device");
  const OnePassState& os = g_onepass[dev];
  if (os.n == 0) return 0;
  const unsigned blocks = (unsigned)std::min<int64_t>((os.n + 7) / 8, (int64_t)sm_count() * 16);
  if (os.vtype == TACOGB_F64)
    TACOGB_LAUNCH("spgemm_compact", st,
                  spgemm_compact<double><<<blocks, 256, 0, st>>>(
                      os.off, Cpos, (int32_t)os.n, os.scrd, (const double*)os.svals, Ccrd,
                      (double*)Cvals));
  else
    TACOGB_LAUNCH("spgemm_compact", st,
                  spgemm_compact<float><<<blocks, 256, 0, st>>>(
                      os.off, Cpos, (int32_t)os.n, os.scrd, (const float*)os.svals, Ccrd,
                      (float*)Cvals));
  return 0;
}

int spgemm_fill(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos, int32_t* Ccrd,
                cudaStream_t st) {
  if (int rc = check_pair(A, B)) return rc;
  if (A->rows == 0) return 0;
  Plan pl;
  if (int rc = make_plan(A, B, pl, st)) return rc;
  return run_bins<1, double>(A, B, pl, Cpos, Ccrd, nullptr, st);
}

int spgemm_numeric(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos,
                   const int32_t* Ccrd, void* Cvals, cudaStream_t st) {
  if (int rc = check_pair(A, B)) return rc;
  TACOGB_CHECK_ARG(A->vtype == B->vtype && (A->vtype == TACOGB_F64 || A->vtype == TACOGB_F32),
                   "SpGEMM: A and B need the same value type (F64 or F32)");
  if (A->rows == 0) return 0;
  TACOGB_CHECK_ARG(A->nnz == 0 || A->vals != nullptr, "SpGEMM: null A values");
  TACOGB_CHECK_ARG(B->nnz == 0 || B->vals != nullptr, "SpGEMM: null B values");
  Plan pl;
  if (int rc = make_plan(A, B, pl, st)) return rc;
  if (A->vtype == TACOGB_F64)
    return run_bins<2, double>(A, B, pl, Cpos, const_cast<int32_t*>(Ccrd), (double*)Cvals, st);
  return run_bins<2, float>(A, B, pl, Cpos, const_cast<int32_t*>(Ccrd), (float*)Cvals, st);
}

}  // namespace tacogb
