// SDDMM, A(i,k) = B(i,k) * C(i,j) * D(j,k): B CSR (I x K), C dense I x J, D dense J x K, the
// result sampled at B's nonzeros.  taco's statement and schedule:
// test/tests-scheduling-eval.cpp:1360-1417 (sddmmGPU) and :270-286 (scheduleSDDMMGPU); its
// CPU form :783-840.  taco's generated loop sums over j, term by term, (B*C)*D into A(i,k).
//
// GB300 layout.  D is transposed once per call into Dt (K x Jp, Jp = J padded to a multiple of
// 32*JL*CH, padding zero) so that the J values a nonzero needs are one contiguous row:
// nonzero (i,k) then reads Dt[k, :] with fully coalesced 16-byte loads, where taco's schedule
// has lanes over j read D[j,k] a row apart.  A warp owns 256 consecutive nonzeros (balanced
// however long the rows are); lanes split j, lane l holding C[i, l*JL .. l*JL+JL) (per chunk)
// in registers for as long as the row lasts.  Nonzeros go eight at a time: their eight Dt
// slices are loaded together, each lane forms eight partial dots, and a reduce-scatter of
// nine shuffles leaves every lane with one whole dot; four groups fill the warp's 32 results,
// multiplied by B's values and written with one coalesced store.
//
// The group loop is kept rolled: unrolled over a batch's four groups the body overflowed the
// instruction cache (ncu: "no instruction" the second stall reason; 6.32 -> 5.69 ms rolled).
//
// FP64 runs natively (DFMA) or in double-float on the FP32 pipe (Dt split into hi/lo float
// pairs by the transpose, C split when its row is loaded): GB300's FP64 pipe retires about
// 1.6 DFMA per clock per SM, so the 2J flops per nonzero are pipe-bound natively.  Values
// outside the pairs' range (|v| outside [2^-40, 2^40), inf, nan) are caught (a flag from the
// transpose for D, a ballot for C rows) and those groups are redone natively from C and D.
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

namespace tacogb {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSdBlock = 256;
constexpr int kSdWarps = kSdBlock / 32;
constexpr int kSdBatches = 8;  // batches of 32 nonzeros per warp
constexpr int kSdWarpNnz = 32 * kSdBatches;
constexpr int kSdSlab = 512;  // j columns per kernel pass; wider J runs slab by slab

// ------------------------------------------------------------------ value policies --------

struct Sd64 {  // FP64, native DFMA
  using V = double;
  using DT = double;
  using CR = double;
  using Acc = double;
  static constexpr bool kChecked = false;
  __device__ static CR cvt_c(double c, bool&) { return c; }
  __device__ static Acc zero() { return 0.0; }
  __device__ static void madd(Acc& a, CR c, DT d) { a = __fma_rn(c, d, a); }
  __device__ static Acc combine(Acc a, Acc b) { return __dadd_rn(a, b); }
  __device__ static Acc shfl_xor(Acc a, int m) { return __shfl_xor_sync(kFull, a, m); }
  __device__ static V fin(Acc a) { return a; }
};

struct Sd32 {  // FP32, native FFMA
  using V = float;
  using DT = float;
  using CR = float;
  using Acc = float;
  static constexpr bool kChecked = false;
  __device__ static CR cvt_c(float c, bool&) { return c; }
  __device__ static Acc zero() { return 0.f; }
  __device__ static void madd(Acc& a, CR c, DT d) { a = __fmaf_rn(c, d, a); }
  __device__ static Acc combine(Acc a, Acc b) { return __fadd_rn(a, b); }
  __device__ static Acc shfl_xor(Acc a, int m) { return __shfl_xor_sync(kFull, a, m); }
  __device__ static V fin(Acc a) { return a; }
};

// FP64 in double-float: per term one exact TwoProduct of the hi parts, two cross-term FMAs and
// a TwoSum into an unnormalised (sum, compensation) pair, about 12 FP32 instructions.
struct SdAcc {
  float s, c;
};
struct SdDFS {
  using V = double;
  using DT = DF;
  using CR = DF;
  using Acc = SdAcc;
  static constexpr bool kChecked = true;
  __device__ static CR cvt_c(double c, bool& ok) {
    DF r;
    ok &= split_df(c, r.h, r.l);
    return r;
  }
  __device__ static Acc zero() { return SdAcc{0.f, 0.f}; }
  __device__ static void madd(Acc& a, CR c, DT d) {
    const float ph = __fmul_rn(c.h, d.h);
    const float pe = __fmaf_rn(c.h, d.h, -ph);
    float cc = __fmaf_rn(c.h, d.l, a.c);
    cc = __fmaf_rn(c.l, d.h, cc);
    float s1, e;
    two_sum(a.s, ph, s1, e);
    a.c = __fadd_rn(cc, __fadd_rn(pe, e));
    a.s = s1;
  }
  __device__ static Acc combine(Acc a, Acc b) {
    float s, e;
    two_sum(a.s, b.s, s, e);
    return SdAcc{s, __fadd_rn(__fadd_rn(a.c, b.c), e)};
  }
  __device__ static Acc shfl_xor(Acc a, int m) {
    return SdAcc{__shfl_xor_sync(kFull, a.s, m), __shfl_xor_sync(kFull, a.c, m)};
  }
  __device__ static V fin(Acc a) {
    DF r;
    two_sum(a.s, a.c, r.h, r.l);
    return df_to_double(r);
  }
};

// ------------------------------------------------------------------ D transpose -----------

__device__ __forceinline__ void put_dt(double* p, double v, bool&) { *p = v; }
__device__ __forceinline__ void put_dt(float* p, float v, bool&) { *p = v; }
__device__ __forceinline__ void put_dt(DF* p, double v, bool& ok) {
  DF r;
  ok &= split_df(v, r.h, r.l);
  *p = r;
}

// Dt[k * Jp + j] = D[j * ldd + k] for j < J, zero for J <= j < Jp (DF output: split into
// double-float pairs, *flag set when a value is outside the pairs' range).  32 x 32 tiles
// through shared memory, reads coalesced along k and writes along j; grid (ceil(K/32), Jp/32),
// block (32, 8).
template <class In, class Out>
__global__ void sddmm_transpose(const In* __restrict__ D, Out* __restrict__ Dt, int32_t J,
                                int32_t K, int64_t ldd, int32_t Jp, int* __restrict__ flag) {
  __shared__ In tile[32][33];
  const int64_t k0 = (int64_t)blockIdx.x * 32;
  const int j0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int j = j0 + ty + 8 * m;
    const int64_t k = k0 + tx;
    tile[ty + 8 * m][tx] = (j < J && k < K) ? D[(int64_t)j * ldd + k] : In(0);
  }
  __syncthreads();
  bool ok = true;
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int64_t k = k0 + ty + 8 * m;
    if (k < K) put_dt(Dt + k * Jp + j0 + tx, tile[tx][ty + 8 * m], ok);
  }
  if (!ok) *flag = 1;
}

// ------------------------------------------------------------------ warp helpers ----------

// Vector load of N consecutive T (N * sizeof(T) in {4, 8, 16, 32} bytes, naturally aligned).
template <class T, int N>
__device__ __forceinline__ void ld_slice(const T* p, T (&r)[N]) {
  constexpr int B = (int)sizeof(T) * N;
  static_assert(B == 4 || B == 8 || B == 16 || B == 32, "slice width");
  if constexpr (B == 4) {
    const float u = __ldg(reinterpret_cast<const float*>(p));
    memcpy(r, &u, 4);
  } else if constexpr (B == 8) {
    const float2 u = __ldg(reinterpret_cast<const float2*>(p));
    memcpy(r, &u, 8);
  } else if constexpr (B == 16) {
    const float4 u = __ldg(reinterpret_cast<const float4*>(p));
    memcpy(r, &u, 16);
  } else {
    const float4 u0 = __ldg(reinterpret_cast<const float4*>(p));
    const float4 u1 = __ldg(reinterpret_cast<const float4*>(p) + 1);
    memcpy(r, &u0, 16);
    memcpy(reinterpret_cast<char*>(r) + 16, &u1, 16);
  }
}

// The same from shared memory.
template <class T, int N>
__device__ __forceinline__ void ld_shared_slice(const T* p, T (&r)[N]) {
  constexpr int B = (int)sizeof(T) * N;
  static_assert(B == 4 || B == 8 || B == 16 || B == 32, "slice width");
  if constexpr (std::is_same<T, double>::value) {
    if constexpr (N == 1) {
      r[0] = *p;
    } else {
#pragma unroll
      for (int i = 0; i < N / 2; i++) {
        const double2 u = reinterpret_cast<const double2*>(p)[i];
        r[2 * i] = u.x;
        r[2 * i + 1] = u.y;
      }
    }
  } else if constexpr (B == 4) {
    const float u = *reinterpret_cast<const float*>(p);
    memcpy(r, &u, 4);
  } else if constexpr (B == 8) {
    const float2 u = *reinterpret_cast<const float2*>(p);
    memcpy(r, &u, 8);
  } else if constexpr (B == 16) {
    const float4 u = *reinterpret_cast<const float4*>(p);
    memcpy(r, &u, 16);
  } else {
    const float4 u0 = reinterpret_cast<const float4*>(p)[0];
    const float4 u1 = reinterpret_cast<const float4*>(p)[1];
    memcpy(r, &u0, 16);
    memcpy(reinterpret_cast<char*>(r) + 16, &u1, 16);
  }
}

// Reduce-scatter of eight per-lane partials: lane l ends with the warp-wide sum of partial
// (l >> 2) & 7.  Halving exchanges over lane bits 4, 3, 2 (4 + 2 + 1 shuffles), then a
// butterfly over bits 1, 0.
template <class P>
__device__ __forceinline__ typename P::Acc sd_reduce8(const typename P::Acc (&v)[8], int lane) {
  using A = typename P::Acc;
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  A w[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const A keep = b4 ? v[i + 4] : v[i];
    const A send = b4 ? v[i] : v[i + 4];
    w[i] = P::combine(keep, P::shfl_xor(send, 16));
  }
  A u[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const A keep = b3 ? w[i + 2] : w[i];
    const A send = b3 ? w[i] : w[i + 2];
    u[i] = P::combine(keep, P::shfl_xor(send, 8));
  }
  A t = P::combine(b2 ? u[1] : u[0], P::shfl_xor(b2 ? u[0] : u[1], 4));
  t = P::combine(t, P::shfl_xor(t, 2));
  t = P::combine(t, P::shfl_xor(t, 1));
  return t;
}

}  // namespace

namespace {

template <class P>
struct SdArgs {
  using V = typename P::V;
  const int32_t* pos;
  const int32_t* crd;
  const V* bvals;
  const V* C;  // C[i * ldc + j] for this slab's j (offset to the slab's first column)
  int64_t ldc;
  const typename P::DT* Dt;  // K x Jp
  int32_t Jp;
  const V* D;  // D[j * ldd + k] for this slab's j (the native redo of a checked policy)
  int64_t ldd;
  int32_t Js;  // columns of j in this slab
  V* acc;      // per-nonzero partial dots across slabs (null with one slab)
  int acc_in, acc_out;
  V* out;          // nonzero values (out_ld == 0) or dense A (row stride out_ld)
  int64_t out_ld;
  int32_t rows;
  int64_t nnz;
  const int* dflag;  // checked policies: set when a D value is outside the pairs' range
};

// Native FP64 dot of group g from C and D themselves (D read a column at a time): the redo
// path of a checked policy, for groups whose values the pairs cannot carry.  Kept out of line
// so that its registers do not weigh on the main loop.
template <int JL, int CH>
__device__ __noinline__ double sd_group_native(const double* __restrict__ C, int64_t ldc,
                                               const double* __restrict__ D, int64_t ldd,
                                               int32_t Js, int kreg, int r, int g, int lane) {
  double part[8];
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int k = __shfl_sync(kFull, kreg, 8 * g + n);
    const int rn = __shfl_sync(kFull, r, 8 * g + n);
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < CH; c++)
#pragma unroll
      for (int e = 0; e < JL; e++) {
        const int j = c * 32 * JL + lane * JL + e;
        if (j < Js) s = __fma_rn(C[(int64_t)rn * ldc + j], D[(int64_t)j * ldd + k], s);
      }
    part[n] = s;
  }
  return sd_reduce8<Sd64>(part, lane);
}

// One warp: nonzeros [p0, p0 + 256) of B.  See the file comment for the scheme.
template <class P, int JL, int CH>
__global__ void __launch_bounds__(kSdBlock, 2) sddmm_kernel(const SdArgs<P> a) {
  using V = typename P::V;
  using DT = typename P::DT;
  using CR = typename P::CR;
  using Acc = typename P::Acc;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t)blockIdx.x * kSdWarps + (threadIdx.x >> 5);
  const int64_t p0 = warp * kSdWarpNnz;
  if (p0 >= a.nnz) return;
  const int64_t pend = min(p0 + (int64_t)kSdWarpNnz, a.nnz);
  bool dok = true;
  if constexpr (P::kChecked) dok = *a.dflag == 0;
  int lo = warp_find_row(a.pos, a.rows, (int32_t)p0, lane);
  int crow = -1;  // row whose C slice creg holds (CH == 1)
  CR creg[JL];
  bool cok = true;

  auto load_c = [&](int rn, int c) {
    bool ok = true;
#pragma unroll
    for (int e = 0; e < JL; e++) {
      const int j = c * 32 * JL + lane * JL + e;
      const V v = j < a.Js ? __ldg(a.C + (int64_t)rn * a.ldc + j) : V(0);
      creg[e] = P::cvt_c(v, ok);
    }
    if constexpr (P::kChecked) cok = __all_sync(kFull, ok);
  };

  for (int64_t base = p0; base < pend; base += 32) {
    const int32_t pl = (int32_t)min(base + lane, a.nnz - 1);
    const int kreg = __ldg(a.crd + pl);
    const int r = warp_batch_rows(a.pos, a.rows, lo, pl, lane);
    lo = __shfl_sync(kFull, r, 31);
    V res = V(0);
#pragma unroll 1  // one group's code: the fully unrolled batch overflows the instruction cache
    for (int g = 0; g < 4; g++) {
      if (base + 8 * g >= pend) break;
      Acc part[8];
#pragma unroll
      for (int n = 0; n < 8; n++) part[n] = P::zero();
      bool gok = dok;
      if (dok) {
#pragma unroll
        for (int c = 0; c < CH; c++) {
          DT d[8][JL];
#pragma unroll
          for (int n = 0; n < 8; n++) {
            const int k = __shfl_sync(kFull, kreg, 8 * g + n);
            ld_slice<DT, JL>(a.Dt + (int64_t)k * a.Jp + c * 32 * JL + lane * JL, d[n]);
          }
          if (CH > 1) crow = -1;
#pragma unroll
          for (int n = 0; n < 8; n++) {
            const int rn = __shfl_sync(kFull, r, 8 * g + n);
            if (rn != crow) {  // warp-uniform
              load_c(rn, c);
              crow = rn;
            }
            if constexpr (P::kChecked) gok &= cok;
#pragma unroll
            for (int e = 0; e < JL; e++) P::madd(part[n], creg[e], d[n][e]);
          }
        }
      }
      V val;
      if constexpr (P::kChecked) {
        if (gok) {
          val = P::fin(sd_reduce8<P>(part, lane));
        } else {
          val = sd_group_native<JL, CH>(a.C, a.ldc, a.D, a.ldd, a.Js, kreg, r, g, lane);
          crow = -1;
        }
      } else {
        val = P::fin(sd_reduce8<P>(part, lane));
      }
      if ((lane & 3) == g) res = val;
    }
    // lane l holds nonzero m of the batch
    const int m = 8 * (lane & 3) + ((lane >> 2) & 7);
    const int rm = __shfl_sync(kFull, r, m);
    const int km = __shfl_sync(kFull, kreg, m);
    const int64_t p = base + m;
    if (p < pend) {
      if (a.acc_in) res += a.acc[p];
      if (a.acc_out) {
        a.acc[p] = res;
      } else {
        const V v = a.bvals[p] * res;
        if (a.out_ld)
          a.out[(int64_t)rm * a.out_ld + km] = v;
        else
          a.out[p] = v;
      }
    }
  }
}

}  // namespace

namespace {

// TMA-staged form for J <= 128 (one chunk per lane): each warp keeps a ring of three stages in
// shared memory, each holding the Dt rows of a group of eight nonzeros, filled by eight 1-D
// bulk copies (one per nonzero, issued by lanes 0-7) completing on the stage's mbarrier.  The
// copies of the next two groups are in flight while a group is computed, so a warp keeps up to
// 24 KB of gathers outstanding without holding them in registers.  Per group the eight rows'
// C slices are settled first (a reload when the row changes), then the 8 x JL products run
// without branches.  Measured slower than the register form at J = 128 in FP64 (8.08 against
// 5.69 ms on the 1,048,576-row power-law B): 1 KB rows leave room for only eight warps per SM,
// too few to cover the double-float arithmetic; it stays a selectable variant.
constexpr int kStWarps = 4;
constexpr int kStStages = 3;

template <class DT, int JL>
constexpr size_t sd_tma_smem() {
  return (size_t)kStWarps * kStStages * 8 * 32 * JL * sizeof(DT) +
         (size_t)kStWarps * kStStages * sizeof(uint64_t);
}

template <class P, int JL>
__global__ void __launch_bounds__(kStWarps * 32) sddmm_tma_kernel(const SdArgs<P> a, int* status) {
  using V = typename P::V;
  using DT = typename P::DT;
  using CR = typename P::CR;
  using Acc = typename P::Acc;
  constexpr int RE = 32 * JL;  // elements of one staged Dt row
  constexpr uint32_t kGroupBytes = 8u * RE * sizeof(DT);
  extern __shared__ __align__(128) unsigned char sd_smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  DT* buf = reinterpret_cast<DT*>(sd_smem) + (size_t)w * kStStages * 8 * RE;
  uint64_t* bars =
      reinterpret_cast<uint64_t*>(sd_smem + (size_t)kStWarps * kStStages * kGroupBytes) +
      w * kStStages;
  const int64_t p0 = ((int64_t)blockIdx.x * kStWarps + w) * kSdWarpNnz;
  if (p0 >= a.nnz) return;  // per warp; the kernel has no CTA barrier
  const int64_t pend = min(p0 + (int64_t)kSdWarpNnz, a.nnz);
  const int ngroups = (int)((pend - p0 + 7) / 8);
  if (lane == 0)
    for (int s = 0; s < kStStages; s++) mbar_init(&bars[s], 1);
  __syncwarp();

  auto issue = [&](int G) {
    const int s = G % kStStages;
    if (lane == 0) mbar_arrive_expect_tx(&bars[s], kGroupBytes);
    __syncwarp();
    if (lane < 8) {
      const int64_t p = min(p0 + 8 * G + lane, a.nnz - 1);
      const int k = __ldg(a.crd + p);
      tma_load_bulk(buf + (s * 8 + lane) * RE, a.Dt + (int64_t)k * RE,
                    (uint32_t)(RE * sizeof(DT)), &bars[s]);
    }
  };
  for (int G = 0; G < kStStages && G < ngroups; G++) issue(G);

  bool dok = true;
  if constexpr (P::kChecked) dok = *a.dflag == 0;
  int lo = warp_find_row(a.pos, a.rows, (int32_t)p0, lane);
  int crow = -1;
  CR creg[JL];
  bool cok = true;
  int kreg = 0, r = 0;
  V res = V(0);
  for (int G = 0; G < ngroups; G++) {
    const int g = G & 3;
    const int64_t base = p0 + 32 * (G >> 2);
    if (g == 0) {  // a new batch of 32 nonzeros: columns and rows, one per lane
      const int32_t pl = (int32_t)min(base + lane, a.nnz - 1);
      kreg = __ldg(a.crd + pl);
      r = warp_batch_rows(a.pos, a.rows, lo, pl, lane);
      lo = __shfl_sync(kFull, r, 31);
      res = V(0);
    }
    const int s = G % kStStages;
    mbar_wait_or_flag(&bars[s], (uint32_t)((G / kStStages) & 1), status);
    const DT* st = buf + s * 8 * RE + lane * JL;
    Acc part[8];
#pragma unroll
    for (int n = 0; n < 8; n++) part[n] = P::zero();
    bool gok = dok;
    if (dok) {
      CR cn[8][JL];
#pragma unroll
      for (int n = 0; n < 8; n++) {
        const int rn = __shfl_sync(kFull, r, 8 * g + n);
        if (rn != crow) {  // warp-uniform
          bool ok = true;
#pragma unroll
          for (int e = 0; e < JL; e++) {
            const int j = lane * JL + e;
            const V v = j < a.Js ? __ldg(a.C + (int64_t)rn * a.ldc + j) : V(0);
            creg[e] = P::cvt_c(v, ok);
          }
          if constexpr (P::kChecked) cok = __all_sync(kFull, ok);
          crow = rn;
        }
        if constexpr (P::kChecked) gok &= cok;
#pragma unroll
        for (int e = 0; e < JL; e++) cn[n][e] = creg[e];
      }
      DT d[8][JL];
#pragma unroll
      for (int n = 0; n < 8; n++) ld_shared_slice<DT, JL>(st + n * RE, d[n]);
#pragma unroll
      for (int e = 0; e < JL; e++)
#pragma unroll
        for (int n = 0; n < 8; n++) P::madd(part[n], cn[n][e], d[n][e]);
    }
    __syncwarp();  // every lane has read stage s
    if (G + kStStages < ngroups) issue(G + kStStages);
    V val;
    if constexpr (P::kChecked) {
      if (gok) {
        val = P::fin(sd_reduce8<P>(part, lane));
      } else {
        val = sd_group_native<JL, 1>(a.C, a.ldc, a.D, a.ldd, a.Js, kreg, r, g, lane);
        crow = -1;
      }
    } else {
      val = P::fin(sd_reduce8<P>(part, lane));
    }
    if ((lane & 3) == g) res = val;
    if (g == 3 || G == ngroups - 1) {
      const int m = 8 * (lane & 3) + ((lane >> 2) & 7);
      const int rm = __shfl_sync(kFull, r, m);
      const int km = __shfl_sync(kFull, kreg, m);
      const int64_t p = base + m;
      if (p < pend && (m >> 3) <= g) {
        V o = res;
        if (a.acc_in) o += a.acc[p];
        if (a.acc_out) {
          a.acc[p] = o;
        } else {
          const V v = a.bvals[p] * o;
          if (a.out_ld)
            a.out[(int64_t)rm * a.out_ld + km] = v;
          else
            a.out[p] = v;
        }
      }
    }
  }
}

}  // namespace

// ------------------------------------------------------------------ host side -------------

namespace {

struct SddmmVariant {
  const char* name;
  int df;   // FP64: 0 native DFMA, 1 double-float (FP32 values always run natively)
  int tma;  // 1: TMA-staged Dt rows for J <= 128 (wider J runs the register form)
};
constexpr SddmmVariant kSddmmVariants[] = {
    {"warp_native", 0, 0}, {"warp_dfs", 1, 0}, {"tma_native", 0, 1}, {"tma_dfs", 1, 1}};
constexpr int kNumSddmmVariants = sizeof(kSddmmVariants) / sizeof(kSddmmVariants[0]);

// Per-lane slice JL and chunks CH for a slab of Js columns of j (Js <= 512).
inline void sd_shape(int32_t Js, int& JL, int& CH) {
  JL = Js <= 32 ? 1 : Js <= 64 ? 2 : 4;
  CH = Js <= 128 ? 1 : Js <= 256 ? 2 : 4;
}

template <class P, int JL, int CH>
int sd_launch(const SdArgs<P>& a, cudaStream_t st) {
  const int64_t warps = (a.nnz + kSdWarpNnz - 1) / kSdWarpNnz;
  const int64_t blocks = (warps + kSdWarps - 1) / kSdWarps;
  TACOGB_CHECK_ARG(blocks < (1ll << 31), "SDDMM: too many nonzeros");
  // no shared memory: keep the whole unified array as L1 for the Dt row gathers
  set_gather_carveout((const void*)sddmm_kernel<P, JL, CH>, 0);
  TACOGB_LAUNCH("sddmm_kernel", st,
                (sddmm_kernel<P, JL, CH><<<(unsigned)blocks, kSdBlock, 0, st>>>(a)));
  return 0;
}

template <class P, int JL>
int sd_launch_tma(const SdArgs<P>& a, cudaStream_t st) {
  const int64_t warps = (a.nnz + kSdWarpNnz - 1) / kSdWarpNnz;
  const int64_t blocks = (warps + kStWarps - 1) / kStWarps;
  TACOGB_CHECK_ARG(blocks < (1ll << 31), "SDDMM: too many nonzeros");
  constexpr size_t smem = sd_tma_smem<typename P::DT, JL>();
  const void* kern = (const void*)sddmm_tma_kernel<P, JL>;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
  int* status = device_status();
  if (!status) return last_code();
  TACOGB_LAUNCH("sddmm_tma_kernel", st,
                (sddmm_tma_kernel<P, JL><<<(unsigned)blocks, kStWarps * 32, smem, st>>>(a,
                                                                                      status)));
  return 0;
}

template <class P>
int sd_dispatch(const SdArgs<P>& a, int JL, int CH, int tma, cudaStream_t st) {
  if (tma && CH == 1) {
    if (JL == 4) return sd_launch_tma<P, 4>(a, st);
    if (JL == 2) return sd_launch_tma<P, 2>(a, st);
    return sd_launch_tma<P, 1>(a, st);
  }
  if (CH == 4) return sd_launch<P, 4, 4>(a, st);
  if (CH == 2) return sd_launch<P, 4, 2>(a, st);
  if (JL == 4) return sd_launch<P, 4, 1>(a, st);
  if (JL == 2) return sd_launch<P, 2, 1>(a, st);
  return sd_launch<P, 1, 1>(a, st);
}

// One SDDMM: per slab of up to 512 columns of j, D's slab transposed into Dt (V -> DT, split
// for the double-float policy), then the kernel; slabs after the first add into acc, the last
// multiplies by B's values and writes the result.
template <class P>
int sd_run(const tacogb_csr* B, int32_t J, const void* Cv, const void* Dv, void* outv,
           int64_t out_ld, int tma, cudaStream_t st) {
  using V = typename P::V;
  using DT = typename P::DT;
  const V* C = (const V*)Cv;
  const V* D = (const V*)Dv;
  V* out = (V*)outv;
  const int64_t nnz = B->nnz;
  const int32_t K = B->cols;
  if (out_ld > 0 && (int64_t)B->rows * K > 0)  // taco's dense result starts from zero
    TACOGB_CUDA_TRY(cudaMemset2DAsync(out, (size_t)out_ld * sizeof(V), 0, (size_t)K * sizeof(V),
                                      (size_t)B->rows, st));
  if (nnz == 0) return 0;
  if (J == 0) {  // empty sum: every sampled value is zero
    if (out_ld == 0) TACOGB_CUDA_TRY(cudaMemsetAsync(out, 0, (size_t)nnz * sizeof(V), st));
    return 0;
  }
  const int slabs = (J + kSdSlab - 1) / kSdSlab;
  int JL0, CH0;
  sd_shape(J < kSdSlab ? J : kSdSlab, JL0, CH0);
  const int32_t Jp0 = 32 * JL0 * CH0;
  const size_t dt_bytes = ((size_t)K * Jp0 * sizeof(DT) + 255) & ~(size_t)255;
  const size_t acc_bytes = slabs > 1 ? (size_t)nnz * sizeof(V) : 0;
  unsigned char* ws = (unsigned char*)scratch(dt_bytes + acc_bytes, 6);
  if (!ws) return last_code();
  DT* Dt = (DT*)ws;
  V* acc = slabs > 1 ? (V*)(ws + dt_bytes) : nullptr;
  int* dflag = nullptr;
  if constexpr (P::kChecked) {
    int* status = device_status();
    if (!status) return last_code();
    dflag = status + kDFlagWord;
  }
  for (int s = 0; s < slabs; s++) {
    const int32_t j0 = s * kSdSlab;
    const int32_t Js = J - j0 < kSdSlab ? J - j0 : kSdSlab;
    int JL, CH;
    sd_shape(Js, JL, CH);
    const int32_t Jp = 32 * JL * CH;
    if (dflag) TACOGB_CUDA_TRY(cudaMemsetAsync(dflag, 0, sizeof(int), st));
    const dim3 tgrid((unsigned)((K + 31) / 32), (unsigned)(Jp / 32));
    TACOGB_LAUNCH("sddmm_transpose", st,
                  (sddmm_transpose<V, DT><<<tgrid, dim3(32, 8), 0, st>>>(
                      D + (int64_t)j0 * K, Dt, Js, K, K, Jp, dflag)));
    SdArgs<P> a;
    a.pos = B->pos;
    a.crd = B->crd;
    a.bvals = (const V*)B->vals;
    a.C = C + j0;
    a.ldc = J;
    a.Dt = Dt;
    a.Jp = Jp;
    a.D = D + (int64_t)j0 * K;
    a.ldd = K;
    a.Js = Js;
    a.acc = acc;
    a.acc_in = s > 0;
    a.acc_out = s < slabs - 1;
    a.out = out;
    a.out_ld = out_ld;
    a.rows = B->rows;
    a.nnz = nnz;
    a.dflag = dflag;
    if (int rc = sd_dispatch<P>(a, JL, CH, tma, st)) return rc;
  }
  return 0;
}

// The two-step form: D's transpose (flag cleared, then set by any value the pairs cannot carry)
// and a product against it, one slab of j.
template <class P>
int sd_pre_transpose(const void* Dv, int32_t J, int32_t K, void* Dtv, cudaStream_t st) {
  using V = typename P::V;
  using DT = typename P::DT;
  int JL, CH;
  sd_shape(J, JL, CH);
  const int32_t Jp = 32 * JL * CH;
  int* dflag = nullptr;
  if constexpr (P::kChecked) {
    int* status = device_status();
    if (!status) return last_code();
    dflag = status + kDFlagWord;
    TACOGB_CUDA_TRY(cudaMemsetAsync(dflag, 0, sizeof(int), st));
  }
  if (K == 0) return 0;
  const dim3 tgrid((unsigned)((K + 31) / 32), (unsigned)(Jp / 32));
  TACOGB_LAUNCH("sddmm_transpose", st,
                (sddmm_transpose<V, DT><<<tgrid, dim3(32, 8), 0, st>>>(
                    (const V*)Dv, (DT*)Dtv, J, K, K, Jp, dflag)));
  return 0;
}

template <class P>
int sd_pre_run(const tacogb_csr* B, int32_t J, const void* C, const void* D, const void* Dt,
               void* out, cudaStream_t st) {
  using V = typename P::V;
  if (B->nnz == 0) return 0;
  int JL, CH;
  sd_shape(J, JL, CH);
  SdArgs<P> a;
  a.pos = B->pos;
  a.crd = B->crd;
  a.bvals = (const V*)B->vals;
  a.C = (const V*)C;
  a.ldc = J;
  a.Dt = (const typename P::DT*)Dt;
  a.Jp = 32 * JL * CH;
  a.D = (const V*)D;
  a.ldd = B->cols;
  a.Js = J;
  a.acc = nullptr;
  a.acc_in = 0;
  a.acc_out = 0;
  a.out = (V*)out;
  a.out_ld = 0;
  a.rows = B->rows;
  a.nnz = B->nnz;
  a.dflag = nullptr;
  if constexpr (P::kChecked) {
    int* status = device_status();
    if (!status) return last_code();
    a.dflag = status + kDFlagWord;
  }
  return sd_dispatch<P>(a, JL, CH, 0, st);
}

}  // namespace

size_t sddmm_pre_bytes(int32_t J, int32_t K, int vtype) {
  if (J <= 0 || J > kSdSlab || K < 0) return 0;
  int JL, CH;
  sd_shape(J, JL, CH);
  const size_t dt = vtype == TACOGB_F32 ? sizeof(float) : sizeof(DF);  // the default policies
  return ((size_t)K * (size_t)(32 * JL * CH) * dt + 255) & ~(size_t)255;
}

int sddmm_pre_transpose(const void* D, int32_t J, int32_t K, int vtype, void* Dt,
                        cudaStream_t st) {
  TACOGB_CHECK_ARG(J > 0 && J <= kSdSlab && K >= 0, "SDDMM: two-step form needs 0 < J <= %d",
                   kSdSlab);
  TACOGB_CHECK_ARG(vtype == TACOGB_F64 || vtype == TACOGB_F32, "SDDMM: unsupported value type %d",
                   vtype);
  return vtype == TACOGB_F32 ? sd_pre_transpose<Sd32>(D, J, K, Dt, st)
                             : sd_pre_transpose<SdDFS>(D, J, K, Dt, st);
}

int sddmm_pre_run(const tacogb_csr* B, int32_t J, const void* C, const void* D, const void* Dt,
                  void* out, cudaStream_t st) {
  TACOGB_CHECK_ARG(B != nullptr && B->rows >= 0 && B->cols >= 0 && B->nnz >= 0,
                   "SDDMM: bad matrix");
  TACOGB_CHECK_ARG(J > 0 && J <= kSdSlab, "SDDMM: two-step form needs 0 < J <= %d", kSdSlab);
  TACOGB_CHECK_ARG(B->vtype == TACOGB_F64 || B->vtype == TACOGB_F32,
                   "SDDMM: unsupported value type %d", B->vtype);
  TACOGB_CHECK_ARG(B->nnz == 0 || (B->pos && B->crd && B->vals && C && D && Dt && out),
                   "SDDMM: null array");
  return B->vtype == TACOGB_F32 ? sd_pre_run<Sd32>(B, J, C, D, Dt, out, st)
                                : sd_pre_run<SdDFS>(B, J, C, D, Dt, out, st);
}

int sddmm_variant_count() { return kNumSddmmVariants; }
const char* sddmm_variant_name(int v) {
  return (v >= 0 && v < kNumSddmmVariants) ? kSddmmVariants[v].name : nullptr;
}

int sddmm_run(const tacogb_csr* B, int32_t J, const void* C, const void* D, void* out,
              int64_t out_ld, int variant, cudaStream_t st) {
  TACOGB_CHECK_ARG(B != nullptr, "SDDMM: null matrix");
  TACOGB_CHECK_ARG(B->rows >= 0 && B->cols >= 0 && B->nnz >= 0 && J >= 0, "SDDMM: negative size");
  TACOGB_CHECK_ARG(B->nnz <= INT32_MAX, "SDDMM: nnz exceeds int32 positions");
  TACOGB_CHECK_ARG(B->rows == 0 || B->pos != nullptr, "SDDMM: null pos");
  TACOGB_CHECK_ARG(B->nnz == 0 || (B->crd != nullptr && B->vals != nullptr),
                   "SDDMM: null crd or values");
  TACOGB_CHECK_ARG(B->nnz == 0 || J == 0 || (C != nullptr && D != nullptr), "SDDMM: null C or D");
  TACOGB_CHECK_ARG(out_ld >= 0, "SDDMM: negative leading dimension");
  TACOGB_CHECK_ARG(out_ld == 0 || out_ld >= B->cols, "SDDMM: dense result stride %lld < %d columns",
                   (long long)out_ld, B->cols);
  TACOGB_CHECK_ARG(out != nullptr || (out_ld == 0 ? B->nnz == 0 : (int64_t)B->rows * B->cols == 0),
                   "SDDMM: null result");
  TACOGB_CHECK_ARG(B->vtype == TACOGB_F64 || B->vtype == TACOGB_F32,
                   "SDDMM: unsupported value type %d", B->vtype);
  // register form, FP64 in double-float on the FP32 pipe: measured fastest (1,048,576-row
  // power-law B, J = 128: 5.69 ms against 8.08 TMA-staged and 10.2 native DFMA)
  if (variant < 0) variant = 1;
  TACOGB_CHECK_ARG(variant < kNumSddmmVariants, "SDDMM: variant %d out of range", variant);
  const SddmmVariant& v = kSddmmVariants[variant];
  if (B->vtype == TACOGB_F32) return sd_run<Sd32>(B, J, C, D, out, out_ld, v.tma, st);
  return v.df ? sd_run<SdDFS>(B, J, C, D, out, out_ld, v.tma, st)
              : sd_run<Sd64>(B, J, C, D, out, out_ld, v.tma, st);
}

}  // namespace tacogb
