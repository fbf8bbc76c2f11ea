// Order-3 kernels over a CSF tensor B ({Sparse,Sparse,Sparse} or {Dense,Sparse,Sparse}):
//   TTV     A(i,j)   = B(i,j,k) * c(k)
//   TTM     A(i,j,l) = B(i,j,k) * C(k,l)
//   MTTKRP  A(i,j)   = B(i,k,l) * C(k,j) * D(l,j)
// taco's statements and schedules: test/tests-scheduling-eval.cpp:993-1206 (CPU), 1420-1580
// (GPU, scheduleTTVGPU / scheduleTTMGPU / scheduleMTTKRPGPU at :288-343).
//
// B's last level is a CSR matrix whose rows are B's fibers: pos2 over nfib fibers, crd2 the
// last coordinate.  So TTV is SpMV and TTM is SpMM over that fiber matrix (the library's
// merge-tile kernels, load-balanced over nonzeros however long the fibers are), each giving
// one value or one dense row per (i,j) fiber; dense results (taco's test form) are zero-filled
// and the fiber results scattered to (i, j).  MTTKRP factors the sum over l inside the sum over
// k: T(f,:) = sum_l B(i,k,l) D(l,:) per level-1 fiber f = (i,k) (SpMM over the fiber matrix),
// then A(i,:) = sum_f C(k_f,:) * T(f,:) over the fibers of i (t3_mttkrp_combine): 2J flops per
// nonzero plus 2J per fiber, where taco's loop spends 3J per nonzero.  TTM and MTTKRP take the
// SpMM variant of the fiber product; for FP64 MTTKRP variant -2 selects the fused kernel
// (t3_mttkrp_fused), which never writes the fiber rows but measured slower (5.41 against 4.28 ms
// on the nell-2-shaped tensor, J = 32: 60 warp-instructions per nonzero against the SpMM's 45).
#include <cstdint>
#include <cstring>

#include "common.cuh"
#include "df.cuh"
#include "kernels.h"

namespace tacogb {

namespace {

// dest[f] = i_f * dims1 + j_f for every fiber f: its level-0 entry e by a binary search over
// pos1 (the last e with pos1[e] <= f), i = crd0[e] (or e itself for a dense level 0).
__global__ void t3_fiber_dest(const int32_t* __restrict__ pos1, const int32_t* __restrict__ crd0,
                              const int32_t* __restrict__ crd1, int32_t n0, int32_t nfib,
                              int32_t dims1, int64_t* __restrict__ dest) {
  const int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfib) return;
  int lo = 0, hi = n0 - 1;  // pos1[0] = 0 <= f < pos1[n0]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pos1 + mid) <= f)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int64_t i = crd0 ? __ldg(crd0 + lo) : lo;
  dest[f] = i * dims1 + __ldg(crd1 + f);
}

template <class V>
__global__ void t3_scatter_vals(const int64_t* __restrict__ dest, const V* __restrict__ y,
                                int32_t nfib, V* __restrict__ A) {
  const int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < nfib) A[dest[f]] = y[f];
}

// A[dest[f] * L + l] = Y[f * L + l]: one thread per element, rows copied whole by consecutive
// threads.
template <class V>
__global__ void t3_scatter_rows(const int64_t* __restrict__ dest, const V* __restrict__ Y,
                                int32_t nfib, int32_t L, V* __restrict__ A) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nfib * L) return;
  const int64_t f = idx / L;
  const int32_t l = (int32_t)(idx - f * L);
  A[dest[f] * L + l] = Y[idx];
}

constexpr int kCombFibers = 64;  // fibers per warp in t3_mttkrp_combine

// A(i,:) += C(crd1[f],:) * T(f,:) for the fibers f of one chunk of 64: one warp per chunk, lanes
// over j, the C and T rows of eight fibers loaded together; each run of fibers of one i is
// summed in registers and added to A(i,:) with one atomic add per lane (A zero-filled first).
// Chunks balance the work however many fibers an i has; an i whose fibers straddle chunks
// receives several adds, in no fixed order (taco's GPU schedule for this statement also uses
// atomics, OutputRaceStrategy::Atomics at test/tests-scheduling-eval.cpp:342).
template <class V>
__global__ void t3_mttkrp_combine(const int32_t* __restrict__ pos1,
                                  const int32_t* __restrict__ crd0,
                                  const int32_t* __restrict__ crd1, int32_t n0, int32_t nfib,
                                  int32_t J, const V* __restrict__ C, const V* __restrict__ T,
                                  V* __restrict__ A) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t f0 = w * kCombFibers;
  if (f0 >= nfib) return;
  const int32_t f1 = (int32_t)min(f0 + kCombFibers, (int64_t)nfib);
  int e0 = 0, hi = n0 - 1;  // the level-0 entry of f0: last e with pos1[e] <= f0
  while (e0 < hi) {
    const int mid = (e0 + hi + 1) >> 1;
    if (__ldg(pos1 + mid) <= f0)
      e0 = mid;
    else
      hi = mid - 1;
  }
  for (int32_t j0 = 0; j0 < J; j0 += 32) {
    const int32_t j = j0 + lane;
    const bool on = j < J;
    int e = e0;
    int32_t nx = __ldg(pos1 + e + 1);
    V acc = V(0);
    for (int32_t fb = (int32_t)f0; fb < f1; fb += 8) {
      const int kq = (lane < 8 && fb + lane < f1) ? __ldg(crd1 + fb + lane) : 0;
      V cv[8], tv[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int k = __shfl_sync(0xffffffffu, kq, q);
        const bool ld = on && fb + q < f1;
        cv[q] = ld ? __ldg(C + (int64_t)k * J + j) : V(0);
        tv[q] = ld ? __ldg(T + (int64_t)(fb + q) * J + j) : V(0);
      }
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int32_t f = fb + q;
        if (f >= f1) break;
        while (f >= nx) {  // the fibers of entry e end here (warp-uniform)
          if (on) atomicAdd(A + (crd0 ? (int64_t)__ldg(crd0 + e) : (int64_t)e) * J + j, acc);
          acc = V(0);
          e++;
          nx = __ldg(pos1 + e + 1);
        }
        acc = fma(cv[q], tv[q], acc);
      }
    }
    if (on) atomicAdd(A + (crd0 ? (int64_t)__ldg(crd0 + e) : (int64_t)e) * J + j, acc);
  }
}

constexpr int kMttkrpFused = -2;  // the variant number of the fused FP64 kernel
constexpr int kFuWarps = 8;
constexpr int kFuNnz = 256;  // nonzeros per warp in t3_mttkrp_fused

// Ds[l * J + j] = D(l, j) as double-float pairs; *flag set when an entry is outside the pairs'
// range (the fused kernel then takes those batches natively).
__global__ void t3_split_d(const double* __restrict__ D, DF* __restrict__ Ds, int64_t n,
                           int* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DF r;
  if (!split_df(D[i], r.h, r.l)) *flag = 1;
  Ds[i] = r;
}

// Fused MTTKRP over 256 consecutive nonzeros per warp (balanced however long the fibers are):
// lanes over j (32 columns per pass), per nonzero the product B * D(l, j) accumulated in
// double-float on the FP32 pipe (12 instructions per term; a batch with a value outside the
// pairs' range runs in native FP64 into a second accumulator), at each fiber end the fiber's sum
// times C(k, j) added to the row sum of i in FP64, and at each change of i (and at the end of
// the chunk) that row sum added into A(i, j) atomically.  Replaces the fiber SpMM, its scratch
// T (nfib x J) and the combine; each nonzero costs a broadcast of its value and column, one
// 8-byte load of D per lane from L2 and the product.
__global__ void __launch_bounds__(kFuWarps * 32) t3_mttkrp_fused(
    const int32_t* __restrict__ pos1, const int32_t* __restrict__ crd0,
    const int32_t* __restrict__ crd1, const int32_t* __restrict__ pos2,
    const int32_t* __restrict__ crd2, const double* __restrict__ vals, int32_t n0, int32_t nfib,
    int64_t nnz, int32_t J, const double* __restrict__ C, const double* __restrict__ D,
    const DF* __restrict__ Ds, const int* __restrict__ dflag, double* __restrict__ A) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t p0 = ((int64_t)blockIdx.x * kFuWarps + (threadIdx.x >> 5)) * kFuNnz;
  if (p0 >= nnz) return;
  const int64_t pend = min(p0 + (int64_t)kFuNnz, nnz);
  const bool dok = *dflag == 0;
  const int f_first = warp_find_row(pos2, nfib, (int32_t)p0, lane);
  const int e_first = warp_find_row(pos1, n0, f_first, lane);
  for (int32_t j0 = 0; j0 < J; j0 += 32) {
    const int32_t j = j0 + lane;
    const bool on = j < J;
    int lo = f_first;        // fiber search base for the next batch
    int cf = f_first;        // current fiber
    int e = e_first;         // its level-0 entry
    int32_t e_end = __ldg(pos1 + e + 1);
    double ck = on ? __ldg(C + (int64_t)__ldg(crd1 + cf) * J + j) : 0.0;
    // the fiber's double-float sum in two interleaved (hi, unnormalised compensation) pairs, so
    // that consecutive terms do not wait on each other; nat: its natively summed part
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
    double nat = 0.0;
    double rowsum = 0.0;  // sum over i's fibers so far of C(k, j) * fiber sum
    auto fiber_sum = [&]() {
      float s, e;
      two_sum(s0, s1, s, e);
      const float c = __fadd_rn(__fadd_rn(c0, c1), e);
      DF t;
      two_sum(s, c, t.h, t.l);
      return __dadd_rn(df_to_double(t), nat);
    };
    for (int64_t base = p0; base < pend; base += 32) {
      const int32_t pl = (int32_t)min(base + lane, pend - 1);
      const int32_t lreg = __ldg(crd2 + pl);
      const double vreg = __ldg(vals + pl);
      const int freg = warp_batch_rows(pos2, nfib, lo, pl, lane);
      lo = __shfl_sync(full, freg, 31);
      const int fprev = __shfl_up_sync(full, freg, 1);
      const unsigned fchg =  // nonzeros that open a new fiber
          __ballot_sync(full, base + lane < pend && freg != (lane == 0 ? cf : fprev));
      DF vs;
      const bool ok = __all_sync(full, split_df(vreg, vs.h, vs.l)) && dok;
      const int cnt = (int)min((int64_t)32, pend - base);
      for (int n0b = 0; n0b < cnt; n0b += 8) {
        DF d[8];
        double dn[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int l = __shfl_sync(full, lreg, n0b + q);
          if (ok) {
            d[q] = on ? Ds[(int64_t)l * J + j] : DF{0.f, 0.f};
          } else {
            dn[q] = on ? __ldg(D + (int64_t)l * J + j) : 0.0;
          }
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int n = n0b + q;
          if (n >= cnt) break;
          if ((fchg >> n) & 1u) {  // fiber cf ends here (warp-uniform)
            rowsum = __fma_rn(ck, fiber_sum(), rowsum);
            s0 = c0 = s1 = c1 = 0.f;
            nat = 0.0;
            const int f = __shfl_sync(full, freg, n);
            while (f >= e_end) {  // entry e ends too
              if (on) atomicAdd(A + (crd0 ? (int64_t)__ldg(crd0 + e) : (int64_t)e) * J + j, rowsum);
              rowsum = 0.0;
              e++;
              e_end = __ldg(pos1 + e + 1);
            }
            cf = f;
            ck = on ? __ldg(C + (int64_t)__ldg(crd1 + cf) * J + j) : 0.0;
          }
          if (ok) {
            const float vh = __shfl_sync(full, vs.h, n), vl = __shfl_sync(full, vs.l, n);
            float& s = (q & 1) ? s1 : s0;
            float& c = (q & 1) ? c1 : c0;
            const float ph = __fmul_rn(vh, d[q].h);
            const float pe = __fmaf_rn(vh, d[q].h, -ph);
            float cc = __fmaf_rn(vh, d[q].l, c);
            cc = __fmaf_rn(vl, d[q].h, cc);
            float sn, er;
            two_sum(s, ph, sn, er);
            c = __fadd_rn(cc, __fadd_rn(pe, er));
            s = sn;
          } else {
            nat = __fma_rn(__shfl_sync(full, vreg, n), dn[q], nat);
          }
        }
        float t0, t1;  // renormalise once per eight terms
        two_sum(s0, c0, t0, t1);
        s0 = t0;
        c0 = t1;
        two_sum(s1, c1, t0, t1);
        s1 = t0;
        c1 = t1;
      }
    }
    rowsum = __fma_rn(ck, fiber_sum(), rowsum);
    if (on) atomicAdd(A + (crd0 ? (int64_t)__ldg(crd0 + e) : (int64_t)e) * J + j, rowsum);
  }
}

int check_csf3(const tacogb_csf3* B, const char* what) {
  TACOGB_CHECK_ARG(B != nullptr, "%s: null tensor", what);
  TACOGB_CHECK_ARG(B->dims[0] >= 0 && B->dims[1] >= 0 && B->dims[2] >= 0 && B->n0 >= 0 &&
                       B->nfib >= 0 && B->nnz >= 0,
                   "%s: negative size", what);
  TACOGB_CHECK_ARG(B->nnz <= INT32_MAX, "%s: nnz exceeds int32 positions", what);
  TACOGB_CHECK_ARG(B->crd0 != nullptr || B->n0 == B->dims[0] || B->n0 == 0,
                   "%s: a dense first level has dims[0] entries", what);
  TACOGB_CHECK_ARG(B->n0 == 0 || (B->pos1 != nullptr), "%s: null pos1", what);
  TACOGB_CHECK_ARG(B->nfib == 0 || (B->crd1 != nullptr && B->pos2 != nullptr),
                   "%s: null level-1 crd or level-2 pos", what);
  TACOGB_CHECK_ARG(B->nnz == 0 || (B->crd2 != nullptr && B->vals != nullptr),
                   "%s: null level-2 crd or values", what);
  TACOGB_CHECK_ARG(B->vtype == TACOGB_F64 || B->vtype == TACOGB_F32,
                   "%s: unsupported value type %d", what, B->vtype);
  return 0;
}

size_t vsize(int vt) { return vt == TACOGB_F64 ? 8 : 4; }

// The fiber matrix: rows are B's (i,j) fibers, columns B's last coordinate.
tacogb_csr fiber_csr(const tacogb_csf3* B) {
  return tacogb_csr{B->nfib, B->dims[2], B->nnz, B->pos2, B->crd2, B->vals, B->vtype};
}

// dest of every fiber, written at ws (nfib int64 values).
int fiber_dest(const tacogb_csf3* B, unsigned char* ws, cudaStream_t st, int64_t*& dest) {
  dest = reinterpret_cast<int64_t*>(ws);
  if (B->nfib == 0) return 0;
  TACOGB_LAUNCH("t3_fiber_dest", st,
                (t3_fiber_dest<<<(unsigned)((B->nfib + 255) / 256), 256, 0, st>>>(
                    B->pos1, B->crd0, B->crd1, B->n0, B->nfib, B->dims[1], dest)));
  return 0;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int ttv_run(const tacogb_csf3* B, const void* c, void* out, bool dense, int variant,
            cudaStream_t st) {
  if (int rc = check_csf3(B, "TTV")) return rc;
  const size_t vb = vsize(B->vtype);
  TACOGB_CHECK_ARG(B->nnz == 0 || c != nullptr, "TTV: null c");
  if (dense) {
    const size_t abytes = (size_t)B->dims[0] * (size_t)B->dims[1] * vb;
    TACOGB_CHECK_ARG(abytes == 0 || out != nullptr, "TTV: null result");
    if (abytes) TACOGB_CUDA_TRY(cudaMemsetAsync(out, 0, abytes, st));
    if (B->nfib == 0) return 0;
    unsigned char* ws = (unsigned char*)scratch(
        align256((size_t)B->nfib * 8) + align256((size_t)B->nfib * vb), 7);
    if (!ws) return last_code();
    int64_t* dest;
    if (int rc = fiber_dest(B, ws, st, dest)) return rc;
    void* y = ws + align256((size_t)B->nfib * 8);
    const tacogb_csr f = fiber_csr(B);
    if (int rc = spmv_run(&f, c, y, variant, st)) return rc;
    if (B->vtype == TACOGB_F64)
      TACOGB_LAUNCH("t3_scatter_vals", st,
                    (t3_scatter_vals<double><<<(unsigned)((B->nfib + 255) / 256), 256, 0, st>>>(
                        dest, (const double*)y, B->nfib, (double*)out)));
    else
      TACOGB_LAUNCH("t3_scatter_vals", st,
                    (t3_scatter_vals<float><<<(unsigned)((B->nfib + 255) / 256), 256, 0, st>>>(
                        dest, (const float*)y, B->nfib, (float*)out)));
    return 0;
  }
  TACOGB_CHECK_ARG(B->nfib == 0 || out != nullptr, "TTV: null result");
  if (B->nfib == 0) return 0;
  const tacogb_csr f = fiber_csr(B);
  return spmv_run(&f, c, out, variant, st);
}

int ttm_run(const tacogb_csf3* B, int32_t L, const void* C, void* out, bool dense, int variant,
            cudaStream_t st) {
  if (int rc = check_csf3(B, "TTM")) return rc;
  TACOGB_CHECK_ARG(L >= 0, "TTM: negative L");
  TACOGB_CHECK_ARG(B->nnz == 0 || L == 0 || C != nullptr, "TTM: null C");
  const size_t vb = vsize(B->vtype);
  if (!dense) {
    TACOGB_CHECK_ARG((int64_t)B->nfib * L == 0 || out != nullptr, "TTM: null result");
    if ((int64_t)B->nfib * L == 0) return 0;
    const tacogb_csr f = fiber_csr(B);
    return spmm_run(&f, L, C, B->vtype, out, variant, st);
  }
  const size_t abytes = (size_t)B->dims[0] * (size_t)B->dims[1] * (size_t)L * vb;
  TACOGB_CHECK_ARG(abytes == 0 || out != nullptr, "TTM: null result");
  if (abytes) TACOGB_CUDA_TRY(cudaMemsetAsync(out, 0, abytes, st));
  if ((int64_t)B->nfib * L == 0) return 0;
  unsigned char* ws = (unsigned char*)scratch(
      align256((size_t)B->nfib * 8) + align256((size_t)B->nfib * L * vb), 7);
  if (!ws) return last_code();
  int64_t* dest;
  if (int rc = fiber_dest(B, ws, st, dest)) return rc;
  void* Y = ws + align256((size_t)B->nfib * 8);
  const tacogb_csr f = fiber_csr(B);
  if (int rc = spmm_run(&f, L, C, B->vtype, Y, variant, st)) return rc;
  const int64_t n = (int64_t)B->nfib * L;
  if (B->vtype == TACOGB_F64)
    TACOGB_LAUNCH("t3_scatter_rows", st,
                  (t3_scatter_rows<double><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                      dest, (const double*)Y, B->nfib, L, (double*)out)));
  else
    TACOGB_LAUNCH("t3_scatter_rows", st,
                  (t3_scatter_rows<float><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                      dest, (const float*)Y, B->nfib, L, (float*)out)));
  return 0;
}

int mttkrp_run(const tacogb_csf3* B, int32_t J, const void* C, const void* D, void* A,
               int variant, cudaStream_t st) {
  if (int rc = check_csf3(B, "MTTKRP")) return rc;
  TACOGB_CHECK_ARG(J >= 0, "MTTKRP: negative J");
  const size_t vb = vsize(B->vtype);
  const size_t abytes = (size_t)B->dims[0] * (size_t)J * vb;
  TACOGB_CHECK_ARG(abytes == 0 || A != nullptr, "MTTKRP: null result");
  TACOGB_CHECK_ARG(B->nnz == 0 || J == 0 || (C != nullptr && D != nullptr),
                   "MTTKRP: null C or D");
  if (abytes) TACOGB_CUDA_TRY(cudaMemsetAsync(A, 0, abytes, st));
  if ((int64_t)B->nfib * J == 0 || B->n0 == 0 || B->nnz == 0) return 0;
  if (B->vtype == TACOGB_F64 && variant == kMttkrpFused) {  // fused: no fiber rows in memory
    const int64_t nd = (int64_t)B->dims[2] * J;
    DF* Ds = (DF*)scratch(align256((size_t)nd * sizeof(DF)), 7);
    if (!Ds) return last_code();
    int* status = device_status();
    if (!status) return last_code();
    int* flag = status + kMFlagWord;
    TACOGB_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    if (nd)
      TACOGB_LAUNCH("t3_split_d", st,
                    (t3_split_d<<<(unsigned)((nd + 255) / 256), 256, 0, st>>>((const double*)D, Ds,
                                                                             nd, flag)));
    const int64_t warps = (B->nnz + kFuNnz - 1) / kFuNnz;
    TACOGB_LAUNCH("t3_mttkrp_fused", st,
                  (t3_mttkrp_fused<<<(unsigned)((warps + kFuWarps - 1) / kFuWarps), kFuWarps * 32,
                                     0, st>>>(B->pos1, B->crd0, B->crd1, B->pos2, B->crd2,
                                              (const double*)B->vals, B->n0, B->nfib, B->nnz, J,
                                              (const double*)C, (const double*)D, Ds, flag,
                                              (double*)A)));
    return 0;
  }
  void* T = scratch(align256((size_t)B->nfib * J * vb), 7);
  if (!T) return last_code();
  const tacogb_csr f = fiber_csr(B);
  // D (dims[2] x J) is small next to B and stays in L2: the streaming tile, which walks
  // nonzeros across fiber boundaries, measured fastest for the fiber product (nell-2's shape,
  // J = 32: 4.02 ms against 4.42 for the library's SpMM default)
  if (variant < 0) variant = spmm_variant_index("stream_w512_dfs");
  if (int rc = spmm_run(&f, J, D, B->vtype, T, variant, st)) return rc;
  return mttkrp_combine_launch(B, J, C, T, A, st);
}

int mttkrp_combine_launch(const tacogb_csf3* B, int32_t J, const void* C, const void* T, void* A,
                          cudaStream_t st) {
  if ((int64_t)B->nfib * J == 0 || B->n0 == 0 || B->nnz == 0) return 0;
  const int64_t threads = (((int64_t)B->nfib + kCombFibers - 1) / kCombFibers) * 32;
  if (B->vtype == TACOGB_F64)
    TACOGB_LAUNCH("t3_mttkrp_combine", st,
                  (t3_mttkrp_combine<double><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                      B->pos1, B->crd0, B->crd1, B->n0, B->nfib, J, (const double*)C,
                      (const double*)T, (double*)A)));
  else
    TACOGB_LAUNCH("t3_mttkrp_combine", st,
                  (t3_mttkrp_combine<float><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
                      B->pos1, B->crd0, B->crd1, B->n0, B->nfib, J, (const float*)C,
                      (const float*)T, (float*)A)));
  return 0;
}

}  // namespace tacogb
