// Shared definitions for the sm_103a kernels and the C-ABI layer of libtacogb.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "taco_gb300.h"

namespace tacogb {

// Error reporting: every entry point returns an int status (0 = success, as taco's generated
// functions do, src/codegen/codegen_c.cpp:591-630) and leaves a message retrievable through
// tacogb_last_error().  Nothing in the library exits the process.
void set_error(int code, const char* fmt, ...);
int last_code();

#define TACOGB_CUDA_TRY(expr)                                                           \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) {                                                            \
      ::tacogb::set_error(TACOGB_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,              \
                          cudaGetErrorString(_e), __FILE__, __LINE__);                  \
      return TACOGB_ERR_CUDA;                                                           \
    }                                                                                   \
  } while (0)

#define TACOGB_CHECK_ARG(cond, ...)                                                     \
  do {                                                                                  \
    if (!(cond)) {                                                                      \
      ::tacogb::set_error(TACOGB_ERR_ARG, __VA_ARGS__);                                 \
      return TACOGB_ERR_ARG;                                                            \
    }                                                                                   \
  } while (0)

inline int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(TACOGB_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
    return TACOGB_ERR_CUDA;
  }
  return 0;
}

// Launch accounting.  Every kernel launch of the library goes through TACOGB_LAUNCH, which
// counts it and, while profiling is on (tacogb_profile_begin/end), brackets it with CUDA events
// on its own stream so that per-kernel device time is measured where the kernel runs.
void prof_before(const char* name, cudaStream_t st);
void prof_after(cudaStream_t st);
// Counts a launch without touching the profiling events (for paths that must not allocate).
void count_launch();

#define TACOGB_LAUNCH(name, st, ...)                                                    \
  do {                                                                                  \
    ::tacogb::prof_before(name, st);                                                    \
    __VA_ARGS__;                                                                        \
    ::tacogb::prof_after(st);                                                           \
    if (int _rc = ::tacogb::launch_check(name)) return _rc;                             \
  } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

// Shared-memory carveout (percent of the maximum) for kernels that gather at random while
// holding staged tiles in shared memory.  Every outstanding gather miss holds L1 capacity: on
// GB300 random 8-byte gathers run at ~0.88 per clock per SM with a 60 KB L1 but at ~0.41 with
// the 28 KB left by the largest carveout, which the driver picks by default whenever it lets
// one more block fit.  Each kernel family passes the percentage measured best for it (-1 keeps
// the driver's choice); TACOGB_SMEM_CARVEOUT, when set, overrides it for every family.
int gather_carveout_pct(int pct);
inline cudaError_t set_gather_carveout(const void* kern, int pct) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                              gather_carveout_pct(pct));
}

// Grow-only device scratch arena, one per device, used by kernels that need temporary global
// memory (partition tables, carry-outs, bin lists, scan partials).  Grown outside any graph
// capture; calls on one device are serialised by the caller's stream order.
void* scratch(size_t bytes, int slot);

// Per-device status word (device memory, zero when healthy).  Kernels that wait on an mbarrier
// or a flag set bit TACOGB_DEV_TIMEOUT when a bounded wait gives up; the taco-ABI entry points
// check it after synchronising, tacogb_device_status() reads and clears it.
constexpr int TACOGB_DEV_TIMEOUT = 1;
int* device_status();
// Per-device mailbox of kMailboxWords 64-bit words in mapped pinned host memory (the device
// address; the same address reads on the host under unified addressing).  Kernels publish
// small results there with plain stores, so the host reads them after a stream synchronisation
// without a device -> host copy queued behind large copies on the copy engines.
// Words 0..59: published index checks (validate.cu); 64..71: SpGEMM's bin sizes and totals;
// the last two: the SpMV longest-row and locality counts.
constexpr int kMailboxWords = 80;
constexpr int kMailboxSpgemm = 64;
constexpr int kMailboxLocality = kMailboxWords - 1;
constexpr int kMailboxRowLen = kMailboxWords - 2;
unsigned long long* host_mailbox();
// Word of the same zero-initialised 256-byte block holding the double-float SpMV's x-range
// flag (set by its prep kernel, cleared by its fix-up kernel).
constexpr int kXFlagWord = 16;
// Word of the same block holding the double-float SpMM's B-range flag (set by its B-split
// kernel, cleared by its fix-up kernel).
constexpr int kBFlagWord = 17;
// Word of the same block holding the double-float SDDMM's D-range flag (cleared before, set by
// its transpose kernel).
constexpr int kDFlagWord = 18;
// Word of the same block holding the fused MTTKRP's D-range flag (cleared before its split).
constexpr int kMFlagWord = 19;
// Word of the same block holding the pipelined SpMM's B-range flag (cleared before its one
// split of B, read by every chunk's product).
constexpr int kPFlagWord = 20;

// ---------------------------------------------------------------- TMA / mbarrier ----------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Ends the life of a completed mbarrier so that its word can be initialised again (a persistent
// CTA re-stages into the same shared memory for every tile).
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Arrive on `bar` and announce `bytes` of asynchronous copies that will complete on it.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bulk (non-tensor) TMA copy global -> this CTA's shared memory, completing on `bar`.
// dst, src 16-byte aligned; bytes a positive multiple of 16.
__device__ __forceinline__ void tma_load_bulk(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Longest a bounded wait polls before it gives up (the library's copies land in microseconds).
constexpr uint64_t kWaitLimitNs = 200ull * 1000 * 1000;

// Waits for phase `phase` of `bar`; false once about limit_ns of wall time (read from the
// global timer every 16 polls, the first reading taken only after 16 failed polls) or
// 2^22 polls have passed, whichever comes first.  try_wait may suspend the thread for a
// system-dependent time per poll; the time check bounds the total whatever that time is.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase,
                                                  uint64_t limit_ns = kWaitLimitNs) {
  uint64_t t0 = 0;
  for (uint32_t it = 0; it < (1u << 22); it++) {
    if (mbar_try_wait(bar, phase)) return true;
    if ((it & 15) == 15) {
      const uint64_t now = globaltimer_ns();
      if (t0 == 0)
        t0 = now;
      else if (now - t0 > limit_ns)
        return false;
    }
    if (it > 64) __nanosleep(64);
  }
  return false;
}

// Waits for the copies of `bar`; on timeout records TACOGB_DEV_TIMEOUT and waits once more
// (again bounded) so that no copy is still writing this CTA's shared memory when it exits.
__device__ __forceinline__ bool mbar_wait_or_flag(uint64_t* bar, uint32_t phase, int* status) {
  if (mbar_wait_bounded(bar, phase)) return true;
  atomicOr(status, TACOGB_DEV_TIMEOUT);
  mbar_wait_bounded(bar, phase);
  return false;
}

// ---------------------------------------------------------------- device helpers ---------

__device__ __forceinline__ double ldg_f64(const double* p) { return __ldg(p); }

__device__ __forceinline__ int32_t ld_stream_i32(const int32_t* p) {
  int32_t v;
  asm volatile("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_stream_f64(const double* p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_stream_f32(const float* p) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// Error-free transformations (Knuth TwoSum, FMA-based TwoProduct) for the compensated FP32
// accumulation: s + e == a + b exactly, p + e == a * b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Compensated accumulator: value hi + lo, kept with |lo| small relative to |hi|.
struct CompF32 {
  float hi, lo;
  __device__ __forceinline__ void zero() { hi = 0.f; lo = 0.f; }
  __device__ __forceinline__ void add_prod(float a, float b) {
    float p, ep, s, es;
    two_prod(a, b, p, ep);
    two_sum(hi, p, s, es);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(es, ep));
  }
  __device__ __forceinline__ void add(const CompF32& o) {
    float s, es;
    two_sum(hi, o.hi, s, es);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(es, o.lo));
  }
  __device__ __forceinline__ float result() const { return __fadd_rn(hi, lo); }
};

// ---------------------------------------------------------------- warp row search ----------

// Row of nonzero p: the last r in [0, rows) with pos[r] <= p (pos[rows] > p).  32-ary search,
// one ballot per level: about log32(rows) dependent loads.
__device__ __forceinline__ int warp_find_row(const int32_t* __restrict__ pos, int32_t rows,
                                             int32_t p, int lane) {
  int lo = 0;
  int len = rows;
  while (len > 1) {
    const int step = (len + 31) >> 5;
    const int64_t off = (int64_t)lane * step;
    const bool ok = off < len && __ldg(pos + lo + off) <= p;
    const unsigned b = __ballot_sync(0xffffffffu, ok);  // a prefix of lanes; lane 0 always set
    const int L = 31 - __clz(b);
    const int nlo = lo + L * step;
    len = min(step, lo + len - nlo);
    lo = nlo;
  }
  return lo;
}

// Each lane's row for its nonzero p, given lo with pos[lo] <= every lane's p: lane m reads the
// row start pos[lo + 1 + m], each lane counts the starts <= its p by a five-step search over
// the lanes' sorted values, and lanes past 32 rows (runs of empty rows) go round again.
__device__ __forceinline__ int warp_batch_rows(const int32_t* __restrict__ pos, int32_t rows,
                                               int lo, int32_t p, int lane) {
  int r = lo;
  bool done = false;
  for (;;) {
    const int q = lo + 1 + lane;
    const int s = q <= rows ? __ldg(pos + q) : INT32_MAX;
    int c = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int v = __shfl_sync(0xffffffffu, s, c + step - 1);
      if (v <= p) c += step;
    }
    if (__shfl_sync(0xffffffffu, s, 31) <= p) c = 32;
    if (!done && c < 32) {
      r = lo + c;
      done = true;
    }
    if (__all_sync(0xffffffffu, done)) break;
    lo += 32;
  }
  return r;
}

}  // namespace tacogb
