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

#define TACOGB_LAUNCH(name, st, ...)                                                    \
  do {                                                                                  \
    ::tacogb::prof_before(name, st);                                                    \
    __VA_ARGS__;                                                                        \
    ::tacogb::prof_after(st);                                                           \
    if (int _rc = ::tacogb::launch_check(name)) return _rc;                             \
  } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

// Grow-only device scratch arena, one per device, used by kernels that need temporary global
// memory (partition tables, carry-outs, bin lists, scan partials).  Grown outside any graph
// capture; calls on one device are serialised by the caller's stream order.
void* scratch(size_t bytes, int slot);

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

}  // namespace tacogb
