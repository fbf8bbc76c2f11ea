// Random-gather throughput probe: the ceiling that bounds SpMV on matrices with scattered
// columns.  Every thread gathers eight 8-byte entries at a time from a table of 16-byte rows
// (one L2 sector per gather, as an x gather of a random-column SpMV), with a chosen load form
// and a chosen amount of shared memory held per SM (which sets how much L1 remains).  The
// caller times the launch; bench.py --workload gather_probe reports gathers per clock per SM.
// Built into its own library (libtacogb_probe.so, include/taco_gb300_probe.h), which only the
// benchmark loads: it is a measurement, not part of libtacogb.

#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "taco_gb300_probe.h"

namespace tacogb {

namespace {

constexpr int kProbeBlocksPerSm = 4;
constexpr int kProbeThreads = 256;
constexpr int kProbeU = 8;  // independent gathers in flight per thread

template <int MODE>
__device__ __forceinline__ double probe_load(const double* p) {
  double v;
  if constexpr (MODE == 0) {
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
  } else if constexpr (MODE == 1) {
    asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(p));
  } else {
    asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  }
  return v;
}

template <int MODE>
__global__ void __launch_bounds__(kProbeThreads)
probe_gather_kernel(const double* __restrict__ table, int32_t rows, const int32_t* __restrict__ idx,
                    int64_t n, double* __restrict__ out) {
  extern __shared__ double held[];  // reserved only: sets the shared-memory configuration
  double s = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * kProbeU;
  for (int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kProbeU; b + kProbeU <= n;
       b += stride) {
    int32_t r[kProbeU];
#pragma unroll
    for (int u = 0; u < kProbeU; u++)
      r[u] = min(max(__ldg(idx + b + u), 0), rows - 1);  // inside the table for any index
    double g[kProbeU];
#pragma unroll
    for (int u = 0; u < kProbeU; u++) g[u] = probe_load<MODE>(table + 2 * r[u]);
#pragma unroll
    for (int u = 0; u < kProbeU; u++) s += g[u];
  }
  if (s == 0.5) held[threadIdx.x] = s;  // keeps the reservation; never taken for the test data
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---- bounded-wait self-test --------------------------------------------------------------
//
// Every TMA-staged kernel of the library waits for its copies with mbar_wait_or_flag: a bounded
// poll that, when it gives up, sets the timeout bit of the device status word, waits once more
// (again bounded) so that no copy still writes shared memory when the CTA exits, and returns.
// This kernel makes that wait run out without any fault: one CTA announces extra bytes more
// than its one bulk copy brings, so the mbarrier phase can never complete.  It then copies what
// landed in shared memory to out, with the wait's verdict in the last int4, so the caller can
// check that the copy itself completed.
constexpr int kWaitBytes = 4096;

__global__ void __launch_bounds__(32)
probe_wait_timeout_kernel(const int4* __restrict__ src, int4* __restrict__ out,
                          int* __restrict__ status, uint32_t extra) {
  __shared__ __align__(128) int4 buf[kWaitBytes / 16];
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncwarp();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, kWaitBytes + extra);
    tma_load_bulk(buf, src, kWaitBytes, &bar);
  }
  __syncwarp();
  const bool ok = mbar_wait_or_flag(&bar, 0, status);
  __syncwarp();
  for (int i = threadIdx.x; i < kWaitBytes / 16; i += 32) out[i] = buf[i];
  if (threadIdx.x == 0) out[kWaitBytes / 16] = make_int4(ok ? 1 : 0, 0, 0, 0);
}

}  // namespace

}  // namespace tacogb

extern "C" int tacogb_probe_wait_timeout(const void* src, void* out, int32_t extra_bytes,
                                         void* stream) {
  using namespace tacogb;
  TACOGB_CHECK_ARG(src != nullptr && out != nullptr, "wait probe: null pointer");
  TACOGB_CHECK_ARG(((uintptr_t)src & 15) == 0 && ((uintptr_t)out & 15) == 0,
                   "wait probe: src and out must be 16-byte aligned");
  TACOGB_CHECK_ARG(extra_bytes >= 0 && extra_bytes <= 4096 && extra_bytes % 16 == 0,
                   "wait probe: extra_bytes %d is not a multiple of 16 in [0, 4096]", extra_bytes);
  int* status = device_status();
  if (!status) return last_code();
  const cudaStream_t st = (cudaStream_t)stream;
  TACOGB_LAUNCH("probe_wait_timeout_kernel", st,
                probe_wait_timeout_kernel<<<1, 32, 0, st>>>((const int4*)src, (int4*)out, status,
                                                            (uint32_t)extra_bytes));
  return 0;
}

extern "C" int tacogb_probe_gather(const double* table, int64_t rows, const int32_t* idx,
                                   int64_t n, double* out, int64_t out_len, int32_t mode,
                                   int32_t smem_kb_per_sm, int32_t carveout, void* stream) {
  using namespace tacogb;
  TACOGB_CHECK_ARG(table != nullptr && idx != nullptr && out != nullptr, "probe: null pointer");
  TACOGB_CHECK_ARG(rows > 0 && rows <= INT32_MAX && n >= 0, "probe: bad sizes");
  TACOGB_CHECK_ARG(mode >= 0 && mode <= 2, "probe: mode %d is not 0, 1 or 2", mode);
  TACOGB_CHECK_ARG(smem_kb_per_sm >= 0 && smem_kb_per_sm <= 220, "probe: shared memory %d KB",
                   smem_kb_per_sm);
  TACOGB_CHECK_ARG(carveout >= -1 && carveout <= 100, "probe: carveout %d", carveout);
  const int grid = sm_count() * kProbeBlocksPerSm;
  TACOGB_CHECK_ARG(out_len >= (int64_t)grid * kProbeThreads, "probe: out needs %lld entries",
                   (long long)grid * kProbeThreads);
  // the kernel writes held[threadIdx.x] only on a path the test data never takes; reserve at
  // least one entry per thread so that even that path stays in bounds
  const int smem = std::max(smem_kb_per_sm * 1024 / kProbeBlocksPerSm,
                            (int)(kProbeThreads * sizeof(double)));
  const cudaStream_t st = (cudaStream_t)stream;
  auto launch = [&](auto kern) -> int {
    TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    TACOGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         carveout));
    TACOGB_LAUNCH("probe_gather_kernel", st,
                  kern<<<grid, kProbeThreads, smem, st>>>(table, (int32_t)rows, idx, n, out));
    return 0;
  };
  if (mode == 0) return launch(probe_gather_kernel<0>);
  if (mode == 1) return launch(probe_gather_kernel<1>);
  return launch(probe_gather_kernel<2>);
}
