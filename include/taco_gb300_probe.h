/* libtacogb_probe — measurement and self-test probes used by bench.py and the tests; not part
 * of libtacogb.
 *
 * It measures the random-gather ceiling that bounds an SpMV over scattered columns (bench.py
 * reports the SpMV kernel's gather rate against it) and holds a self-test of the bounded
 * device-side waits that the failure-detection tests drive.  No counterpart in taco.
 */
#ifndef TACO_GB300_PROBE_H
#define TACO_GB300_PROBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Random-gather throughput probe.  Launches 4 blocks of 256 threads per SM on `stream`; each thread gathers entries table[2 * idx[i]] (rows of 16 bytes,
 * idx clamped into [0, rows)) eight at a time with load form `mode` (0 ld.global.nc,
 * 1 ld.global.cg, 2 ld.global.nc.L1::no_allocate) while every block holds
 * smem_kb_per_sm / 4 KB of shared memory; carveout is the preferred shared-memory carveout in
 * percent (-1: the driver's choice).  out needs 1024 * SMs entries.  The caller times it. */
int tacogb_probe_gather(const double* table, int64_t rows, const int32_t* idx, int64_t n,
                        double* out, int64_t out_len, int32_t mode, int32_t smem_kb_per_sm,
                        int32_t carveout, void* stream);

/* Self-test of the bounded device-side waits (no counterpart in taco).  One CTA copies 4096
 * bytes from src (device, 16-byte aligned) into shared memory with a bulk copy whose mbarrier
 * was told to expect 4096 + extra_bytes bytes, waits with the same bounded wait the library's
 * TMA-staged kernels use, and writes the shared-memory contents to out (4096 bytes) followed by
 * one int4 whose first int is 1 when the wait completed and 0 when it gave up.  With
 * extra_bytes > 0 (a multiple of 16, at most 4096) the wait cannot complete: it gives up after
 * its poll limit (about 0.1 s), sets the timeout bit of the device status word
 * (tacogb_device_status, TACOGB_ERR_TIMEOUT from the next taco-ABI call) and waits once more,
 * bounded, before the CTA exits.  Stream-ordered; the caller synchronises. */
int tacogb_probe_wait_timeout(const void* src, void* out, int32_t extra_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TACO_GB300_PROBE_H */
