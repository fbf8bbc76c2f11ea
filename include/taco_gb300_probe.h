/* libtacogb_probe — a measurement probe used by bench.py, not part of libtacogb.
 *
 * It measures the random-gather ceiling that bounds an SpMV over scattered columns; bench.py
 * reports the SpMV kernel's gather rate against it.  No counterpart in taco.
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

#ifdef __cplusplus
}
#endif

#endif /* TACO_GB300_PROBE_H */
