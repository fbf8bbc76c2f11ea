// Internal entry points shared between the translation units of libtacogb.
#pragma once

#include <cuda_runtime.h>
#include "taco_gb300.h"

namespace tacogb {

// SpMV (spmv.cu)
int spmv_variant_count();
const char* spmv_variant_name(int v);
int spmv_default_variant(const tacogb_csr* A);
int spmv_run(const tacogb_csr* A, const void* x, void* y, int variant, cudaStream_t st);

}  // namespace tacogb
