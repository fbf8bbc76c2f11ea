// Index-level validation at the taco-ABI boundary (validate.cu).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace tacogb {

// True unless tacogb_set_validation(0) turned the checks off.
bool validation_on();

// Checks one compressed level on the GPU (pos and crd device-accessible): pos[0] == 0, pos
// non-decreasing and within [0, nnz], pos[outer] == nnz, 0 <= crd < inner, crd strictly
// increasing within each segment.  Synchronises st; TACOGB_ERR_ARG with a message on failure.
int validate_level_device(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
                          const int32_t* crd, int64_t nnz, cudaStream_t st);

// One level's check around a call's staging: begin() records the level as the caller passed it;
// finish() checks the device copies dpos/dcrd the kernels will read (validate_level_device), or,
// when the staging failed (dpos null) and the level is host-resident, checks it on the host so
// that invalid input is reported before the staging error.  Call finish() before returning any
// error of the staging in between.
class LevelCheck {
 public:
  void begin(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
             const int32_t* crd, int64_t nnz, bool host_resident);
  int finish(cudaStream_t st, const void* dpos, const void* dcrd);

 private:
  const char* what_ = "";
  int64_t outer_ = 0, nnz_ = 0;
  int32_t inner_ = 0;
  const int32_t* pos_ = nullptr;
  const int32_t* crd_ = nullptr;
  bool active_ = false, host_ = false;
};

}  // namespace tacogb
