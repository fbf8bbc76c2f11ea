// Index-level validation at the taco-ABI boundary (validate.cu).
#pragma once

#include <cstdint>
#include <thread>

#include <cuda_runtime.h>

namespace tacogb {

// True unless tacogb_set_validation(0) turned the checks off.
bool validation_on();

// Checks one compressed level on the GPU (pos and crd device-accessible): pos[0] == 0, pos
// non-decreasing and within [0, nnz], pos[outer] == nnz, 0 <= crd < inner, crd strictly
// increasing within each segment.  Synchronises st; TACOGB_ERR_ARG with a message on failure.
int validate_level_device(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
                          const int32_t* crd, int64_t nnz, cudaStream_t st);

// One level's check around a call's staging: begin() starts host threads on host-resident
// arrays (so the check overlaps the copies to the GPU); finish() joins them, or, when the level
// is not host-resident, runs validate_level_device on its device copies dpos/dcrd.  finish()
// reports a failed check before anything else, so call it before returning any error of the
// staging in between (dpos null skips the device check after a failed staging).
class LevelCheck {
 public:
  void begin(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
             const int32_t* crd, int64_t nnz, bool host_resident);
  int finish(cudaStream_t st, const void* dpos, const void* dcrd);
  ~LevelCheck();

 private:
  const char* what_ = "";
  int64_t outer_ = 0, nnz_ = 0;
  int32_t inner_ = 0;
  const int32_t* pos_ = nullptr;
  const int32_t* crd_ = nullptr;
  bool active_ = false, host_ = false;
  int rc_ = 0;
  char msg_[256] = "";
  std::thread worker_;
};

}  // namespace tacogb
