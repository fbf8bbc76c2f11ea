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

// The same check in one launch without synchronising (the pipelined products, deferred checks):
// level_check_enqueue checks a level (device arrays) on st and publishes its five totals into
// the host mailbox set `box_index` (< kMaxPublishedChecks); with `gate`, a level that fails is
// rewritten into a harmless one in the same launch (pos becomes 0, ..., 0, nnz and crd all 0,
// which every kernel reads in bounds; needs inner >= 1 when nnz > 0), so a kernel launched
// after it on st never gathers through a bad index.  level_verdict reads a published set after
// st has been synchronised: 0, or TACOGB_ERR_ARG with a message whose segment and position are
// offset by seg_base and pos_base (the level's place in the whole operand).
constexpr int kMaxPublishedChecks = 12;
int level_check_enqueue(int64_t outer, int32_t inner, int32_t* pos, int32_t* crd, int64_t nnz,
                        int box_index, bool gate, cudaStream_t st);
int level_verdict(const char* what, int index, int64_t seg_base, int64_t pos_base);

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
  // The check without waiting for the host, for a level held in the library's own staging
  // buffers (rewritable): checked and, when it fails, made harmless on the device in one launch
  // (level_check_enqueue with gate), so the kernels launched after it on st may run; verdict()
  // after the caller's last synchronisation of st reports it (TACOGB_ERR_ARG with the first
  // fault; the result's contents are then unspecified).  A level in the caller's memory (not
  // rewritable), or one with nonzeros but no columns, is checked as finish() does.
  int finish_deferred(cudaStream_t st, void* dpos, void* dcrd, bool rewritable);
  int verdict();

 private:
  const char* what_ = "";
  int64_t outer_ = 0, nnz_ = 0;
  int32_t inner_ = 0;
  const int32_t* pos_ = nullptr;
  const int32_t* crd_ = nullptr;
  bool active_ = false, host_ = false, pending_ = false;
};

}  // namespace tacogb
