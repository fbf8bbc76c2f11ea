// Validation of compressed index levels (pos, crd) at the taco-ABI boundary.
//
// taco's pack builds pos and crd that are valid by construction (src/tensor.cpp:295-463: sort,
// then the generated pack appends sorted, distinct coordinates), and its generated kernels trust
// them.  A caller of this C ABI hands over arrays that nothing has checked, and a corrupt crd
// here becomes an out-of-bounds gather on the GPU.  So before any kernel that gathers through a
// level runs, the level is checked for
//   pos[0] == 0,  pos non-decreasing,  pos[outer] == nnz (when nnz is known separately),
//   0 <= crd[p] < inner,  crd strictly increasing within each segment [pos[i], pos[i+1]),
// and a violation returns TACOGB_ERR_ARG with the first offending index.
//
// The check runs on the GPU, on the arrays the kernels will read (the caller's device or managed
// arrays, or the staged copies of host arrays): one streaming kernel that reads pos and crd
// once, in bounds (crd at [0, nnz) only, pos at [0, outer]), then one synchronisation to read
// the verdict before any gathering kernel is launched.  A check is one launch that also
// publishes its verdict into mapped host memory, so it issues no copies: in the pipelined
// products it runs between large copies in flight on the copy engines and does not queue
// behind them.  When a call cannot reach a GPU at all,
// host-resident levels are checked on the host instead, so that invalid input is still reported
// as TACOGB_ERR_ARG rather than as the missing device; tacogb_validate_level_host exposes that
// host check (multi-threaded for large levels).
// Sortedness on the GPU: a descent (crd[p] <= crd[p-1]) is legal only where p starts a
// non-empty segment, so the kernel counts all descents and the descents at segment starts; the
// two counts agree exactly when every segment is sorted.

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "threads.h"
#include "validate.h"

namespace tacogb {

namespace {

std::atomic<int> g_validate{1};

enum : unsigned {
  kBadPos0 = 1,      // pos[0] != 0
  kBadPosOrder = 2,  // pos decreases
  kBadCrdRange = 4,  // crd outside [0, inner)
  kBadCrdOrder = 8,  // crd not strictly increasing within a segment
  kBadPosEnd = 16,   // pos[outer] != nnz, or pos outside [0, nnz]
};

void describe(unsigned bits, int64_t at_pos, int64_t at_crd, const char* what, char* msg,
              size_t cap) {
  if (bits & kBadPos0)
    snprintf(msg, cap, "%s: pos[0] is not 0", what);
  else if (bits & kBadPosOrder)
    snprintf(msg, cap, "%s: pos decreases at segment %lld", what, (long long)at_pos);
  else if (bits & kBadPosEnd)
    snprintf(msg, cap, "%s: pos leaves [0, nnz] at segment %lld", what, (long long)at_pos);
  else if (bits & kBadCrdRange)
    snprintf(msg, cap, "%s: crd out of range at position %lld", what, (long long)at_crd);
  else if (at_crd >= 0)
    snprintf(msg, cap, "%s: crd not strictly increasing within a segment at position %lld",
             what, (long long)at_crd);
  else
    snprintf(msg, cap, "%s: crd not strictly increasing within a segment", what);
}

// Host check of segments [s0, s1): first offending segment / position per kind.
struct HostPart {
  unsigned bits = 0;
  int64_t at_pos = INT64_MAX, at_crd = INT64_MAX;
};

void host_check_range(int64_t s0, int64_t s1, int32_t inner, const int32_t* pos,
                      const int32_t* crd, int64_t nnz, HostPart& r) {
  for (int64_t i = s0; i < s1; i++) {
    const int64_t a = pos[i], b = pos[i + 1];
    if (b < a) {
      r.bits |= kBadPosOrder;
      r.at_pos = std::min(r.at_pos, i);
      continue;
    }
    if (a < 0 || b > nnz) {
      r.bits |= kBadPosEnd;
      r.at_pos = std::min(r.at_pos, i);
      continue;
    }
    if (!crd) continue;
    int32_t prev = -1;
    for (int64_t p = a; p < b; p++) {
      const int32_t c = crd[p];
      if (c < 0 || c >= inner) {
        r.bits |= kBadCrdRange;
        r.at_crd = std::min(r.at_crd, p);
        break;
      }
      if (c <= prev) {
        r.bits |= kBadCrdOrder;
        r.at_crd = std::min(r.at_crd, p);
        break;
      }
      prev = c;
    }
  }
}

int host_threads(int64_t work) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  if (work < (1 << 20)) return 1;
  return (int)std::min<unsigned>(hw, 32);
}

// The whole host check; threads take chunks of segments from a shared counter.
int host_check(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
               const int32_t* crd, int64_t nnz, char* msg, size_t cap) {
  if (pos[0] != 0) {
    describe(kBadPos0, 0, 0, what, msg, cap);
    return TACOGB_ERR_ARG;
  }
  if ((int64_t)pos[outer] != nnz) {
    describe(kBadPosEnd, outer, 0, what, msg, cap);
    return TACOGB_ERR_ARG;
  }
  const int nt = host_threads(outer + nnz);
  const int64_t chunks = std::max<int64_t>(1, std::min<int64_t>(outer, (int64_t)nt * 16));
  const int64_t per = (outer + chunks - 1) / std::max<int64_t>(chunks, 1);
  std::vector<HostPart> parts(nt);
  std::atomic<int64_t> next{0};
  auto worker = [&](int t) {
    if (t > 0) spread_thread();
    for (;;) {
      const int64_t k = next.fetch_add(1);
      if (k >= chunks) break;
      const int64_t s0 = k * per, s1 = std::min(outer, s0 + per);
      if (s0 < s1) host_check_range(s0, s1, inner, pos, crd, nnz, parts[t]);
    }
  };
  if (nt == 1) {
    worker(0);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) th.emplace_back(worker, t);
    for (auto& x : th) x.join();
  }
  HostPart all;
  for (auto& p : parts) {
    all.bits |= p.bits;
    all.at_pos = std::min(all.at_pos, p.at_pos);
    all.at_crd = std::min(all.at_crd, p.at_crd);
  }
  if (all.bits) {
    describe(all.bits, all.at_pos, all.at_crd, what, msg, cap);
    return TACOGB_ERR_ARG;
  }
  return 0;
}

// Running totals of one check: bits, first bad segment, first bad position, descents, descents
// at the starts of non-empty segments, and the count of blocks done.  Initialised once per
// device; the last block of every check puts them back.
struct CheckState {
  unsigned long long bits, bad_seg, bad_p, desc, desc_start;
  unsigned int done;
};
constexpr CheckState kCheckInit{0, ~0ull, ~0ull, 0, 0, 0u};

// One check of a level in one launch.  Every block folds its part into the totals (one atomic
// per warp and total); the last block to finish publishes the totals into the host mailbox
// (box[0..4], plain stores to mapped host memory), rewrites the level into a harmless one when
// `gate` is set and the totals show a violation (pos = 0, ..., 0, nnz; crd = 0), and restores
// the totals for the next check.  Plain loads: the last block may write what all blocks read.
__global__ void level_check_fused(int64_t outer, int32_t inner, int32_t* pos, int32_t* crd,
                                  int64_t nnz, CheckState* cs, volatile unsigned long long* box,
                                  int gate) {
  unsigned bits = 0;
  unsigned long long bad_seg = ~0ull, bad_p = ~0ull, desc = 0, desc_start = 0;
  const int64_t n = std::max<int64_t>(std::max(outer, nnz), 1);  // thread 0 reads pos[0]
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    if (k == 0 && pos[0] != 0) bits |= kBadPos0;
    if (k < outer) {
      const int64_t a = pos[k], b = pos[k + 1];
      if (b < a) {
        bits |= kBadPosOrder;
        bad_seg = min(bad_seg, (unsigned long long)k);
      } else if (a < 0 || b > nnz) {
        bits |= kBadPosEnd;
        bad_seg = min(bad_seg, (unsigned long long)k);
      } else if (crd && a < b && a > 0) {
        desc_start += crd[a] <= crd[a - 1];
      }
    }
    if (k < nnz && crd) {
      const int32_t c = crd[k];
      if (c < 0 || c >= inner) {
        bits |= kBadCrdRange;
        bad_p = min(bad_p, (unsigned long long)k);
      }
      if (k > 0) desc += c <= crd[k - 1];
    }
  }
  const unsigned lane = threadIdx.x & 31;
  bits = __reduce_or_sync(0xffffffffu, bits);
  for (int o = 16; o; o >>= 1) {
    bad_seg = min(bad_seg, __shfl_xor_sync(0xffffffffu, bad_seg, o));
    bad_p = min(bad_p, __shfl_xor_sync(0xffffffffu, bad_p, o));
    desc += __shfl_xor_sync(0xffffffffu, desc, o);
    desc_start += __shfl_xor_sync(0xffffffffu, desc_start, o);
  }
  if (lane == 0) {
    if (bits) atomicOr(&cs->bits, (unsigned long long)bits);
    if (bad_seg != ~0ull) atomicMin(&cs->bad_seg, bad_seg);
    if (bad_p != ~0ull) atomicMin(&cs->bad_p, bad_p);
    if (desc) atomicAdd(&cs->desc, desc);
    if (desc_start) atomicAdd(&cs->desc_start, desc_start);
  }
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this block's totals before its count
    last = atomicAdd(&cs->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  volatile CheckState* v = cs;
  const unsigned long long tb = v->bits, ts = v->bad_seg, tp = v->bad_p, td = v->desc,
                           tds = v->desc_start;
  if (gate && (tb != 0 || td != tds)) {
    const int64_t m = std::max(outer + 1, nnz);
    for (int64_t k = threadIdx.x; k < m; k += blockDim.x) {
      if (k <= outer) pos[k] = k == outer ? (int32_t)nnz : 0;
      if (k < nnz && crd) crd[k] = 0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    box[0] = tb;
    box[1] = ts;
    box[2] = tp;
    box[3] = td;
    box[4] = tds;
    v->bits = kCheckInit.bits;
    v->bad_seg = kCheckInit.bad_seg;
    v->bad_p = kCheckInit.bad_p;
    v->desc = kCheckInit.desc;
    v->desc_start = kCheckInit.desc_start;
    __threadfence();
    v->done = 0u;
    __threadfence_system();
  }
}

std::mutex g_state_mu;
CheckState* g_state[64] = {};

// This device's check totals (allocated and initialised on first use), or null.
CheckState* check_state() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    set_error(TACOGB_ERR_CUDA, "validate: no current device");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_state_mu);
  if (!g_state[dev]) {
    CheckState* p = nullptr;
    if (cudaMalloc(&p, sizeof(CheckState)) != cudaSuccess ||
        cudaMemcpy(p, &kCheckInit, sizeof(CheckState), cudaMemcpyHostToDevice) != cudaSuccess) {
      if (p) cudaFree(p);
      set_error(TACOGB_ERR_ALLOC, "validate: check state allocation failed");
      return nullptr;
    }
    g_state[dev] = p;
  }
  return g_state[dev];
}

}  // namespace

bool validation_on() { return g_validate.load(std::memory_order_relaxed) != 0; }

static_assert(5 * kMaxPublishedChecks <= kMailboxRowLen, "published checks fit the mailbox");

int level_check_enqueue(int64_t outer, int32_t inner, int32_t* pos, int32_t* crd, int64_t nnz,
                        int box_index, bool gate, cudaStream_t st) {
  TACOGB_CHECK_ARG(box_index >= 0 && box_index < kMaxPublishedChecks, "validate: check %d",
                   box_index);
  TACOGB_CHECK_ARG(pos != nullptr, "validate: null pos");
  TACOGB_CHECK_ARG(!gate || inner > 0 || nnz == 0, "validate: no columns to gate nonzeros to");
  CheckState* cs = check_state();
  if (!cs) return last_code();
  unsigned long long* box = host_mailbox();
  if (!box) return last_code();
  const int64_t n = std::max<int64_t>(std::max(outer, nnz), 1);
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
  TACOGB_LAUNCH("level_check_fused", st,
                level_check_fused<<<(unsigned)blocks, 256, 0, st>>>(
                    outer, inner, pos, crd, nnz, cs, box + 5 * box_index, gate ? 1 : 0));
  return 0;
}

int level_verdict(const char* what, int index, int64_t seg_base, int64_t pos_base) {
  volatile unsigned long long* box = host_mailbox();
  if (!box) return last_code();
  unsigned long long h[5];
  for (int i = 0; i < 5; i++) h[i] = box[5 * index + i];
  unsigned bits = (unsigned)h[0];
  if (!(bits & (kBadPosOrder | kBadPosEnd)) && h[3] != h[4]) bits |= kBadCrdOrder;
  if (bits) {
    // the kernel locates range errors; an order error is known from the two counts only
    char msg[256];
    describe(bits, seg_base + (int64_t)h[1],
             (bits & kBadCrdRange) ? pos_base + (int64_t)h[2] : -1, what, msg, sizeof(msg));
    set_error(TACOGB_ERR_ARG, "%s", msg);
    return TACOGB_ERR_ARG;
  }
  return 0;
}

int validate_level_device(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
                          const int32_t* crd, int64_t nnz, cudaStream_t st) {
  if (outer <= 0 && nnz <= 0) return 0;
  TACOGB_CHECK_ARG(pos != nullptr, "%s: null pos", what);
  // read only (no gate)
  if (int rc = level_check_enqueue(outer, inner, const_cast<int32_t*>(pos),
                                   const_cast<int32_t*>(crd), nnz, 0, false, st))
    return rc;
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return level_verdict(what, 0, 0, 0);
}

void LevelCheck::begin(const char* what, int64_t outer, int32_t inner, const int32_t* pos,
                       const int32_t* crd, int64_t nnz, bool host_resident) {
  what_ = what;
  outer_ = outer;
  inner_ = inner;
  pos_ = pos;
  crd_ = crd;
  nnz_ = nnz;
  active_ = validation_on() && (outer > 0 || nnz > 0);
  host_ = host_resident;
}

int LevelCheck::finish_deferred(cudaStream_t st, void* dpos, void* dcrd, bool rewritable) {
  if (!active_) return 0;
  if (!rewritable || dpos == nullptr || (inner_ <= 0 && nnz_ > 0)) return finish(st, dpos, dcrd);
  active_ = false;
  if (int rc = level_check_enqueue(outer_, inner_, (int32_t*)dpos, (int32_t*)dcrd, nnz_, 0, true,
                                   st))
    return rc;
  pending_ = true;
  return 0;
}

int LevelCheck::verdict() {
  if (!pending_) return 0;
  pending_ = false;
  return level_verdict(what_, 0, 0, 0);
}

int LevelCheck::finish(cudaStream_t st, const void* dpos, const void* dcrd) {
  if (!active_) return 0;
  active_ = false;
  if (dpos)
    return validate_level_device(what_, outer_, inner_, (const int32_t*)dpos,
                                 (const int32_t*)dcrd, nnz_, st);
  if (!host_ || !pos_) return 0;  // nothing reached the GPU: the staging error is reported
  char msg[256];
  const int rc = host_check(what_, outer_, inner_, pos_, crd_, nnz_, msg, sizeof(msg));
  if (rc) set_error(rc, "%s", msg);
  return rc;
}

}  // namespace tacogb

using namespace tacogb;

extern "C" {

int tacogb_set_validation(int32_t on) {
  return g_validate.exchange(on ? 1 : 0);
}

int tacogb_validate_level_host(int64_t outer, int32_t inner, const int32_t* pos,
                               const int32_t* crd, int64_t nnz) {
  TACOGB_CHECK_ARG(outer >= 0 && inner >= 0 && nnz >= 0, "validate: negative size");
  if (outer == 0 && nnz == 0) return 0;
  TACOGB_CHECK_ARG(pos != nullptr && (nnz == 0 || crd != nullptr), "validate: null pos or crd");
  char msg[256];
  const int rc = host_check("level", outer, inner, pos, crd, nnz, msg, sizeof(msg));
  if (rc) set_error(rc, "%s", msg);
  return rc;
}

int tacogb_csr_validate(const tacogb_csr* A, void* stream) {
  TACOGB_CHECK_ARG(A != nullptr, "validate: null matrix");
  TACOGB_CHECK_ARG(A->rows >= 0 && A->cols >= 0 && A->nnz >= 0, "validate: negative size");
  return validate_level_device("CSR matrix", A->rows, A->cols, A->pos, A->crd, A->nnz,
                               (cudaStream_t)stream);
}

}  // extern "C"
