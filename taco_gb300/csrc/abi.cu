// The C-ABI layer of libtacogb: error state, per-device scratch arena, and taco's kernel ABI
// (assemble / compute / evaluate over taco_tensor_t, plus the packed _shim_ forms) forwarding to
// the device-pointer layer.
//
// taco_tensor_t handling follows what taco's generated code reads from the struct
// (src/codegen/codegen.cpp:232-350 unpack text): dimensions[m], indices[m][0]/[1] for a
// compressed mode, vals; csize is in bits (src/storage/storage.cpp:61-63).

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <initializer_list>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

#include "common.cuh"
#include "kernels.h"
#include "threads.h"
#include "validate.h"

namespace tacogb {

// ------------------------------------------------------------------ errors ----------------

namespace {
thread_local char g_err[512] = "";
thread_local int g_code = 0;
}  // namespace

void set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  g_code = code;
}
int last_code() { return g_code ? g_code : TACOGB_ERR_CUDA; }

// ------------------------------------------------------------------ profiling -------------

namespace {
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<ProfRec> g_prof;
std::vector<cudaEvent_t> g_event_pool;
size_t g_event_next = 0;
long long g_launches = 0;

cudaEvent_t pool_event() {
  if (g_event_next == g_event_pool.size()) {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    g_event_pool.push_back(e);
  }
  return g_event_pool[g_event_next++];
}
}  // namespace

void prof_before(const char* name, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_launches++;
  if (!g_prof_on) return;
  ProfRec r{name, pool_event(), nullptr};
  cudaEventRecord(r.a, st);
  g_prof.push_back(r);
}

void count_launch() {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_launches++;
}

void prof_after(cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_on || g_prof.empty()) return;
  g_prof.back().b = pool_event();
  cudaEventRecord(g_prof.back().b, st);
}

// ------------------------------------------------------------------ device state ----------

namespace {

constexpr int kMaxDevices = 64;
constexpr int kScratchSlots = 15;  // spmv, spmm, spgemm x2, tuner, pack, sddmm, tensor3, formats x3,
                                   // index validation, one-pass SpGEMM x2, the pipelined SpMM's
                                   // second product stream
constexpr int kSpmmLaneSlot = 14;

struct DeviceState {
  int sms = 0;
  void* scratch[kScratchSlots] = {};
  size_t scratch_cap[kScratchSlots] = {};
  // staging buffers for host-memory operands of the taco ABI
  std::vector<void*> stage;
  std::vector<size_t> stage_cap;
  cudaStream_t stream = nullptr;
  // the pipelined products' copy streams (host -> device, device -> host), the two streams of
  // products that may overlap, and chunk events
  cudaStream_t h2d = nullptr, d2h = nullptr, lanes[2] = {nullptr, nullptr};
  cudaEvent_t ev[2 * 16 + 1] = {};
  int* status = nullptr;  // device status word (see device_status())
  unsigned long long* mailbox = nullptr;  // mapped pinned host words (see host_mailbox())
};

std::mutex g_mu;
DeviceState g_dev[kMaxDevices];

DeviceState* current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return nullptr;
  return &g_dev[d];
}

}  // namespace

int sm_count() {
  DeviceState* ds = current_device();
  if (!ds) return 148;
  if (ds->sms == 0) {
    int d = 0, v = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d);
    ds->sms = v > 0 ? v : 148;
  }
  return ds->sms;
}

int gather_carveout_pct(int pct) {
  static const int env = [] {
    const char* e = getenv("TACOGB_SMEM_CARVEOUT");
    const int v = e ? atoi(e) : -2;
    return (v >= -1 && v <= 100) ? v : -2;
  }();
  return env != -2 ? env : pct;
}

void* scratch(size_t bytes, int slot) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState* ds = current_device();
  if (!ds || slot < 0 || slot >= kScratchSlots) {
    set_error(TACOGB_ERR_ARG, "scratch: no device or bad slot");
    return nullptr;
  }
  if (bytes == 0) bytes = 256;
  if (ds->scratch_cap[slot] < bytes) {
    size_t cap = bytes + bytes / 4;
    if (ds->scratch[slot]) cudaFree(ds->scratch[slot]);
    ds->scratch[slot] = nullptr;
    ds->scratch_cap[slot] = 0;
    cudaError_t e = cudaMalloc(&ds->scratch[slot], cap);
    if (e != cudaSuccess) {
      set_error(TACOGB_ERR_ALLOC, "scratch: cudaMalloc(%zu) failed: %s", cap, cudaGetErrorString(e));
      return nullptr;
    }
    ds->scratch_cap[slot] = cap;
  }
  return ds->scratch[slot];
}

int* device_status() {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState* ds = current_device();
  if (!ds) return nullptr;
  if (!ds->status) {
    if (cudaMalloc(&ds->status, 256) != cudaSuccess) {
      ds->status = nullptr;
      set_error(TACOGB_ERR_ALLOC, "device status: cudaMalloc failed");
      return nullptr;
    }
    cudaMemset(ds->status, 0, 256);
  }
  return ds->status;
}

unsigned long long* host_mailbox() {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState* ds = current_device();
  if (!ds) return nullptr;
  if (!ds->mailbox) {
    void* p = nullptr;
    cudaError_t e = cudaHostAlloc(&p, kMailboxWords * sizeof(unsigned long long), cudaHostAllocMapped);
    if (e != cudaSuccess) {
      set_error(TACOGB_ERR_ALLOC, "mailbox: cudaHostAlloc failed: %s", cudaGetErrorString(e));
      return nullptr;
    }
    void* d = nullptr;
    e = cudaHostGetDevicePointer(&d, p, 0);
    if (e != cudaSuccess || d != p) {
      // unified addressing gives one address for both sides; without it there is no mailbox
      cudaFreeHost(p);
      set_error(TACOGB_ERR_CUDA, "mailbox: mapped host memory has no common address");
      return nullptr;
    }
    std::memset(p, 0, kMailboxWords * sizeof(unsigned long long));
    ds->mailbox = (unsigned long long*)p;
  }
  return ds->mailbox;
}

namespace {

// Reads and clears the device status word; TACOGB_ERR_TIMEOUT when a bounded wait gave up.
int consume_device_status() {
  int* st = device_status();
  if (!st) return TACOGB_ERR_ALLOC;
  int h = 0;
  TACOGB_CUDA_TRY(cudaMemcpy(&h, st, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    TACOGB_CUDA_TRY(cudaMemset(st, 0, sizeof(int)));
    set_error(TACOGB_ERR_TIMEOUT, "a bounded device-side wait timed out (status %d)", h);
    return TACOGB_ERR_TIMEOUT;
  }
  return 0;
}

// Device staging buffer `slot` with room for `bytes` (for host-resident taco operands).
void* stage_buffer(int slot, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState* ds = current_device();
  if (!ds) return nullptr;
  if ((int)ds->stage.size() <= slot) {
    ds->stage.resize(slot + 1, nullptr);
    ds->stage_cap.resize(slot + 1, 0);
  }
  if (bytes == 0) bytes = 16;
  if (ds->stage_cap[slot] < bytes) {
    if (ds->stage[slot]) cudaFree(ds->stage[slot]);
    ds->stage[slot] = nullptr;
    ds->stage_cap[slot] = 0;
    if (cudaMalloc(&ds->stage[slot], bytes) != cudaSuccess) {
      set_error(TACOGB_ERR_ALLOC, "staging: cudaMalloc(%zu) failed", bytes);
      return nullptr;
    }
    ds->stage_cap[slot] = bytes;
  }
  return ds->stage[slot];
}

cudaStream_t lib_stream() {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState* ds = current_device();
  if (!ds) return nullptr;
  if (!ds->stream) cudaStreamCreateWithFlags(&ds->stream, cudaStreamNonBlocking);
  return ds->stream;
}

// The pipelined SpMV's two copy streams and its events (created once per device).
bool pipeline_streams(cudaStream_t* h2d, cudaStream_t* d2h, cudaStream_t* lanes,
                      cudaEvent_t** ev) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState* ds = current_device();
  if (!ds) return false;
  if (!ds->h2d && cudaStreamCreateWithFlags(&ds->h2d, cudaStreamNonBlocking) != cudaSuccess)
    return false;
  if (!ds->d2h && cudaStreamCreateWithFlags(&ds->d2h, cudaStreamNonBlocking) != cudaSuccess)
    return false;
  for (int l = 0; l < 2; l++) {
    if (!ds->lanes[l] &&
        cudaStreamCreateWithFlags(&ds->lanes[l], cudaStreamNonBlocking) != cudaSuccess)
      return false;
    lanes[l] = ds->lanes[l];
  }
  for (cudaEvent_t& e : ds->ev)
    if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
  *h2d = ds->h2d;
  *d2h = ds->d2h;
  *ev = ds->ev;
  return true;
}

// True when the GPU can dereference p directly (device or managed memory).
bool device_accessible(const void* p) {
  if (!p) return true;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// An operand array as seen by the kernels: either the caller's pointer (device-accessible) or
// a staging copy.
struct Operand {
  const void* host = nullptr;
  void* dev = nullptr;
  size_t bytes = 0;
  bool staged = false;
};

// A host -> device copy over the GB300 host link runs at full rate only from a host address on
// a 128-byte boundary (1.25 GB in 18 pinned copies: 5.96 ms from aligned sources, 6.73 ms from
// sources 16 bytes past one; the device address and device -> host copies are indifferent).
// Operand arrays start where the caller's allocator put them (malloc: 16 bytes into a page) and
// pipeline chunks where a row starts, so a large copy from an unaligned source goes as a head up
// to the next 128-byte boundary and an aligned body (5.99 ms in the same test).
constexpr size_t kHostLine = 128;
constexpr size_t kSplitHeadMin = (size_t)4 << 20;  // below this one more copy costs more

cudaError_t copy_h2d(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  const size_t mis = (uintptr_t)src & (kHostLine - 1);
  if (mis == 0 || bytes < kSplitHeadMin)
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
  const size_t head = kHostLine - mis;
  const cudaError_t e = cudaMemcpyAsync(dst, src, head, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync((unsigned char*)dst + head, (const unsigned char*)src + head,
                         bytes - head, cudaMemcpyHostToDevice, st);
}

int stage_in(Operand& o, const void* p, size_t bytes, int slot, cudaStream_t st) {
  o.host = p;
  o.bytes = bytes;
  if (device_accessible(p)) {
    o.dev = const_cast<void*>(p);
    return 0;
  }
  o.dev = stage_buffer(slot, bytes);
  if (!o.dev) return TACOGB_ERR_ALLOC;
  o.staged = true;
  if (bytes) TACOGB_CUDA_TRY(copy_h2d(o.dev, p, bytes, st));
  return 0;
}

// Stages one compressed level (pos: outer + 1 entries, crd: nnz entries, and optionally the
// values: vbytes) into slots slot, slot + 1, slot + 2 and checks it (validate.h) on the arrays
// the kernels will read.  A failed check is reported before any error of the staging.
// The same without the check yet: chk records the level, and the caller runs
// chk.finish(st, op.dev, oc.dev) once it has issued its other copies, so that the check's
// synchronisation waits for all of them together.  When the staging fails, chk diagnoses
// host-resident input first.
int stage_level(const char* what, int64_t outer, int32_t inner, int64_t nnz, const void* pos,
                const void* crd, const void* vals, size_t vbytes, int slot, cudaStream_t st,
                Operand& op, Operand& oc, Operand* ov, LevelCheck& chk) {
  chk.begin(what, outer, inner, (const int32_t*)pos, (const int32_t*)crd, nnz,
            !device_accessible(pos) && !device_accessible(crd));
  int src = stage_in(op, pos, ((size_t)outer + 1) * 4, slot, st);
  if (!src) src = stage_in(oc, crd, (size_t)nnz * 4, slot + 1, st);
  if (!src && ov) src = stage_in(*ov, vals, vbytes, slot + 2, st);
  if (src) {
    if (int rc = chk.finish(st, nullptr, nullptr)) return rc;
  }
  return src;
}

int stage_checked_level(const char* what, int64_t outer, int32_t inner, int64_t nnz,
                        const void* pos, const void* crd, const void* vals, size_t vbytes,
                        int slot, cudaStream_t st, Operand& op, Operand& oc, Operand* ov) {
  LevelCheck chk;
  if (int rc = stage_level(what, outer, inner, nnz, pos, crd, vals, vbytes, slot, st, op, oc, ov,
                           chk))
    return rc;
  return chk.finish(st, op.dev, oc.dev);
}

int value_type_of_csize(int32_t csize) {
  switch (csize) {
    case 64: return TACOGB_F64;
    case 32: return TACOGB_F32;
    case 16: return TACOGB_BF16;
  }
  return -1;
}

size_t value_bytes(int vt) { return vt == TACOGB_F64 ? 8 : vt == TACOGB_F32 ? 4 : 2; }

// Reads an int32 that may live in host, managed or device memory.
int read_i32(const int32_t* p, int32_t* out) {
  if (!device_accessible(p)) {
    *out = *p;
    return 0;
  }
  cudaPointerAttributes at;
  cudaPointerGetAttributes(&at, p);
  if (at.type == cudaMemoryTypeManaged) {
    TACOGB_CUDA_TRY(cudaDeviceSynchronize());
    *out = *p;
    return 0;
  }
  TACOGB_CUDA_TRY(cudaMemcpy(out, p, sizeof(int32_t), cudaMemcpyDeviceToHost));
  return 0;
}

// Allocation for a result array, with the allocator taco releases it with
// (src/storage/array.cpp:22-33): cudaMallocManaged when the operands are GPU memory (taco's
// CUDA build), malloc otherwise.
// Device -> host copies into fresh host allocations (the malloc'd results taco frees).  A copy
// into pages the OS has not mapped yet pays a fault and the page's zeroing per page inside the
// copy: 200 MB took 8.5-12.7 ms that way on the GB300 machine's host, against 1.4 ms into mapped
// pageable or pinned memory, while eight threads map 134 MB in about 1.2 ms.  So for large
// results, host threads map the pages chunk by chunk (one write per page, inside the buffer
// only) and each chunk's copy is issued on st as soon as its pages are mapped: the mapping of
// later chunks overlaps the copies of earlier ones.  Small results are copied directly (the
// threads would cost more than the faults).
struct HostCopy {
  void* dst;
  const void* src;
  size_t bytes;
};

// Maps the pages of [p, p + bytes) of host memory (one write per page, inside the range only)
// with up to eight threads; for pageable destinations of device -> host copies, before the copy
// is issued.
void map_host_pages(void* p, size_t bytes) {
  if (!bytes) return;
  const long pg = sysconf(_SC_PAGESIZE);
  const size_t page = pg > 0 ? (size_t)pg : 4096;
  const int nt = (int)std::min<size_t>({8, std::max(1u, std::thread::hardware_concurrency()),
                                        std::max<size_t>(1, bytes >> 22)});
  auto touch = [=](size_t a, size_t b) {
    volatile unsigned char* q = (volatile unsigned char*)p;
    for (size_t o = a; o < b; o = (o / page + 1) * page) q[o] = 0;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; t++)
    th.emplace_back([=] {
      spread_thread();
      touch(bytes * t / nt, bytes * (t + 1) / nt);
    });
  touch(0, bytes / nt);
  for (auto& x : th) x.join();
}

// True for results of 4 MB or more in pageable host memory, whose pages are best mapped before
// the copies into them.
bool wants_page_mapping(const void* dst, size_t bytes) {
  if (bytes < ((size_t)4 << 20)) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, dst) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return at.type == cudaMemoryTypeUnregistered;
}

int copy_to_fresh_host(std::initializer_list<HostCopy> copies, cudaStream_t st) {
  constexpr size_t kPipelineBytes = (size_t)64 << 20, kChunk = (size_t)16 << 20;
  size_t total = 0;
  bool pinned = false;  // page-locked destinations are mapped already
  for (const HostCopy& c : copies) {
    total += c.bytes;
    cudaPointerAttributes at;
    if (c.bytes && cudaPointerGetAttributes(&at, c.dst) == cudaSuccess)
      pinned = pinned || at.type == cudaMemoryTypeHost;
    else
      cudaGetLastError();
  }
  if (total < kPipelineBytes || pinned) {
    for (const HostCopy& c : copies)
      if (c.bytes)
        TACOGB_CUDA_TRY(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, st));
    return 0;
  }
  // the chunks of every copy, in order
  std::vector<HostCopy> chunks;
  for (const HostCopy& c : copies)
    for (size_t o = 0; o < c.bytes; o += kChunk)
      chunks.push_back({(unsigned char*)c.dst + o, (const unsigned char*)c.src + o,
                        std::min(kChunk, c.bytes - o)});
  const long pg = sysconf(_SC_PAGESIZE);
  const size_t page = pg > 0 ? (size_t)pg : 4096;
  const int nt = (int)std::min(8u, std::max(1u, std::thread::hardware_concurrency()));
  std::vector<std::atomic<int>> done(chunks.size());
  for (auto& d : done) d.store(0, std::memory_order_relaxed);
  auto worker = [&](int t) {
    spread_thread();
    for (size_t k = 0; k < chunks.size(); k++) {
      const HostCopy& c = chunks[k];
      const size_t a = c.bytes * t / nt, b = c.bytes * (t + 1) / nt;
      volatile unsigned char* p = (volatile unsigned char*)c.dst;
      for (size_t o = a; o < b; o = (o / page + 1) * page) p[o] = 0;
      done[k].fetch_add(1, std::memory_order_release);
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) th.emplace_back(worker, t);
  cudaError_t err = cudaSuccess;
  for (size_t k = 0; k < chunks.size(); k++) {
    while (done[k].load(std::memory_order_acquire) < nt) std::this_thread::yield();
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(chunks[k].dst, chunks[k].src, chunks[k].bytes, cudaMemcpyDeviceToHost,
                            st);
  }
  for (auto& x : th) x.join();
  if (err != cudaSuccess) {
    set_error(TACOGB_ERR_CUDA, "copy to host: %s", cudaGetErrorString(err));
    return TACOGB_ERR_CUDA;
  }
  return 0;
}

void* alloc_result(size_t bytes, bool managed) {
  if (bytes == 0) bytes = 1;
  if (managed) {
    void* p = nullptr;
    if (cudaMallocManaged(&p, bytes) != cudaSuccess) {
      set_error(TACOGB_ERR_ALLOC, "cudaMallocManaged(%zu) failed", bytes);
      return nullptr;
    }
    // the kernels write it first: populate it on this GPU in bulk rather than page by page
    // under the kernels' stores (0.2 GB of SpGEMM results: 6.2 ms of faults otherwise)
    int dev = 0;
    if (bytes >= ((size_t)1 << 20) && cudaGetDevice(&dev) == cudaSuccess) {
      cudaMemLocation loc{};
      loc.type = cudaMemLocationTypeDevice;
      loc.id = dev;
      if (cudaMemPrefetchAsync(p, bytes, loc, 0, lib_stream()) != cudaSuccess) cudaGetLastError();
    }
    return p;
  }
  void* p = malloc(bytes);
  if (!p) set_error(TACOGB_ERR_ALLOC, "malloc(%zu) failed", bytes);
  return p;
}

// ------------------------------------------------------------ struct validation -----------

int check_dense_vector(const taco_tensor_t* t, const char* name) {
  TACOGB_CHECK_ARG(t != nullptr, "%s: null tensor", name);
  TACOGB_CHECK_ARG(t->order == 1, "%s: expected order 1, got %d", name, t->order);
  TACOGB_CHECK_ARG(t->mode_types == nullptr || t->mode_types[0] == taco_mode_dense,
                   "%s: expected a {Dense} vector", name);
  TACOGB_CHECK_ARG(t->dimensions != nullptr, "%s: null dimensions", name);
  return 0;
}

int check_dense_matrix(const taco_tensor_t* t, const char* name) {
  TACOGB_CHECK_ARG(t != nullptr, "%s: null tensor", name);
  TACOGB_CHECK_ARG(t->order == 2, "%s: expected order 2, got %d", name, t->order);
  TACOGB_CHECK_ARG(t->mode_types == nullptr ||
                       (t->mode_types[0] == taco_mode_dense && t->mode_types[1] == taco_mode_dense),
                   "%s: expected {Dense,Dense}", name);
  TACOGB_CHECK_ARG(t->mode_ordering == nullptr ||
                       (t->mode_ordering[0] == 0 && t->mode_ordering[1] == 1),
                   "%s: expected row-major mode ordering {0,1}", name);
  TACOGB_CHECK_ARG(t->dimensions != nullptr, "%s: null dimensions", name);
  return 0;
}

// Rows j*rows_chunk.. of a chunked SpMV: pos of every chunk rebased to start at zero, each chunk
// at its own 4-entry-aligned offset (so the warp tiles' bulk copies stay 16-byte aligned).
__global__ void spmv_rebase_pos(const int32_t* __restrict__ pos, const int64_t* __restrict__ meta,
                                int chunks, int32_t* __restrict__ out) {
  // meta: per chunk (first row, rows, output offset)
  const int j = blockIdx.y;
  if (j >= chunks) return;
  const int64_t r0 = meta[3 * j], nr = meta[3 * j + 1], o = meta[3 * j + 2];
  const int32_t base = __ldg(pos + r0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nr;
       i += (int64_t)gridDim.x * blockDim.x)
    out[o + i] = __ldg(pos + r0 + i) - base;
}

int check_csr(const taco_tensor_t* t, const char* name) {
  TACOGB_CHECK_ARG(t != nullptr, "%s: null tensor", name);
  TACOGB_CHECK_ARG(t->order == 2, "%s: expected order 2, got %d", name, t->order);
  TACOGB_CHECK_ARG(t->mode_types != nullptr && t->mode_types[0] == taco_mode_dense &&
                       t->mode_types[1] == taco_mode_sparse,
                   "%s: expected CSR {Dense,Sparse}", name);
  TACOGB_CHECK_ARG(t->mode_ordering == nullptr ||
                       (t->mode_ordering[0] == 0 && t->mode_ordering[1] == 1),
                   "%s: expected mode ordering {0,1} (CSR, not CSC)", name);
  TACOGB_CHECK_ARG(t->dimensions != nullptr && t->indices != nullptr && t->indices[1] != nullptr,
                   "%s: missing dimensions or indices", name);
  return 0;
}

}  // namespace
}  // namespace tacogb

using namespace tacogb;

// =================================================================== exported ==============

extern "C" {

const char* tacogb_last_error(void) { return g_err; }

int tacogb_device_status(int32_t* status) {
  int* st = device_status();
  if (!st) return TACOGB_ERR_ALLOC;
  int h = 0;
  TACOGB_CUDA_TRY(cudaMemcpy(&h, st, sizeof(int), cudaMemcpyDeviceToHost));
  TACOGB_CUDA_TRY(cudaMemset(st, 0, sizeof(int)));
  if (status) *status = h;
  return 0;
}

long long tacogb_launch_count(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  return g_launches;
}

void tacogb_profile_begin(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.clear();
  g_event_next = 0;
  g_prof_on = true;
}

void tacogb_profile_enable(int32_t on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = on != 0;
}

int tacogb_profile_end(int32_t max_kernels, char* names, double* total_ms, int32_t* launches) {
  std::vector<ProfRec> recs;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_on = false;
    recs.swap(g_prof);
  }
  int n = 0;
  for (const ProfRec& r : recs) {
    if (!r.b) continue;
    if (cudaEventSynchronize(r.b) != cudaSuccess) {
      set_error(TACOGB_ERR_CUDA, "profile: event synchronize failed");
      return -TACOGB_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    int k = 0;
    while (k < n && strncmp(names + 64 * k, r.name, 63) != 0) k++;
    if (k == n) {
      if (n == max_kernels) continue;
      strncpy(names + 64 * n, r.name, 63);
      names[64 * n + 63] = 0;
      total_ms[n] = 0.0;
      launches[n] = 0;
      n++;
    }
    total_ms[k] += ms;
    launches[k] += 1;
  }
  return n;
}
const char* tacogb_version(void) { return "taco_gb300 0.1 (sm_103a)"; }

int tacogb_spmv(const tacogb_csr* A, const void* x, void* y, int32_t variant, void* stream) {
  return spmv_run(A, x, y, variant, (cudaStream_t)stream);
}
int tacogb_spmv_variant_count(void) { return spmv_variant_count(); }
int tacogb_spmv_auto_variant(const tacogb_csr* A, void* stream) {
  TACOGB_CHECK_ARG(A != nullptr && A->nnz >= 0, "SpMV: bad matrix");
  return spmv_auto_variant(A, (cudaStream_t)stream);
}
const char* tacogb_spmv_variant_name(int32_t v) { return spmv_variant_name(v); }

int tacogb_spmm(const tacogb_csr* A, int32_t N, const void* B, int32_t btype, void* C,
                int32_t variant, void* stream) {
  return spmm_run(A, N, B, btype, C, variant, (cudaStream_t)stream);
}
int tacogb_spmm_variant_count(void) { return spmm_variant_count(); }
const char* tacogb_spmm_variant_name(int32_t v) { return spmm_variant_name(v); }

int tacogb_spgemm_symbolic(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos,
                           int64_t* nnzC, void* stream) {
  return spgemm_symbolic(A, B, Cpos, nnzC, (cudaStream_t)stream);
}
int tacogb_spgemm_fill(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos,
                       int32_t* Ccrd, void* stream) {
  return spgemm_fill(A, B, Cpos, Ccrd, (cudaStream_t)stream);
}
int tacogb_spgemm_numeric(const tacogb_csr* A, const tacogb_csr* B, const int32_t* Cpos,
                          const int32_t* Ccrd, void* Cvals, void* stream) {
  return spgemm_numeric(A, B, Cpos, Ccrd, Cvals, (cudaStream_t)stream);
}
int tacogb_spgemm_onepass(const tacogb_csr* A, const tacogb_csr* B, int32_t* Cpos,
                          int64_t* nnzC, void* stream) {
  return spgemm_onepass(A, B, Cpos, nnzC, (cudaStream_t)stream);
}
int tacogb_spgemm_onepass_finish(const int32_t* Cpos, int32_t* Ccrd, void* Cvals, void* stream) {
  return spgemm_onepass_finish(Cpos, Ccrd, Cvals, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- SpMV taco ABI -----------

// ------------------------------------------------------- SpMV operand formats (taco ABI) ---
//
// Besides CSR A with dense x and y, tacogb_spmv_assemble/compute take the format combinations of
// taco's spmv tests (test/tests-expr_storage.cpp:873-937): A CSC ({Dense,Sparse}, mode ordering
// {1,0}) or DCSR ({Sparse,Sparse}); x {Sparse}; y {Sparse} when A is DCSR (y's coordinates are
// A's stored rows, taco's generated assemble for that statement).

namespace {

enum { kFmtOther = 0, kFmtCSR, kFmtCSC, kFmtDCSR, kFmtDCSC };

int mat_format(const taco_tensor_t* A) {
  if (!A || A->order != 2 || !A->mode_types || !A->dimensions || !A->indices) return kFmtOther;
  const bool o01 = !A->mode_ordering || (A->mode_ordering[0] == 0 && A->mode_ordering[1] == 1);
  const bool o10 = A->mode_ordering && A->mode_ordering[0] == 1 && A->mode_ordering[1] == 0;
  const int m0 = A->mode_types[0], m1 = A->mode_types[1];
  if (m0 == taco_mode_dense && m1 == taco_mode_sparse) return o01 ? kFmtCSR : o10 ? kFmtCSC : kFmtOther;
  if (m0 == taco_mode_sparse && m1 == taco_mode_sparse) return o01 ? kFmtDCSR : o10 ? kFmtDCSC : kFmtOther;
  return kFmtOther;
}

bool is_sparse_vector(const taco_tensor_t* t) {
  return t && t->order == 1 && t->mode_types && t->mode_types[0] == taco_mode_sparse;
}

bool plain_spmv(const taco_tensor_t* y, const taco_tensor_t* A, const taco_tensor_t* x) {
  return mat_format(A) == kFmtCSR && !is_sparse_vector(x) && !is_sparse_vector(y);
}

int check_any_vector(const taco_tensor_t* t, const char* name) {
  TACOGB_CHECK_ARG(t != nullptr && t->order == 1 && t->dimensions != nullptr,
                   "%s: expected an order-1 tensor", name);
  if (is_sparse_vector(t))
    TACOGB_CHECK_ARG(t->indices && t->indices[0], "%s: missing sparse indices", name);
  return 0;
}

// The checks shared by the format path's assemble and compute; *fmt receives A's format.
int check_spmv_formats(const taco_tensor_t* y, const taco_tensor_t* A, const taco_tensor_t* x,
                       int* fmt) {
  *fmt = mat_format(A);
  TACOGB_CHECK_ARG(*fmt != kFmtOther && *fmt != kFmtDCSC,
                   "spmv: A must be CSR, CSC ({Dense,Sparse} ordered {1,0}) or DCSR");
  if (int rc = check_any_vector(y, "spmv result y")) return rc;
  if (int rc = check_any_vector(x, "spmv operand x")) return rc;
  TACOGB_CHECK_ARG(!is_sparse_vector(y) || *fmt == kFmtDCSR,
                   "spmv: a {Sparse} result needs a DCSR A (its stored rows are y's pattern)");
  const int vt = value_type_of_csize(A->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "spmv: unsupported csize %d", A->csize);
  TACOGB_CHECK_ARG(x->csize == A->csize && y->csize == A->csize,
                   "spmv: operand component sizes differ");
  TACOGB_CHECK_ARG(y->dimensions[0] == A->dimensions[0] && x->dimensions[0] == A->dimensions[1],
                   "spmv: shapes differ (y %d, A %dx%d, x %d)", y->dimensions[0],
                   A->dimensions[0], A->dimensions[1], x->dimensions[0]);
  return 0;
}

// A DCSR operand's level-0 row list and level-1 arrays on the device (slots base .. base+4).
int dcsr_operand(const taco_tensor_t* A, int base, cudaStream_t st, tacogb_dcsr& out) {
  const int32_t* pos0 = (const int32_t*)A->indices[0][0];
  TACOGB_CHECK_ARG(pos0 != nullptr && A->indices[1], "DCSR: missing indices");
  tacogb_dcsr d{};
  d.rows = A->dimensions[0];
  d.cols = A->dimensions[1];
  d.vtype = value_type_of_csize(A->csize);
  if (int rc = read_i32(pos0 + 1, &d.n0)) return rc;
  // checked before pos1 is read at it: at most one stored row per row of A
  TACOGB_CHECK_ARG(d.n0 >= 0 && d.n0 <= d.rows, "DCSR: level-0 pos ends at %d, beyond %d rows",
                   d.n0, d.rows);
  const int32_t* pos1 = (const int32_t*)A->indices[1][0];
  TACOGB_CHECK_ARG(pos1 != nullptr, "DCSR: null pos");
  int32_t nnz = 0;
  if (int rc = read_i32(pos1 + d.n0, &nnz)) return rc;
  d.nnz = nnz;
  Operand o0p, o0, op, oc, ov;
  if (int rc = stage_checked_level("DCSR level 0", 1, d.rows, d.n0, pos0, A->indices[0][1],
                                   nullptr, 0, 83, st, o0p, o0, nullptr))
    return rc;
  if (int rc = stage_checked_level("DCSR level 1", d.n0, d.cols, nnz, pos1, A->indices[1][1],
                                   A->vals, (size_t)nnz * value_bytes(d.vtype), base + 1, st, op,
                                   oc, &ov))
    return rc;
  d.crd0 = (const int32_t*)o0.dev;
  d.pos = (const int32_t*)op.dev;
  d.crd = (const int32_t*)oc.dev;
  d.vals = ov.dev;
  out = d;
  return 0;
}

// x as a dense device vector: a {Dense} x staged as is, a {Sparse} x scattered into zeros.
int dense_x(const taco_tensor_t* x, int vt, int base, cudaStream_t st, const void** out) {
  const int32_t n = x->dimensions[0];
  const size_t vb = value_bytes(vt);
  if (!is_sparse_vector(x)) {
    Operand o;
    if (int rc = stage_in(o, x->vals, (size_t)n * vb, base, st)) return rc;
    *out = o.dev;
    return 0;
  }
  const int32_t* pos = (const int32_t*)x->indices[0][0];
  TACOGB_CHECK_ARG(pos != nullptr, "spmv: null pos of the sparse x");
  int32_t k = 0;
  if (int rc = read_i32(pos + 1, &k)) return rc;
  Operand op, oi, ov;
  if (int rc = stage_checked_level("spmv operand x", 1, n, k, pos, x->indices[0][1], x->vals,
                                   (size_t)k * vb, 80, st, op, oi, &ov))
    return rc;
  void* d = stage_buffer(base + 2, (size_t)n * vb);
  if (!d) return TACOGB_ERR_ALLOC;
  if (int rc = densify_run(n, k, (const int32_t*)oi.dev, ov.dev, vt, d, st)) return rc;
  *out = d;
  return 0;
}

int spmv_fmt_assemble(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x) {
  int fmt;
  if (int rc = check_spmv_formats(y, A, x, &fmt)) return rc;
  const int vt = value_type_of_csize(A->csize);
  const bool managed = A->vals != nullptr && device_accessible(A->vals);
  if (!is_sparse_vector(y)) {
    void* p = alloc_result((size_t)y->dimensions[0] * value_bytes(vt), managed);
    if (!p) return TACOGB_ERR_ALLOC;
    y->vals = (uint8_t*)p;
    return 0;
  }
  int32_t n0 = 0;  // y's pattern: A's stored rows
  if (int rc = read_i32((const int32_t*)A->indices[0][0] + 1, &n0)) return rc;
  TACOGB_CHECK_ARG(n0 >= 0 && n0 <= A->dimensions[0],
                   "spmv: A's level-0 pos ends at %d, beyond %d rows", n0, A->dimensions[0]);
  int32_t* pos = (int32_t*)alloc_result(2 * sizeof(int32_t), managed);
  int32_t* crd = (int32_t*)alloc_result((size_t)n0 * 4, managed);
  void* vals = alloc_result((size_t)n0 * value_bytes(vt), managed);
  if (!pos || !crd || !vals) return TACOGB_ERR_ALLOC;
  const int32_t head[2] = {0, n0};
  cudaStream_t st = lib_stream();
  TACOGB_CUDA_TRY(cudaMemcpyAsync(pos, head, sizeof(head), cudaMemcpyDefault, st));
  if (n0)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(crd, A->indices[0][1], (size_t)n0 * 4, cudaMemcpyDefault, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  y->indices[0][0] = (uint8_t*)pos;
  y->indices[0][1] = (uint8_t*)crd;
  y->vals = (uint8_t*)vals;
  return 0;
}

int spmv_fmt_compute(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x) {
  int fmt;
  if (int rc = check_spmv_formats(y, A, x, &fmt)) return rc;
  TACOGB_CHECK_ARG(y->vals != nullptr, "spmv: result values not assembled");
  const int vt = value_type_of_csize(A->csize);
  const size_t vb = value_bytes(vt);
  const int32_t rows = A->dimensions[0], cols = A->dimensions[1];
  cudaStream_t st = lib_stream();
  const void* xd = nullptr;
  if (int rc = dense_x(x, vt, 45, st, &xd)) return rc;
  const bool sparse_y = is_sparse_vector(y);
  size_t ybytes = (size_t)rows * vb;
  tacogb_dcsr d{};
  if (fmt == kFmtDCSR) {
    if (int rc = dcsr_operand(A, 40, st, d)) return rc;
    if (sparse_y) ybytes = (size_t)d.n0 * vb;
  }
  void* yd = y->vals;
  const bool staged = !device_accessible(y->vals);
  if (staged) {
    yd = stage_buffer(48, ybytes);
    if (!yd) return TACOGB_ERR_ALLOC;
  }
  if (fmt == kFmtDCSR) {
    if (int rc = spmv_dcsr_run(&d, xd, yd, !sparse_y, st)) return rc;
  } else {
    // CSR, or CSC: level 1 runs over columns (cols + 1 pos entries, crd = rows)
    const int32_t outer = fmt == kFmtCSC ? cols : rows;
    const int32_t* pos = (const int32_t*)A->indices[1][0];
    TACOGB_CHECK_ARG(pos != nullptr, "spmv: null pos");
    int32_t nnz = 0;
    if (int rc = read_i32(pos + outer, &nnz)) return rc;
    Operand op, oc, ov;
    if (int rc = stage_checked_level("spmv operand A", outer, fmt == kFmtCSC ? rows : cols, nnz,
                                     pos, A->indices[1][1], A->vals, (size_t)nnz * vb, 40, st,
                                     op, oc, &ov))
      return rc;
    tacogb_csr c{rows, cols, nnz, (const int32_t*)op.dev, (const int32_t*)oc.dev, ov.dev, vt};
    if (int rc = fmt == kFmtCSC ? spmv_csc_run(&c, xd, yd, st)
                                : spmv_run(&c, xd, yd, TACOGB_VARIANT_AUTO, st))
      return rc;
  }
  if (staged && ybytes)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(y->vals, yd, ybytes, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return consume_device_status();
}

}  // namespace

int tacogb_spmv_assemble(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x) {
  if (!plain_spmv(y, A, x)) return spmv_fmt_assemble(y, A, x);
  if (int rc = check_dense_vector(y, "spmv result y")) return rc;
  if (int rc = check_csr(A, "spmv operand A")) return rc;
  const int vt = value_type_of_csize(y->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "spmv: unsupported csize %d", y->csize);
  const bool managed = device_accessible(A->vals) && A->vals != nullptr;
  void* p = alloc_result((size_t)y->dimensions[0] * value_bytes(vt), managed);
  if (!p) return TACOGB_ERR_ALLOC;
  y->vals = (uint8_t*)p;
  return 0;
}

// A CSR product over host operands as a pipeline (SpMV: dense operand x, result y; SpMM: B and
// C, N values per row; SDDMM: D, each chunk's rows of C, one value per nonzero; MTTKRP's fiber
// product: D, fiber rows kept on the device): the rows are cut into chunks by nonzeros (equal
// shares but smaller first and last chunks, below); one stream copies the dense operand, pos
// and then every chunk's crd and values (and rows of the row operand) to the GPU, the library
// stream checks each chunk as soon as its copy has landed and multiplies it (or hands it to one
// of two lane streams), and a third stream returns each chunk's part of the result.  The copies of later chunks overlap the checks, products and
// returns of earlier ones, so the call takes little more than its copies (the host link bounds
// it).  The checks never wait for the host: a chunk that fails is rewritten on the device into
// a harmless level before its product runs, and the verdicts are read after the last chunk, so
// an invalid operand returns TACOGB_ERR_ARG (first failing chunk, positions in the whole
// operand) with the result's contents unspecified.  Results are those of the unchunked product
// up to summation order within merge tiles.
namespace {
constexpr int kPipeChunks = 8;
// chunk events: landed (j), product done (kPipeChunks + j), dense operand and pos in
// (2 kPipeChunks), checked (2 kPipeChunks + 1 + j)
static_assert(3 * kPipeChunks + 1 <= (int)(sizeof(DeviceState::ev) / sizeof(cudaEvent_t)),
              "chunk events");
constexpr int64_t kPipeMinNnz = (int64_t)1 << 23;  // below this, copy then compute

// One kind of product of the pipeline.  reserve() takes any buffers it needs before the copies
// are issued (an allocation later could wait on them); prepare() runs on the library stream
// once the dense operand has landed; run() multiplies one chunk (rowop: the chunk's rows of the
// row operand, when the product has one).  A product whose lanes() is true may run two chunks
// at the same time, on two streams (lane 0 and 1): each launch of a chunk ends in a partly
// filled last wave, which the next chunk's start then fills.
struct ChunkProduct {
  virtual ~ChunkProduct() = default;
  virtual int reserve(int32_t /*cols*/, int32_t /*N*/, int32_t /*btype*/, int /*vt*/) { return 0; }
  virtual int prepare(const void* /*dense*/, int32_t /*cols*/, int32_t /*N*/, cudaStream_t) {
    return 0;
  }
  virtual bool lanes() const { return false; }
  virtual int run(const tacogb_csr* A, const void* dense, void* result, int32_t N, int32_t btype,
                  const void* rowop, int lane, cudaStream_t st) = 0;
};

struct SpmvChunks final : ChunkProduct {  // one lane: the SpMV products share scratch
  int run(const tacogb_csr* A, const void* x, void* y, int32_t, int32_t, const void*, int,
          cudaStream_t st) override {
    return spmv_run(A, x, y, TACOGB_VARIANT_AUTO, st);
  }
};

// FP64: B split into double-float pairs once, when it lands, and every chunk multiplied over
// the split (the library's default FP64 tile, without a split per chunk); FP64 with odd N:
// the double-float tile that splits B on the fly; FP32 and BF16 B: the library's default.
struct SpmmChunks final : ChunkProduct {
  void* bdf = nullptr;
  int* flag = nullptr;
  int32_t n = 0;
  int reserve(int32_t cols, int32_t N, int32_t btype, int vt) override {
    n = N;
    // the split takes pairs of B's elements: N even (the staged B is 256-byte aligned)
    if (vt != TACOGB_F64 || btype != TACOGB_F64 || N <= 0 || N % 2 != 0) return 0;
    int* status = device_status();
    if (!status) return last_code();
    flag = status + kPFlagWord;
    bdf = stage_buffer(60, (size_t)cols * N * sizeof(double) + 64);
    return bdf ? 0 : TACOGB_ERR_ALLOC;
  }
  int prepare(const void* B, int32_t cols, int32_t N, cudaStream_t st) override {
    return bdf ? spmm_split_once((const double*)B, cols, N, bdf, flag, st) : 0;
  }
  // over the split B the products can overlap (each lane has its own scratch); that pays for
  // short chunk products: N = 64, 7.61 -> 7.39 ms per call, but N = 256, 27.0 -> 28.5 ms, whose
  // chunks run many waves each and compete when two run at once
  bool lanes() const override { return bdf != nullptr && n <= 64; }
  int run(const tacogb_csr* A, const void* B, void* C, int32_t N, int32_t btype, const void*,
          int lane, cudaStream_t st) override {
    if (bdf)
      return spmm_run_presplit(A, N, (const double*)B, bdf, flag, (double*)C, st,
                               lane ? kSpmmLaneSlot : 1);
    static const int df = spmm_variant_index("merge_w512_df");
    return spmm_run(A, N, B, btype, C, A->vtype == TACOGB_F64 ? df : TACOGB_VARIANT_AUTO, st);
  }
};

// SDDMM, values at B's nonzeros: the dense operand is D (J x K), transposed once when it lands;
// the row operand is C (each chunk's rows); the result is one value per nonzero.
struct SddmmChunks final : ChunkProduct {
  void* dt = nullptr;
  int vt = TACOGB_F64;
  int reserve(int32_t cols, int32_t J, int32_t, int vtype) override {
    vt = vtype;
    dt = stage_buffer(61, sddmm_pre_bytes(J, cols, vtype));
    return dt ? 0 : TACOGB_ERR_ALLOC;
  }
  int prepare(const void* D, int32_t cols, int32_t J, cudaStream_t st) override {
    return sddmm_pre_transpose(D, J, cols, vt, dt, st);
  }
  bool lanes() const override { return true; }  // no scratch: chunks may overlap
  int run(const tacogb_csr* B, const void* D, void* out, int32_t J, int32_t, const void* C, int,
          cudaStream_t st) override {
    return sddmm_pre_run(B, J, C, D, dt, out, st);
  }
};

// MTTKRP's fiber product: the fiber level (a CSR of fibers over B's last mode) times D, one row
// of J values per fiber, kept on the device for the combine.
struct FiberSpmmChunks final : ChunkProduct {  // one lane: spmm_run's scratch is shared
  int run(const tacogb_csr* F, const void* D, void* T, int32_t J, int32_t, const void*, int,
          cudaStream_t st) override {
    static const int v = spmm_variant_index("stream_w512_dfs");  // as mttkrp_run
    return spmm_run(F, J, D, F->vtype, T, v, st);
  }
};

// rowop (optional): a host operand of rowop_row_bytes per row of A, copied chunk by chunk with
// A's rows.  The result has res_unit_bytes per row of A, or per nonzero of A (res_per_nnz).
// dev_result (optional): a device buffer that keeps the result (rows of A, in order) for a
// later step on the library stream; nothing is returned to the host then.
int csr_product_pipelined(const char* what, const taco_tensor_t* A, int vt, int32_t rows,
                          int32_t cols, int32_t nnz, const void* dense, size_t dense_bytes,
                          int32_t N, int32_t btype, void* result, size_t res_unit_bytes,
                          ChunkProduct& prod, const void* rowop = nullptr,
                          size_t rowop_row_bytes = 0, bool res_per_nnz = false,
                          void* dev_result = nullptr) {
  const int32_t* pos = (const int32_t*)A->indices[1][0];
  const int32_t* crd = (const int32_t*)A->indices[1][1];
  const size_t vb = value_bytes(vt);
  cudaStream_t st = lib_stream(), h2d, d2h, lanes[2];
  cudaEvent_t* ev;
  if (!st || !pipeline_streams(&h2d, &d2h, lanes, &ev)) {
    set_error(TACOGB_ERR_CUDA, "%s: no GPU streams", what);
    return TACOGB_ERR_CUDA;
  }
  // chunk boundaries on the host pos: first row whose start reaches the chunk's share of the
  // nonzeros.  Shares are equal but for the first two and the last two chunks (a quarter and a
  // half of one, from five chunks on): the products start once the first chunk is in, and the
  // last chunk's product and return are the part of the call that no copy overlaps.  Measured
  // against equal shares: SpMV 6.22 -> 6.14 ms (FP64) and 4.21 -> 4.14 ms (FP32) on the
  // 1.0e8-nonzero power-law matrix, SpMM N=64 unchanged (7.62 ms); small last chunks alone
  // (4,...,4,2,1) slowed SpMM to 7.77 ms, whose products wait for B and the first chunk.
  const int K = (int)std::min<int64_t>(kPipeChunks, std::max<int64_t>(1, nnz / (kPipeMinNnz / 2)));
  TACOGB_CHECK_ARG(pos[0] == 0, "%s: pos[0] is not 0", what);
  auto weight_before = [K](int j) -> int64_t {  // in quarters of a full chunk
    int64_t w = 0;
    for (int i = 0; i < j; i++) {
      const int edge = std::min(i, K - 1 - i);  // 0 at either end
      w += K < 5 || edge >= 2 ? 4 : edge == 1 ? 2 : 1;
    }
    return w;
  };
  const int64_t weight_all = weight_before(K);
  int32_t rb[kPipeChunks + 1];
  rb[0] = 0;
  for (int j = 1; j < K; j++) {
    const int64_t target = (int64_t)nnz * weight_before(j) / weight_all;
    int32_t lo = rb[j - 1], hi = rows;
    while (lo < hi) {
      const int32_t mid = lo + (hi - lo) / 2;
      if ((int64_t)pos[mid] < target) lo = mid + 1; else hi = mid;
    }
    rb[j] = lo;
  }
  rb[K] = rows;
  // each chunk is checked on the device into its own counters (no synchronisation per chunk)
  static_assert(kPipeChunks <= kMaxPublishedChecks, "one published check per chunk");
  const bool check = validation_on();
  TACOGB_CHECK_ARG(cols > 0 || nnz == 0, "%s: %d nonzeros in a matrix of 0 columns", what, nnz);
  int64_t meta[3 * kPipeChunks], coff[kPipeChunks + 1], voff[kPipeChunks + 1];
  int64_t poff = 0, c = 0, v = 0;
  for (int j = 0; j < K; j++) {
    const int64_t k0 = pos[rb[j]], k1 = pos[rb[j + 1]];
    TACOGB_CHECK_ARG(k1 >= k0, "%s: pos decreases before segment %d", what, rb[j + 1]);
    meta[3 * j] = rb[j];
    meta[3 * j + 1] = rb[j + 1] - rb[j];
    meta[3 * j + 2] = poff;
    poff += ((rb[j + 1] - rb[j] + 1) + 3) & ~(int64_t)3;
    coff[j] = c;
    voff[j] = v;
    c += ((k1 - k0) + 3) & ~(int64_t)3;  // every chunk's crd and values start 16-byte aligned
    v += ((k1 - k0) + 3) & ~(int64_t)3;
  }
  int32_t* dpos = (int32_t*)stage_buffer(5, ((size_t)rows + 1) * 4);
  int32_t* dposc = (int32_t*)stage_buffer(0, (size_t)poff * 4 + 64);
  int32_t* dcrd = (int32_t*)stage_buffer(1, (size_t)c * 4 + 64);
  unsigned char* dval = (unsigned char*)stage_buffer(2, (size_t)v * vb + 64);
  void* ddense = stage_buffer(3, dense_bytes + 64);
  // results per nonzero sit at the chunks' value offsets (16-byte aligned per chunk)
  unsigned char* dres =
      dev_result ? (unsigned char*)dev_result
                 : (unsigned char*)stage_buffer(
                       4, (res_per_nnz ? (size_t)v : (size_t)rows) * res_unit_bytes + 64);
  unsigned char* drow =
      rowop ? (unsigned char*)stage_buffer(9, (size_t)rows * rowop_row_bytes + 64) : nullptr;
  int64_t* dmeta = (int64_t*)stage_buffer(8, sizeof(meta));
  if (!dpos || !dposc || !dcrd || !dval || !ddense || !dres || !dmeta || (rowop && !drow))
    return TACOGB_ERR_ALLOC;
  if (int rc = prod.reserve(cols, N, btype, vt)) return rc;
  // Every copy is issued up front on the host -> device stream.  A copy from pageable memory
  // returns only once it is (nearly) done, so with pageable operands a copier thread issues
  // them and publishes each chunk's event once it is recorded; the loop below waits for that on
  // the host before it queues the chunk's wait on the device (a wait queued before the event is
  // recorded would not wait).  recorded: -2 nothing yet, -1 the dense operand and pos, j the
  // chunks up to j (K after a failed copy, with copy_err set).
  std::atomic<int> recorded{-2};
  std::atomic<int> copy_err{0};
  auto issue = [&]() {
    cudaError_t e = cudaMemcpyAsync(dmeta, meta, sizeof(int64_t) * 3 * K, cudaMemcpyHostToDevice,
                                    h2d);
    if (e == cudaSuccess && dense_bytes) e = copy_h2d(ddense, dense, dense_bytes, h2d);
    if (e == cudaSuccess) e = copy_h2d(dpos, pos, ((size_t)rows + 1) * 4, h2d);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 * kPipeChunks], h2d);
    if (e == cudaSuccess) recorded.store(-1, std::memory_order_release);
    for (int j = 0; j < K && e == cudaSuccess; j++) {
      const int64_t k0 = pos[rb[j]], n = pos[rb[j + 1]] - k0;
      if (n) {
        e = copy_h2d(dcrd + coff[j], crd + k0, (size_t)n * 4, h2d);
        if (e == cudaSuccess)
          e = copy_h2d(dval + voff[j] * vb, (const unsigned char*)A->vals + k0 * vb,
                       (size_t)n * vb, h2d);
      }
      if (e == cudaSuccess && rowop && rb[j + 1] > rb[j])
        e = copy_h2d(drow + (size_t)rb[j] * rowop_row_bytes,
                     (const unsigned char*)rowop + (size_t)rb[j] * rowop_row_bytes,
                     (size_t)(rb[j + 1] - rb[j]) * rowop_row_bytes, h2d);
      if (e == cudaSuccess) e = cudaEventRecord(ev[j], h2d);
      if (e == cudaSuccess) recorded.store(j, std::memory_order_release);
    }
    if (e != cudaSuccess) {
      copy_err.store((int)e);
      recorded.store(K, std::memory_order_release);
    }
  };
  auto pageable = [](const void* p) {
    cudaPointerAttributes at;
    if (!p) return false;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return true;
    }
    return at.type == cudaMemoryTypeUnregistered;
  };
  const bool pageable_in = pageable(pos) || pageable(crd) || pageable(A->vals) ||
                           (dense_bytes && pageable(dense));
  std::thread copier;
  int dev = 0;
  if (pageable_in && cudaGetDevice(&dev) == cudaSuccess)
    copier = std::thread([&, dev] {
      spread_thread();
      if (cudaSetDevice(dev) != cudaSuccess) {  // a new thread starts on device 0
        copy_err.store((int)cudaErrorInvalidDevice);
        recorded.store(K, std::memory_order_release);
        return;
      }
      issue();
    });
  else
    issue();
  int rc = 0;
  // the host side of a chunk's readiness: its events recorded (or a copy failed)
  auto wait_recorded = [&](int j) {
    while (recorded.load(std::memory_order_acquire) < j) std::this_thread::yield();
    if (const int e = copy_err.load()) {
      set_error(TACOGB_ERR_CUDA, "%s: copy: %s", what, cudaGetErrorString((cudaError_t)e));
      rc = TACOGB_ERR_CUDA;
    }
    return rc == 0;
  };
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == 0) {
      set_error(TACOGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
      rc = TACOGB_ERR_CUDA;
    }
    return rc == 0;
  };
  // A pageable result of up to 64 MB (an evaluate's fresh y) is page-locked for the call, so
  // that its returns are asynchronous copies like a pinned result's (a copy into pageable memory
  // completes before cudaMemcpyAsync returns, which holds the chunk loop); a larger one has its
  // pages mapped by host threads chunk by chunk before each chunk's return.
  const size_t all_res = (res_per_nnz ? (size_t)nnz : (size_t)rows) * res_unit_bytes;
  const bool map_pages = !dev_result && wants_page_mapping(result, all_res);
  bool registered = false;
  if (map_pages && all_res <= ((size_t)64 << 20)) {
    registered = cudaHostRegister(result, all_res, cudaHostRegisterDefault) == cudaSuccess;
    if (!registered) cudaGetLastError();
  }
  const bool map_now = map_pages && !registered && all_res <= ((size_t)64 << 20);
  if (map_now) map_host_pages(result, all_res);
  // chunks' pos rebased once the dense operand and pos are in
  if (wait_recorded(-1) && cu(cudaStreamWaitEvent(st, ev[2 * kPipeChunks], 0))) {
    count_launch();
    spmv_rebase_pos<<<dim3(64, K), 256, 0, st>>>(dpos, dmeta, K, dposc);
    rc = launch_check("spmv_rebase_pos");
    if (rc == 0) rc = prod.prepare(ddense, cols, N, st);
  }
  for (int j = 0; j < K && rc == 0; j++) {
    const int32_t nr = (int32_t)meta[3 * j + 1];
    const int32_t n = pos[rb[j + 1]] - pos[rb[j]];
    if (!wait_recorded(j) || !cu(cudaStreamWaitEvent(st, ev[j], 0))) break;
    int32_t* cpos = dposc + meta[3 * j + 2];
    int32_t* ccrd = dcrd + coff[j];
    tacogb_csr cj{nr, cols, n, cpos, ccrd, dval + voff[j] * vb, vt};
    if (check) {
      // a chunk that fails its check is made harmless before its product runs; the verdicts
      // are read once every chunk is done
      rc = level_check_enqueue(nr, cols, cpos, ccrd, n, j, true, st);
      if (rc) break;
    }
    // this chunk's result: rows rb[j].., or its nonzeros (at voff[j] here, pos[rb[j]] on the host)
    const size_t r_dev = res_per_nnz ? (size_t)voff[j] : (size_t)rb[j];
    const size_t r_host = res_per_nnz ? (size_t)pos[rb[j]] : (size_t)rb[j];
    const size_t r_cnt = res_per_nnz ? (size_t)n : (size_t)nr;
    // a product with two lanes runs its chunks on the two lane streams in turn, each after its
    // chunk's check, so that the checks (in order on the library stream) never wait behind a
    // product and two products can overlap
    const bool two = prod.lanes();
    const int lane = two ? (j & 1) : 0;
    cudaStream_t ps = two ? lanes[lane] : st;
    if (two && (!cu(cudaEventRecord(ev[2 * kPipeChunks + 1 + j], st)) ||
                !cu(cudaStreamWaitEvent(ps, ev[2 * kPipeChunks + 1 + j], 0))))
      break;
    rc = prod.run(&cj, ddense, dres + r_dev * res_unit_bytes, N, btype,
                  drow ? drow + (size_t)rb[j] * rowop_row_bytes : nullptr, lane, ps);
    if (rc) break;
    if (dev_result) continue;  // every stream is synchronised before the call returns
    if (!cu(cudaEventRecord(ev[kPipeChunks + j], ps)) ||
        !cu(cudaStreamWaitEvent(d2h, ev[kPipeChunks + j], 0)))
      break;
    unsigned char* hres = (unsigned char*)result + r_host * res_unit_bytes;
    if (map_pages && !map_now && !registered) map_host_pages(hres, r_cnt * res_unit_bytes);
    if (r_cnt && !cu(cudaMemcpyAsync(hres, dres + r_dev * res_unit_bytes, r_cnt * res_unit_bytes,
                                     cudaMemcpyDeviceToHost, d2h)))
      break;
  }
  if (copier.joinable()) copier.join();
  // nothing may still be copying when the call returns, whatever happened
  const cudaError_t e0a = cudaStreamSynchronize(lanes[0]), e0b = cudaStreamSynchronize(lanes[1]);
  const cudaError_t e0 = e0a != cudaSuccess ? e0a : e0b;
  const cudaError_t e1 = cudaStreamSynchronize(h2d), e2 = cudaStreamSynchronize(st),
                    e3 = cudaStreamSynchronize(d2h);
  if (registered && cudaHostUnregister(result) != cudaSuccess) cudaGetLastError();
  if (rc) return rc;
  if (e0 != cudaSuccess || e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    set_error(TACOGB_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString(e0 != cudaSuccess   ? e0
                                 : e1 != cudaSuccess ? e1
                                 : e2 != cudaSuccess ? e2
                                                     : e3));
    return TACOGB_ERR_CUDA;
  }
  // the first chunk that failed, with its segment and position in the whole operand
  if (check)
    for (int j = 0; j < K; j++)
      if (int v = level_verdict(what, j, rb[j], pos[rb[j]])) return v;
  return consume_device_status();
}

// Large host operands, every array host-resident: the pipelined path.
bool pipeline_applies(int32_t nnz, std::initializer_list<const void*> arrays) {
  if (nnz < kPipeMinNnz) return false;
  for (const void* p : arrays)
    if (p == nullptr || device_accessible(p)) return false;
  return true;
}
}  // namespace

int tacogb_spmv_compute(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x) {
  if (!plain_spmv(y, A, x)) return spmv_fmt_compute(y, A, x);
  if (int rc = check_dense_vector(y, "spmv result y")) return rc;
  if (int rc = check_csr(A, "spmv operand A")) return rc;
  if (int rc = check_dense_vector(x, "spmv operand x")) return rc;
  const int vt = value_type_of_csize(A->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "spmv: unsupported csize %d", A->csize);
  TACOGB_CHECK_ARG(x->csize == A->csize && y->csize == A->csize,
                   "spmv: operand component sizes differ (%d, %d, %d)", y->csize, A->csize,
                   x->csize);
  const int32_t rows = A->dimensions[0], cols = A->dimensions[1];
  TACOGB_CHECK_ARG(y->dimensions[0] == rows, "spmv: y has %d rows, A has %d", y->dimensions[0], rows);
  TACOGB_CHECK_ARG(x->dimensions[0] == cols, "spmv: x has %d rows, A has %d columns",
                   x->dimensions[0], cols);
  TACOGB_CHECK_ARG(y->vals != nullptr, "spmv: result values not assembled");
  const int32_t* pos = (const int32_t*)A->indices[1][0];
  const int32_t* crd = (const int32_t*)A->indices[1][1];
  TACOGB_CHECK_ARG(pos != nullptr, "spmv: null pos");
  int32_t nnz = 0;
  if (int rc = read_i32(pos + rows, &nnz)) return rc;
  TACOGB_CHECK_ARG(nnz >= 0, "spmv: negative nnz");
  const size_t vb = value_bytes(vt);
  // large host operands: copies, checks, products and returns overlapped chunk by chunk
  if (pipeline_applies(nnz, {pos, crd, A->vals, x->vals, y->vals})) {
    SpmvChunks spmv_chunks;
    return csr_product_pipelined("spmv operand A", A, vt, rows, cols, nnz, x->vals,
                                 (size_t)cols * vb, 1, vt, y->vals, vb, spmv_chunks);
  }

  cudaStream_t st = lib_stream();
  Operand opos, ocrd, ovals, ox;
  LevelCheck chk;
  if (int rc = stage_level("spmv operand A", rows, cols, nnz, pos, crd, A->vals, (size_t)nnz * vb,
                           0, st, opos, ocrd, &ovals, chk))
    return rc;
  if (int rc = stage_in(ox, x->vals, (size_t)cols * vb, 3, st)) return rc;
  // staged copies are checked without a wait (a failing one is made harmless on the device)
  if (int rc = chk.finish_deferred(st, opos.dev, ocrd.dev, opos.staged && ocrd.staged)) return rc;
  void* ydev = y->vals;
  const bool y_staged = !device_accessible(y->vals);
  if (y_staged) {
    ydev = stage_buffer(4, (size_t)rows * vb);
    if (!ydev) return TACOGB_ERR_ALLOC;
  }
  tacogb_csr csr{rows, cols, nnz, (const int32_t*)opos.dev, (const int32_t*)ocrd.dev, ovals.dev, vt};
  if (int rc = spmv_run(&csr, ox.dev, ydev, TACOGB_VARIANT_AUTO, st)) return rc;
  if (y_staged && rows)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(y->vals, ydev, (size_t)rows * vb, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (int rc = chk.verdict()) return rc;
  return consume_device_status();
}

int tacogb_spmv_evaluate(taco_tensor_t* y, taco_tensor_t* A, taco_tensor_t* x) {
  if (int rc = tacogb_spmv_assemble(y, A, x)) return rc;
  return tacogb_spmv_compute(y, A, x);
}

int _shim_tacogb_spmv_assemble(void** a) {
  return tacogb_spmv_assemble((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}
int _shim_tacogb_spmv_compute(void** a) {
  return tacogb_spmv_compute((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}
int _shim_tacogb_spmv_evaluate(void** a) {
  return tacogb_spmv_evaluate((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}

// ---------------------------------------------------------------- SpMM taco ABI -----------

int tacogb_spmm_assemble(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = check_dense_matrix(C, "spmm result C")) return rc;
  if (mat_format(A) != kFmtDCSR)
    if (int rc = check_csr(A, "spmm operand A")) return rc;
  const int vt = value_type_of_csize(C->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "spmm: unsupported result csize %d",
                   C->csize);
  const bool managed = device_accessible(A->vals) && A->vals != nullptr;
  void* p = alloc_result((size_t)C->dimensions[0] * (size_t)C->dimensions[1] * value_bytes(vt),
                         managed);
  if (!p) return TACOGB_ERR_ALLOC;
  C->vals = (uint8_t*)p;
  return 0;
}

// C = A B with A DCSR ({Sparse,Sparse}; taco's spmmDCSRGPU, test/tests-scheduling-eval.cpp
// :1309-1358), B and C dense row-major, FP64 or FP32.
static int spmm_dcsr_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = check_dense_matrix(C, "spmm result C")) return rc;
  if (int rc = check_dense_matrix(B, "spmm operand B")) return rc;
  const int vt = value_type_of_csize(A->csize);
  TACOGB_CHECK_ARG((vt == TACOGB_F64 || vt == TACOGB_F32) && B->csize == A->csize &&
                       C->csize == A->csize,
                   "spmm: DCSR A needs FP64 or FP32 operands of one type");
  const int32_t rows = A->dimensions[0], cols = A->dimensions[1], N = B->dimensions[1];
  TACOGB_CHECK_ARG(B->dimensions[0] == cols && C->dimensions[0] == rows && C->dimensions[1] == N,
                   "spmm: shapes differ");
  TACOGB_CHECK_ARG(C->vals != nullptr, "spmm: result values not assembled");
  cudaStream_t st = lib_stream();
  tacogb_dcsr d;
  if (int rc = dcsr_operand(A, 40, st, d)) return rc;
  const size_t vb = value_bytes(vt);
  Operand ob;
  if (int rc = stage_in(ob, B->vals, (size_t)cols * N * vb, 44, st)) return rc;
  const size_t cbytes = (size_t)rows * N * vb;
  void* cdev = C->vals;
  const bool staged = !device_accessible(C->vals);
  if (staged) {
    cdev = stage_buffer(48, cbytes);
    if (!cdev) return TACOGB_ERR_ALLOC;
  }
  if (int rc = spmm_dcsr_run(&d, N, ob.dev, cdev, st)) return rc;
  if (staged && cbytes)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(C->vals, cdev, cbytes, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return consume_device_status();
}

int tacogb_spmm_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (mat_format(A) == kFmtDCSR) return spmm_dcsr_compute(C, A, B);
  if (int rc = check_dense_matrix(C, "spmm result C")) return rc;
  if (int rc = check_csr(A, "spmm operand A")) return rc;
  if (int rc = check_dense_matrix(B, "spmm operand B")) return rc;
  const int at = value_type_of_csize(A->csize), bt = value_type_of_csize(B->csize);
  const int ct = value_type_of_csize(C->csize);
  TACOGB_CHECK_ARG((at == TACOGB_F64 && bt == TACOGB_F64 && ct == TACOGB_F64) ||
                       (at == TACOGB_F32 && (bt == TACOGB_F32 || bt == TACOGB_BF16) &&
                        ct == TACOGB_F32),
                   "spmm: unsupported component sizes (C %d, A %d, B %d)", C->csize, A->csize,
                   B->csize);
  const int32_t rows = A->dimensions[0], cols = A->dimensions[1], N = B->dimensions[1];
  TACOGB_CHECK_ARG(B->dimensions[0] == cols, "spmm: B has %d rows, A has %d columns",
                   B->dimensions[0], cols);
  TACOGB_CHECK_ARG(C->dimensions[0] == rows && C->dimensions[1] == N,
                   "spmm: C is %dx%d, expected %dx%d rows", C->dimensions[0], C->dimensions[1],
                   rows, N);
  TACOGB_CHECK_ARG(C->vals != nullptr, "spmm: result values not assembled");
  const int32_t* pos = (const int32_t*)A->indices[1][0];
  const int32_t* crd = (const int32_t*)A->indices[1][1];
  TACOGB_CHECK_ARG(pos != nullptr, "spmm: null pos");
  int32_t nnz = 0;
  if (int rc = read_i32(pos + rows, &nnz)) return rc;
  // large host operands: copies, checks, products and returns overlapped chunk by chunk
  if (pipeline_applies(nnz, {pos, crd, A->vals, B->vals, C->vals})) {
    SpmmChunks spmm_chunks;
    return csr_product_pipelined("spmm operand A", A, at, rows, cols, nnz, B->vals,
                                 (size_t)cols * N * value_bytes(bt), N, bt, C->vals,
                                 (size_t)N * value_bytes(ct), spmm_chunks);
  }
  cudaStream_t st = lib_stream();
  Operand opos, ocrd, ovals, ob;
  LevelCheck chk;
  if (int rc = stage_level("spmm operand A", rows, cols, nnz, pos, crd, A->vals,
                           (size_t)nnz * value_bytes(at), 0, st, opos, ocrd, &ovals, chk))
    return rc;
  if (int rc = stage_in(ob, B->vals, (size_t)cols * N * value_bytes(bt), 3, st)) return rc;
  // staged copies are checked without a wait (a failing one is made harmless on the device)
  if (int rc = chk.finish_deferred(st, opos.dev, ocrd.dev, opos.staged && ocrd.staged)) return rc;
  const size_t cbytes = (size_t)rows * N * value_bytes(ct);
  void* cdev = C->vals;
  const bool c_staged = !device_accessible(C->vals);
  if (c_staged) {
    cdev = stage_buffer(4, cbytes);
    if (!cdev) return TACOGB_ERR_ALLOC;
  }
  tacogb_csr csr{rows, cols, nnz, (const int32_t*)opos.dev, (const int32_t*)ocrd.dev, ovals.dev, at};
  if (int rc = spmm_run(&csr, N, ob.dev, bt, cdev, TACOGB_VARIANT_AUTO, st)) return rc;
  if (c_staged && cbytes)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(C->vals, cdev, cbytes, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (int rc = chk.verdict()) return rc;
  return consume_device_status();
}

int tacogb_spmm_evaluate(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = tacogb_spmm_assemble(C, A, B)) return rc;
  return tacogb_spmm_compute(C, A, B);
}

int _shim_tacogb_spmm_assemble(void** a) {
  return tacogb_spmm_assemble((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}
int _shim_tacogb_spmm_compute(void** a) {
  return tacogb_spmm_compute((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}
int _shim_tacogb_spmm_evaluate(void** a) {
  return tacogb_spmm_evaluate((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}

// ---------------------------------------------------------------- SpGEMM taco ABI ---------

namespace {

// A matrix operand of SpGEMM as device CSR arrays: CSR as it is; DCSR with its pointer array
// expanded to every row; CSC transposed on the GPU; DCSC expanded to CSC, then transposed
// (taco's spgemm format test, test/tests-scheduling-eval.cpp:655-662).  Host arrays are staged
// into slots base .. base+9.
int csr_operand(const char* what, const taco_tensor_t* T, int base, bool with_vals,
                cudaStream_t st, tacogb_csr& out) {
  const int fmt = mat_format(T);
  if (fmt != kFmtCSR) {
    const int32_t rows = T->dimensions[0], cols = T->dimensions[1];
    const int vt = value_type_of_csize(T->csize);
    TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "spgemm: unsupported csize %d",
                     T->csize);
    const bool doubly = fmt == kFmtDCSR || fmt == kFmtDCSC;
    const int32_t outer = (fmt == kFmtCSC || fmt == kFmtDCSC) ? cols : rows;
    const int32_t* p1 = (const int32_t*)T->indices[1][0];
    TACOGB_CHECK_ARG(p1 != nullptr, "spgemm: null pos");
    int32_t n0 = outer;
    if (doubly) {
      TACOGB_CHECK_ARG(T->indices[0] && T->indices[0][0], "spgemm: null level-0 pos");
      if (int rc = read_i32((const int32_t*)T->indices[0][0] + 1, &n0)) return rc;
      TACOGB_CHECK_ARG(n0 >= 0 && n0 <= outer, "spgemm: level-0 pos ends at %d, beyond %d", n0,
                       outer);
    }
    int32_t nnz = 0;
    if (int rc = read_i32(p1 + n0, &nnz)) return rc;
    const size_t vb = value_bytes(vt);
    Operand op, oc, ov;
    const int32_t inner = (fmt == kFmtCSC || fmt == kFmtDCSC) ? rows : cols;
    if (int rc = stage_checked_level(what, n0, inner, nnz, p1, T->indices[1][1], T->vals,
                                     (size_t)nnz * vb, base, st, op, oc, &ov))
      return rc;
    const int32_t* pos = (const int32_t*)op.dev;
    if (doubly) {  // every row (column) gets its range
      Operand o0p, o0;
      if (int rc = stage_checked_level(what, 1, outer, n0, T->indices[0][0], T->indices[0][1],
                                       nullptr, 0, base + 20, st, o0p, o0, nullptr))
        return rc;
      int32_t* full = (int32_t*)stage_buffer(base + 4, ((size_t)outer + 1) * 4);
      if (!full) return TACOGB_ERR_ALLOC;
      if (int rc = expand_pos_run((const int32_t*)o0.dev, pos, n0, outer, full, st)) return rc;
      pos = full;
    }
    if (fmt == kFmtDCSR) {
      out = tacogb_csr{rows, cols, nnz, pos, (const int32_t*)oc.dev, ov.dev, vt};
      return 0;
    }
    int32_t* cpos = (int32_t*)stage_buffer(base + 5, ((size_t)rows + 1) * 4);
    int32_t* ccrd = (int32_t*)stage_buffer(base + 6, (size_t)nnz * 4);
    void* cval = stage_buffer(base + 7, (size_t)nnz * vb);
    if (!cpos || !ccrd || !cval) return TACOGB_ERR_ALLOC;
    if (int rc = csc_to_csr_run(rows, cols, nnz, pos, (const int32_t*)oc.dev, ov.dev, vt, cpos,
                                ccrd, cval, st))
      return rc;
    out = tacogb_csr{rows, cols, nnz, cpos, ccrd, cval, vt};
    return 0;
  }
  const int32_t rows = T->dimensions[0], cols = T->dimensions[1];
  const int32_t* pos = (const int32_t*)T->indices[1][0];
  const int32_t* crd = (const int32_t*)T->indices[1][1];
  TACOGB_CHECK_ARG(pos != nullptr, "spgemm: null pos");
  int32_t nnz = 0;
  if (int rc = read_i32(pos + rows, &nnz)) return rc;
  const int vt = value_type_of_csize(T->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "spgemm: unsupported csize %d", T->csize);
  Operand op, oc, ov;
  if (int rc = stage_checked_level(what, rows, cols, nnz, pos, crd, T->vals,
                                   (size_t)nnz * value_bytes(vt), base, st, op, oc,
                                   with_vals ? &ov : nullptr))
    return rc;
  out = tacogb_csr{rows, cols, nnz, (const int32_t*)op.dev, (const int32_t*)oc.dev,
                   with_vals ? ov.dev : nullptr, vt};
  return 0;
}

int check_spgemm(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = check_csr(C, "spgemm result C")) return rc;
  TACOGB_CHECK_ARG(mat_format(A) != kFmtOther && mat_format(B) != kFmtOther,
                   "spgemm: operands must be CSR, DCSR, CSC or DCSC");
  TACOGB_CHECK_ARG(A->dimensions[1] == B->dimensions[0], "spgemm: A has %d columns, B has %d rows",
                   A->dimensions[1], B->dimensions[0]);
  TACOGB_CHECK_ARG(C->dimensions[0] == A->dimensions[0] && C->dimensions[1] == B->dimensions[1],
                   "spgemm: C is %dx%d, expected %dx%d", C->dimensions[0], C->dimensions[1],
                   A->dimensions[0], B->dimensions[1]);
  TACOGB_CHECK_ARG(A->csize == B->csize && C->csize == A->csize,
                   "spgemm: component sizes differ (C %d, A %d, B %d)", C->csize, A->csize,
                   B->csize);
  return 0;
}

}  // namespace

int tacogb_spgemm_assemble(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = check_spgemm(C, A, B)) return rc;
  cudaStream_t st = lib_stream();
  tacogb_csr a, b;
  if (int rc = csr_operand("spgemm operand A", A, 60, false, st, a)) return rc;
  if (int rc = csr_operand("spgemm operand B", B, 70, false, st, b)) return rc;
  const int32_t rows = a.rows;
  const bool managed = device_accessible(A->indices[1][0]);
  int32_t* dpos = (int32_t*)stage_buffer(6, ((size_t)rows + 1) * 4);
  if (!dpos) return TACOGB_ERR_ALLOC;
  int64_t nnz = 0;
  if (int rc = spgemm_symbolic(&a, &b, dpos, &nnz, st)) return rc;
  int32_t* dcrd = (int32_t*)stage_buffer(7, (size_t)nnz * 4);
  if (!dcrd) return TACOGB_ERR_ALLOC;
  if (int rc = spgemm_fill(&a, &b, dpos, dcrd, st)) return rc;
  int32_t* pos = (int32_t*)alloc_result(((size_t)rows + 1) * 4, managed);
  int32_t* crd = (int32_t*)alloc_result((size_t)nnz * 4, managed);
  void* vals = alloc_result((size_t)nnz * value_bytes(a.vtype), managed);
  if (!pos || !crd || !vals) return TACOGB_ERR_ALLOC;
  TACOGB_CUDA_TRY(cudaMemcpyAsync(pos, dpos, ((size_t)rows + 1) * 4, cudaMemcpyDefault, st));
  if (nnz) TACOGB_CUDA_TRY(cudaMemcpyAsync(crd, dcrd, (size_t)nnz * 4, cudaMemcpyDefault, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  C->indices[1][0] = (uint8_t*)pos;
  C->indices[1][1] = (uint8_t*)crd;
  C->vals = (uint8_t*)vals;
  return consume_device_status();
}

int tacogb_spgemm_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = check_spgemm(C, A, B)) return rc;
  TACOGB_CHECK_ARG(C->indices[1][0] != nullptr && C->indices[1][1] != nullptr && C->vals != nullptr,
                   "spgemm: result not assembled");
  cudaStream_t st = lib_stream();
  tacogb_csr a, b, c;
  if (int rc = csr_operand("spgemm operand A", A, 60, true, st, a)) return rc;
  if (int rc = csr_operand("spgemm operand B", B, 70, true, st, b)) return rc;
  if (int rc = csr_operand("spgemm result C", C, 6, false, st, c)) return rc;
  const size_t vbytes = (size_t)c.nnz * value_bytes(a.vtype);
  void* dvals = C->vals;
  const bool staged = !device_accessible(C->vals);
  if (staged) {
    dvals = stage_buffer(9, vbytes);
    if (!dvals) return TACOGB_ERR_ALLOC;
  }
  if (int rc = spgemm_numeric(&a, &b, c.pos, c.crd, dvals, st)) return rc;
  if (staged && vbytes)
    if (int rc = copy_to_fresh_host({{C->vals, dvals, vbytes}}, st)) return rc;
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return consume_device_status();
}

// evaluate = assemble and compute in one pass (spgemm_onepass): one sort per row.
int tacogb_spgemm_evaluate(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  if (int rc = check_spgemm(C, A, B)) return rc;
  cudaStream_t st = lib_stream();
  tacogb_csr a, b;
  if (int rc = csr_operand("spgemm operand A", A, 60, true, st, a)) return rc;
  if (int rc = csr_operand("spgemm operand B", B, 70, true, st, b)) return rc;
  const int32_t rows = a.rows;
  const bool managed = device_accessible(A->indices[1][0]);
  int32_t* dpos = (int32_t*)stage_buffer(6, ((size_t)rows + 1) * 4);
  if (!dpos) return TACOGB_ERR_ALLOC;
  int64_t nnz = 0;
  if (int rc = spgemm_onepass(&a, &b, dpos, &nnz, st)) return rc;
  const size_t vb = value_bytes(a.vtype);
  int32_t* pos = (int32_t*)alloc_result(((size_t)rows + 1) * 4, managed);
  int32_t* crd = (int32_t*)alloc_result((size_t)nnz * 4, managed);
  void* vals = alloc_result((size_t)nnz * vb, managed);
  if (!pos || !crd || !vals) return TACOGB_ERR_ALLOC;
  int32_t* dcrd = managed ? crd : (int32_t*)stage_buffer(7, (size_t)nnz * 4);
  void* dvals = managed ? vals : stage_buffer(9, (size_t)nnz * vb);
  if (!dcrd || !dvals) return TACOGB_ERR_ALLOC;
  if (int rc = spgemm_onepass_finish(dpos, dcrd, dvals, st)) return rc;
  TACOGB_CUDA_TRY(cudaMemcpyAsync(pos, dpos, ((size_t)rows + 1) * 4, cudaMemcpyDefault, st));
  if (!managed && nnz)
    if (int rc = copy_to_fresh_host({{crd, dcrd, (size_t)nnz * 4}, {vals, dvals, (size_t)nnz * vb}},
                                    st))
      return rc;
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  C->indices[1][0] = (uint8_t*)pos;
  C->indices[1][1] = (uint8_t*)crd;
  C->vals = (uint8_t*)vals;
  return consume_device_status();
}

int _shim_tacogb_spgemm_assemble(void** a) {
  return tacogb_spgemm_assemble((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}
int _shim_tacogb_spgemm_compute(void** a) {
  return tacogb_spgemm_compute((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}
int _shim_tacogb_spgemm_evaluate(void** a) {
  return tacogb_spgemm_evaluate((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]);
}

// ------------------------------------------------------------------ pack ------------------
//
// Replaces TensorBase::pack (src/tensor.cpp:295-463) for a 2-D CSR tensor: taco's coordinate
// buffer (any order, duplicates) becomes pos/crd/vals allocated with the allocator taco frees
// them with, stored in the tensor as unpackTensorData (src/tensor.cpp:263-292) does.

int tacogb_pack_taco(taco_tensor_t* T, const void* buffer, int64_t n) {
  TACOGB_CHECK_ARG(T != nullptr, "pack: null tensor");
  TACOGB_CHECK_ARG(T->order == 2 && T->dimensions && T->mode_types && T->indices,
                   "pack: expected a 2-D tensor");
  TACOGB_CHECK_ARG(T->mode_types[0] == taco_mode_dense && T->mode_types[1] == taco_mode_sparse,
                   "pack: expected the CSR format {Dense, Sparse}");
  TACOGB_CHECK_ARG(T->mode_ordering == nullptr ||
                       (T->mode_ordering[0] == 0 && T->mode_ordering[1] == 1),
                   "pack: expected mode ordering (0, 1)");
  const int vt = value_type_of_csize(T->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "pack: csize %d bits", T->csize);
  TACOGB_CHECK_ARG(n >= 0 && (n == 0 || buffer != nullptr), "pack: bad coordinate buffer");
  const int32_t rows = T->dimensions[0], cols = T->dimensions[1];
  const size_t vb = value_bytes(vt);
  cudaStream_t st = lib_stream();
  const bool managed = n > 0 && device_accessible(buffer);
  Operand in;
  if (int rc = stage_in(in, buffer, (size_t)n * (8 + vb), 10, st)) return rc;
  int32_t* dr = (int32_t*)stage_buffer(11, (size_t)n * 4);
  int32_t* dc = (int32_t*)stage_buffer(12, (size_t)n * 4);
  void* dv = stage_buffer(13, (size_t)n * vb);
  int32_t* dpos = (int32_t*)stage_buffer(14, ((size_t)rows + 1) * 4);
  int32_t* dcrd = (int32_t*)stage_buffer(15, (size_t)n * 4);
  void* dvals = stage_buffer(16, (size_t)n * vb);
  if (!dr || !dc || !dv || !dpos || !dcrd || !dvals) return TACOGB_ERR_ALLOC;
  // Large host results (taco frees them) are allocated now at their upper bound, n entries
  // (duplicates only lower the count), and host threads map their pages while the GPU packs:
  // the returns then land in mapped memory instead of faulting page by page inside the copies
  // (1.0e8 coordinates: the pages of the 1.2 GB of results take about 10 ms to map).
  const bool premap = !managed && (size_t)n * (4 + vb) >= ((size_t)64 << 20);
  int32_t* pos = nullptr;
  int32_t* crd = nullptr;
  void* vals = nullptr;
  std::thread mapper;
  if (premap) {
    pos = (int32_t*)alloc_result(((size_t)rows + 1) * 4, false);
    crd = (int32_t*)alloc_result((size_t)n * 4, false);
    vals = alloc_result((size_t)n * vb, false);
    if (!pos || !crd || !vals) {
      free(pos);
      free(crd);
      free(vals);
      return TACOGB_ERR_ALLOC;
    }
    mapper = std::thread([=] {
      spread_thread();
      map_host_pages(pos, ((size_t)rows + 1) * 4);
      map_host_pages(crd, (size_t)n * 4);
      map_host_pages(vals, (size_t)n * vb);
    });
  }
  auto fail = [&](int rc) {  // every return after the mapper started
    if (mapper.joinable()) mapper.join();
    if (premap) {
      free(pos);
      free(crd);
      free(vals);
    }
    return rc;
  };
  int64_t nnz = 0;
  if (int rc = pack_split_records(in.dev, n, vt, dr, dc, dv, st)) return fail(rc);
  if (int rc = pack_csr(rows, cols, n, dr, dc, dv, vt, dpos, dcrd, dvals, &nnz, st))
    return fail(rc);
  if (premap) {
    mapper.join();
    cudaError_t e = cudaMemcpyAsync(pos, dpos, ((size_t)rows + 1) * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nnz)
      e = cudaMemcpyAsync(crd, dcrd, (size_t)nnz * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nnz)
      e = cudaMemcpyAsync(vals, dvals, (size_t)nnz * vb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error(TACOGB_ERR_CUDA, "pack: %s", cudaGetErrorString(e));
      return fail(TACOGB_ERR_CUDA);
    }
    T->indices[1][0] = (uint8_t*)pos;
    T->indices[1][1] = (uint8_t*)crd;
    T->vals = (uint8_t*)vals;
    return 0;
  }
  pos = (int32_t*)alloc_result(((size_t)rows + 1) * 4, managed);
  crd = (int32_t*)alloc_result((size_t)nnz * 4, managed);
  vals = alloc_result((size_t)nnz * vb, managed);
  if (!pos || !crd || !vals) return TACOGB_ERR_ALLOC;
  TACOGB_CUDA_TRY(cudaMemcpyAsync(pos, dpos, ((size_t)rows + 1) * 4, cudaMemcpyDefault, st));
  if (nnz && managed) {
    TACOGB_CUDA_TRY(cudaMemcpyAsync(crd, dcrd, (size_t)nnz * 4, cudaMemcpyDefault, st));
    TACOGB_CUDA_TRY(cudaMemcpyAsync(vals, dvals, (size_t)nnz * vb, cudaMemcpyDefault, st));
  } else if (nnz) {
    if (int rc = copy_to_fresh_host({{crd, dcrd, (size_t)nnz * 4}, {vals, dvals, (size_t)nnz * vb}},
                                    st))
      return rc;
  }
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  T->indices[1][0] = (uint8_t*)pos;
  T->indices[1][1] = (uint8_t*)crd;
  T->vals = (uint8_t*)vals;
  return 0;
}

// ------------------------------------------------------------------ SDDMM -----------------
//
// A(i,k) = B(i,k) * C(i,j) * D(j,k) (test/tests-scheduling-eval.cpp:783-840 and 1360-1417).
// A is either taco's test form, {Dense,Dense} I x K (zero outside B's pattern), or CSR with
// B's pattern (assemble copies B's pos and crd).

int tacogb_sddmm(const tacogb_csr* B, int32_t J, const void* C, const void* D, void* out,
                 int32_t variant, void* stream) {
  return sddmm_run(B, J, C, D, out, 0, variant, (cudaStream_t)stream);
}
int tacogb_sddmm_dense(const tacogb_csr* B, int32_t J, const void* C, const void* D, void* A,
                       int64_t lda, int32_t variant, void* stream) {
  TACOGB_CHECK_ARG(lda > 0 || (B != nullptr && (int64_t)B->rows * B->cols == 0),
                   "sddmm: dense result needs a positive row stride");
  return sddmm_run(B, J, C, D, A, lda > 0 ? lda : 1, variant, (cudaStream_t)stream);
}
int tacogb_sddmm_variant_count(void) { return sddmm_variant_count(); }
const char* tacogb_sddmm_variant_name(int32_t v) { return sddmm_variant_name(v); }

namespace {
bool is_csr_result(const taco_tensor_t* A) {
  return A != nullptr && A->order == 2 && A->mode_types != nullptr &&
         A->mode_types[1] == taco_mode_sparse;
}

int check_sddmm(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (is_csr_result(A)) {
    if (int rc = check_csr(A, "sddmm result A")) return rc;
  } else if (int rc = check_dense_matrix(A, "sddmm result A")) {
    return rc;
  }
  if (int rc = check_csr(B, "sddmm operand B")) return rc;
  if (int rc = check_dense_matrix(C, "sddmm operand C")) return rc;
  if (int rc = check_dense_matrix(D, "sddmm operand D")) return rc;
  const int32_t I = B->dimensions[0], K = B->dimensions[1];
  TACOGB_CHECK_ARG(A->dimensions[0] == I && A->dimensions[1] == K,
                   "sddmm: A is %dx%d, B is %dx%d", A->dimensions[0], A->dimensions[1], I, K);
  TACOGB_CHECK_ARG(C->dimensions[0] == I, "sddmm: C has %d rows, B has %d", C->dimensions[0], I);
  TACOGB_CHECK_ARG(D->dimensions[1] == K, "sddmm: D has %d columns, B has %d", D->dimensions[1],
                   K);
  TACOGB_CHECK_ARG(C->dimensions[1] == D->dimensions[0], "sddmm: C has %d columns, D has %d rows",
                   C->dimensions[1], D->dimensions[0]);
  const int vt = value_type_of_csize(B->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "sddmm: unsupported csize %d", B->csize);
  TACOGB_CHECK_ARG(A->csize == B->csize && C->csize == B->csize && D->csize == B->csize,
                   "sddmm: operand component sizes differ (%d, %d, %d, %d)", A->csize, B->csize,
                   C->csize, D->csize);
  return 0;
}
}  // namespace

int tacogb_sddmm_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (int rc = check_sddmm(A, B, C, D)) return rc;
  const int vt = value_type_of_csize(B->csize);
  const int32_t I = B->dimensions[0], K = B->dimensions[1];
  const bool managed = device_accessible(B->vals) && B->vals != nullptr;
  if (!is_csr_result(A)) {
    void* p = alloc_result((size_t)I * (size_t)K * value_bytes(vt), managed);
    if (!p) return TACOGB_ERR_ALLOC;
    A->vals = (uint8_t*)p;
    return 0;
  }
  const int32_t* bpos = (const int32_t*)B->indices[1][0];
  TACOGB_CHECK_ARG(bpos != nullptr, "sddmm: null pos");
  int32_t nnz = 0;
  if (int rc = read_i32(bpos + I, &nnz)) return rc;
  int32_t* pos = (int32_t*)alloc_result(((size_t)I + 1) * 4, managed);
  int32_t* crd = (int32_t*)alloc_result((size_t)nnz * 4, managed);
  void* vals = alloc_result((size_t)nnz * value_bytes(vt), managed);
  if (!pos || !crd || !vals) return TACOGB_ERR_ALLOC;
  cudaStream_t st = lib_stream();
  TACOGB_CUDA_TRY(cudaMemcpyAsync(pos, bpos, ((size_t)I + 1) * 4, cudaMemcpyDefault, st));
  if (nnz)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(crd, B->indices[1][1], (size_t)nnz * 4, cudaMemcpyDefault, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  A->indices[1][0] = (uint8_t*)pos;
  A->indices[1][1] = (uint8_t*)crd;
  A->vals = (uint8_t*)vals;
  return 0;
}

int tacogb_sddmm_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (int rc = check_sddmm(A, B, C, D)) return rc;
  TACOGB_CHECK_ARG(A->vals != nullptr, "sddmm: result values not assembled");
  const int vt = value_type_of_csize(B->csize);
  const size_t vb = value_bytes(vt);
  const int32_t I = B->dimensions[0], K = B->dimensions[1], J = C->dimensions[1];
  const int32_t* pos = (const int32_t*)B->indices[1][0];
  TACOGB_CHECK_ARG(pos != nullptr, "sddmm: null pos");
  int32_t nnz = 0;
  if (int rc = read_i32(pos + I, &nnz)) return rc;
  const bool dense = !is_csr_result(A);
  // large host operands, values at B's nonzeros: D copied and transposed first, then B's rows
  // with their rows of C copied, checked, multiplied and returned chunk by chunk
  if (!dense && sddmm_pre_bytes(J, K, vt) > 0 &&
      pipeline_applies(nnz, {pos, B->indices[1][1], B->vals, C->vals, D->vals, A->vals})) {
    SddmmChunks chunks;
    return csr_product_pipelined("sddmm operand B", B, vt, I, K, nnz, D->vals,
                                 (size_t)J * K * vb, J, vt, A->vals, vb, chunks, C->vals,
                                 (size_t)J * vb, true);
  }
  cudaStream_t st = lib_stream();
  Operand opos, ocrd, ovals, oc, od;
  LevelCheck chk;
  if (int rc = stage_level("sddmm operand B", I, K, nnz, pos, B->indices[1][1], B->vals,
                           (size_t)nnz * vb, 20, st, opos, ocrd, &ovals, chk))
    return rc;
  if (int rc = stage_in(oc, C->vals, (size_t)I * J * vb, 23, st)) return rc;
  if (int rc = stage_in(od, D->vals, (size_t)J * K * vb, 24, st)) return rc;
  if (int rc = chk.finish(st, opos.dev, ocrd.dev)) return rc;
  const size_t obytes = dense ? (size_t)I * (size_t)K * vb : (size_t)nnz * vb;
  void* odev = A->vals;
  const bool staged = !device_accessible(A->vals);
  if (staged) {
    odev = stage_buffer(25, obytes);
    if (!odev) return TACOGB_ERR_ALLOC;
  }
  tacogb_csr b{I, K, nnz, (const int32_t*)opos.dev, (const int32_t*)ocrd.dev, ovals.dev, vt};
  if (int rc = sddmm_run(&b, J, oc.dev, od.dev, odev, dense ? (K > 0 ? K : 1) : 0,
                         TACOGB_VARIANT_AUTO, st))
    return rc;
  if (staged && obytes)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(A->vals, odev, obytes, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return consume_device_status();
}

int tacogb_sddmm_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (int rc = tacogb_sddmm_assemble(A, B, C, D)) return rc;
  return tacogb_sddmm_compute(A, B, C, D);
}

int _shim_tacogb_sddmm_assemble(void** a) {
  return tacogb_sddmm_assemble((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2],
                               (taco_tensor_t*)a[3]);
}
int _shim_tacogb_sddmm_compute(void** a) {
  return tacogb_sddmm_compute((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2],
                              (taco_tensor_t*)a[3]);
}
int _shim_tacogb_sddmm_evaluate(void** a) {
  return tacogb_sddmm_evaluate((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2],
                               (taco_tensor_t*)a[3]);
}

// ------------------------------------------------------------------ order-3 ---------------
//
// TTV, TTM and MTTKRP over B {Sparse,Sparse,Sparse} or {Dense,Sparse,Sparse}
// (test/tests-scheduling-eval.cpp:993-1206, 1420-1580), dense results.

int tacogb_ttv(const tacogb_csf3* B, const void* c, void* out, int32_t variant, void* stream) {
  return ttv_run(B, c, out, false, variant, (cudaStream_t)stream);
}
int tacogb_ttv_dense(const tacogb_csf3* B, const void* c, void* A, int32_t variant,
                     void* stream) {
  return ttv_run(B, c, A, true, variant, (cudaStream_t)stream);
}
int tacogb_ttm(const tacogb_csf3* B, int32_t L, const void* C, void* out, int32_t variant,
               void* stream) {
  return ttm_run(B, L, C, out, false, variant, (cudaStream_t)stream);
}
int tacogb_ttm_dense(const tacogb_csf3* B, int32_t L, const void* C, void* A, int32_t variant,
                     void* stream) {
  return ttm_run(B, L, C, A, true, variant, (cudaStream_t)stream);
}
int tacogb_mttkrp(const tacogb_csf3* B, int32_t J, const void* C, const void* D, void* A,
                  int32_t variant, void* stream) {
  return mttkrp_run(B, J, C, D, A, variant, (cudaStream_t)stream);
}

extern "C++" {  // the helpers below include a template
namespace {

int check_dense_order(const taco_tensor_t* t, int order, const char* name) {
  TACOGB_CHECK_ARG(t != nullptr, "%s: null tensor", name);
  TACOGB_CHECK_ARG(t->order == order, "%s: expected order %d, got %d", name, order, t->order);
  TACOGB_CHECK_ARG(t->dimensions != nullptr, "%s: null dimensions", name);
  for (int m = 0; m < order; m++) {
    TACOGB_CHECK_ARG(t->mode_types == nullptr || t->mode_types[m] == taco_mode_dense,
                     "%s: expected every mode dense", name);
    TACOGB_CHECK_ARG(t->mode_ordering == nullptr || t->mode_ordering[m] == m,
                     "%s: expected row-major mode ordering", name);
  }
  return 0;
}

// B's arrays as a tacogb_csf3 on the device (host arrays staged in slots base + 1 .. base + 5
// and base + 60 .. base + 62), each level checked on the way (stage_checked_level).
// leaf = false stages only levels 0 and 1 (pos2, crd2 and the values stay null in out).
int csf3_operand(const taco_tensor_t* T, int base, cudaStream_t st, tacogb_csf3& out,
                 bool leaf = true) {
  TACOGB_CHECK_ARG(T != nullptr && T->order == 3 && T->dimensions && T->mode_types && T->indices,
                   "order-3 operand B: expected an order-3 tensor");
  const bool dense0 = T->mode_types[0] == taco_mode_dense;
  TACOGB_CHECK_ARG((dense0 || T->mode_types[0] == taco_mode_sparse) &&
                       T->mode_types[1] == taco_mode_sparse && T->mode_types[2] == taco_mode_sparse,
                   "operand B: expected {Sparse,Sparse,Sparse} or {Dense,Sparse,Sparse}");
  for (int m = 0; m < 3; m++)
    TACOGB_CHECK_ARG(T->mode_ordering == nullptr || T->mode_ordering[m] == m,
                     "operand B: expected mode ordering (0, 1, 2)");
  TACOGB_CHECK_ARG(T->indices[1] && T->indices[2] && (dense0 || T->indices[0]),
                   "operand B: missing indices");
  const int vt = value_type_of_csize(T->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "operand B: unsupported csize %d",
                   T->csize);
  tacogb_csf3 b{};
  for (int m = 0; m < 3; m++) b.dims[m] = T->dimensions[m];
  b.vtype = vt;
  const int32_t* crd0 = nullptr;
  if (dense0) {
    b.n0 = b.dims[0];
  } else {
    const int32_t* pos0 = (const int32_t*)T->indices[0][0];
    TACOGB_CHECK_ARG(pos0 != nullptr, "operand B: null level-0 pos");
    int32_t p0 = 0;
    if (int rc = read_i32(pos0, &p0)) return rc;
    if (int rc = read_i32(pos0 + 1, &b.n0)) return rc;
    TACOGB_CHECK_ARG(p0 == 0 && b.n0 >= 0 && b.n0 <= b.dims[0],
                     "operand B: level-0 pos must be {0, n} with n <= %d", b.dims[0]);
    crd0 = (const int32_t*)T->indices[0][1];
  }
  const int32_t* pos1 = (const int32_t*)T->indices[1][0];
  const int32_t* crd1 = (const int32_t*)T->indices[1][1];
  const int32_t* pos2 = (const int32_t*)T->indices[2][0];
  const int32_t* crd2 = (const int32_t*)T->indices[2][1];
  TACOGB_CHECK_ARG(pos1 != nullptr && pos2 != nullptr, "operand B: null pos");
  if (int rc = read_i32(pos1 + b.n0, &b.nfib)) return rc;
  // checked before pos2 is read at it: a valid level 1 holds at most n0 * dims[1] fibers
  TACOGB_CHECK_ARG(b.nfib >= 0 && (int64_t)b.nfib <= (int64_t)b.n0 * b.dims[1],
                   "operand B: level-1 pos ends at %d, more fibers than %d x %d", b.nfib, b.n0,
                   b.dims[1]);
  int32_t nnz = 0;
  if (int rc = read_i32(pos2 + b.nfib, &nnz)) return rc;
  b.nnz = nnz;
  Operand o0p, o0, op1, oc1, op2, oc2, ov;
  if (crd0) {
    if (int rc = stage_checked_level("order-3 operand B level 0", 1, b.dims[0], b.n0,
                                     T->indices[0][0], crd0, nullptr, 0, base + 60, st, o0p, o0,
                                     nullptr))
      return rc;
    b.crd0 = (const int32_t*)o0.dev;
  }
  if (int rc = stage_checked_level("order-3 operand B level 1", b.n0, b.dims[1], b.nfib, pos1,
                                   crd1, nullptr, 0, base + 1, st, op1, oc1, nullptr))
    return rc;
  b.pos1 = (const int32_t*)op1.dev;
  b.crd1 = (const int32_t*)oc1.dev;
  if (leaf) {
    if (int rc = stage_checked_level("order-3 operand B level 2", b.nfib, b.dims[2], b.nnz, pos2,
                                     crd2, T->vals, (size_t)b.nnz * value_bytes(vt), base + 3, st,
                                     op2, oc2, &ov))
      return rc;
    b.pos2 = (const int32_t*)op2.dev;
    b.crd2 = (const int32_t*)oc2.dev;
    b.vals = ov.dev;
  }
  out = b;
  return 0;
}

// The shared body of the three compute entry points: B and the dense operands staged, the
// result written in place (device-accessible) or through a staging buffer.
template <class Run>
int t3_compute(taco_tensor_t* A, taco_tensor_t* B, size_t abytes, int nops,
               taco_tensor_t* const* ops, const size_t* op_bytes, Run run) {
  TACOGB_CHECK_ARG(A->vals != nullptr || abytes == 0, "result values not assembled");
  cudaStream_t st = lib_stream();
  tacogb_csf3 b;
  if (int rc = csf3_operand(B, 30, st, b)) return rc;
  const void* dev[2] = {nullptr, nullptr};
  Operand o[2];
  for (int q = 0; q < nops; q++) {
    if (int rc = stage_in(o[q], ops[q]->vals, op_bytes[q], 37 + q, st)) return rc;
    dev[q] = o[q].dev;
  }
  void* adev = A->vals;
  const bool staged = !device_accessible(A->vals);
  if (staged) {
    adev = stage_buffer(39, abytes);
    if (!adev) return TACOGB_ERR_ALLOC;
  }
  if (int rc = run(b, dev, adev, st)) return rc;
  if (staged && abytes)
    TACOGB_CUDA_TRY(cudaMemcpyAsync(A->vals, adev, abytes, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return consume_device_status();
}

int t3_assemble(taco_tensor_t* A, taco_tensor_t* B, size_t elems) {
  const int vt = value_type_of_csize(A->csize);
  TACOGB_CHECK_ARG(vt == TACOGB_F64 || vt == TACOGB_F32, "result: unsupported csize %d", A->csize);
  const bool managed = B->vals != nullptr && device_accessible(B->vals);
  void* p = alloc_result(elems * value_bytes(vt), managed);
  if (!p) return TACOGB_ERR_ALLOC;
  A->vals = (uint8_t*)p;
  return 0;
}

int check_same_csize(const taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C,
                     const taco_tensor_t* D) {
  TACOGB_CHECK_ARG(A->csize == B->csize && C->csize == B->csize && (!D || D->csize == B->csize),
                   "operand component sizes differ");
  return 0;
}

int check_ttv(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c) {
  if (int rc = check_dense_order(A, 2, "ttv result A")) return rc;
  if (int rc = check_dense_order(c, 1, "ttv operand c")) return rc;
  TACOGB_CHECK_ARG(B != nullptr && B->order == 3 && B->dimensions, "ttv: B must be order 3");
  TACOGB_CHECK_ARG(A->dimensions[0] == B->dimensions[0] && A->dimensions[1] == B->dimensions[1],
                   "ttv: A is %dx%d, B is %dx%dx%d", A->dimensions[0], A->dimensions[1],
                   B->dimensions[0], B->dimensions[1], B->dimensions[2]);
  TACOGB_CHECK_ARG(c->dimensions[0] == B->dimensions[2], "ttv: c has %d entries, B's k is %d",
                   c->dimensions[0], B->dimensions[2]);
  return check_same_csize(A, B, c, nullptr);
}

int check_ttm(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C) {
  if (int rc = check_dense_order(A, 3, "ttm result A")) return rc;
  if (int rc = check_dense_order(C, 2, "ttm operand C")) return rc;
  TACOGB_CHECK_ARG(B != nullptr && B->order == 3 && B->dimensions, "ttm: B must be order 3");
  TACOGB_CHECK_ARG(A->dimensions[0] == B->dimensions[0] && A->dimensions[1] == B->dimensions[1] &&
                       A->dimensions[2] == C->dimensions[1],
                   "ttm: A's shape does not match B and C");
  TACOGB_CHECK_ARG(C->dimensions[0] == B->dimensions[2], "ttm: C has %d rows, B's k is %d",
                   C->dimensions[0], B->dimensions[2]);
  return check_same_csize(A, B, C, nullptr);
}

int check_mttkrp(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (int rc = check_dense_order(A, 2, "mttkrp result A")) return rc;
  if (int rc = check_dense_order(C, 2, "mttkrp operand C")) return rc;
  if (int rc = check_dense_order(D, 2, "mttkrp operand D")) return rc;
  TACOGB_CHECK_ARG(B != nullptr && B->order == 3 && B->dimensions, "mttkrp: B must be order 3");
  const int32_t J = A->dimensions[1];
  TACOGB_CHECK_ARG(A->dimensions[0] == B->dimensions[0], "mttkrp: A has %d rows, B's i is %d",
                   A->dimensions[0], B->dimensions[0]);
  TACOGB_CHECK_ARG(C->dimensions[0] == B->dimensions[1] && C->dimensions[1] == J,
                   "mttkrp: C must be %d x %d", B->dimensions[1], J);
  TACOGB_CHECK_ARG(D->dimensions[0] == B->dimensions[2] && D->dimensions[1] == J,
                   "mttkrp: D must be %d x %d", B->dimensions[2], J);
  return check_same_csize(A, B, C, D);
}

size_t vbytes_of(const taco_tensor_t* t) { return value_bytes(value_type_of_csize(t->csize)); }

}  // namespace
}  // extern "C++"

int tacogb_ttv_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c) {
  if (int rc = check_ttv(A, B, c)) return rc;
  return t3_assemble(A, B, (size_t)A->dimensions[0] * A->dimensions[1]);
}
int tacogb_ttv_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c) {
  if (int rc = check_ttv(A, B, c)) return rc;
  const size_t vb = vbytes_of(B);
  taco_tensor_t* ops[1] = {c};
  const size_t ob[1] = {(size_t)c->dimensions[0] * vb};
  return t3_compute(A, B, (size_t)A->dimensions[0] * A->dimensions[1] * vb, 1, ops, ob,
                    [](const tacogb_csf3& b, const void* const* d, void* a, cudaStream_t st) {
                      return ttv_run(&b, d[0], a, true, TACOGB_VARIANT_AUTO, st);
                    });
}
int tacogb_ttv_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c) {
  if (int rc = tacogb_ttv_assemble(A, B, c)) return rc;
  return tacogb_ttv_compute(A, B, c);
}

int tacogb_ttm_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C) {
  if (int rc = check_ttm(A, B, C)) return rc;
  return t3_assemble(A, B, (size_t)A->dimensions[0] * A->dimensions[1] * A->dimensions[2]);
}
int tacogb_ttm_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C) {
  if (int rc = check_ttm(A, B, C)) return rc;
  const size_t vb = vbytes_of(B);
  const int32_t L = C->dimensions[1];
  taco_tensor_t* ops[1] = {C};
  const size_t ob[1] = {(size_t)C->dimensions[0] * L * vb};
  return t3_compute(A, B, (size_t)A->dimensions[0] * A->dimensions[1] * L * vb, 1, ops, ob,
                    [L](const tacogb_csf3& b, const void* const* d, void* a, cudaStream_t st) {
                      return ttm_run(&b, L, d[0], a, true, TACOGB_VARIANT_AUTO, st);
                    });
}
int tacogb_ttm_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C) {
  if (int rc = tacogb_ttm_assemble(A, B, C)) return rc;
  return tacogb_ttm_compute(A, B, C);
}

int tacogb_mttkrp_assemble(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C,
                           taco_tensor_t* D) {
  if (int rc = check_mttkrp(A, B, C, D)) return rc;
  return t3_assemble(A, B, (size_t)A->dimensions[0] * A->dimensions[1]);
}
// MTTKRP over large host operands: the fiber level (pos2, crd2, values: nearly all of B's
// bytes) is copied chunk by chunk and multiplied by D as it lands, into fiber rows kept on the
// device; then B's upper levels and C are staged, the combine runs and A comes back.
int mttkrp_pipelined(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D,
                     int32_t J, int vt, bool* applied) {
  *applied = false;
  const size_t vb = value_bytes(vt);
  const bool dense0 = B->mode_types[0] == taco_mode_dense;
  const int32_t* pos0 = dense0 ? nullptr : (const int32_t*)B->indices[0][0];
  const int32_t* pos1 = (const int32_t*)B->indices[1][0];
  const int32_t* pos2 = (const int32_t*)B->indices[2][0];
  std::initializer_list<const void*> arrays = {
      pos1, B->indices[1][1], pos2, B->indices[2][1], B->vals, C->vals, D->vals, A->vals,
      dense0 ? (const void*)B->vals : (const void*)pos0,
      dense0 ? (const void*)B->vals : (const void*)B->indices[0][1]};
  for (const void* p : arrays)
    if (p == nullptr || device_accessible(p)) return 0;
  const int32_t n0 = dense0 ? B->dimensions[0] : pos0[1];
  // checked before pos1[n0] is read on the host
  TACOGB_CHECK_ARG(n0 >= 0 && n0 <= B->dimensions[0] && (dense0 || pos0[0] == 0),
                   "order-3 operand B: level-0 pos must be {0, n} with n <= %d",
                   B->dimensions[0]);
  const int32_t nfib = pos1[n0];
  TACOGB_CHECK_ARG(nfib >= 0 && (int64_t)nfib <= (int64_t)n0 * B->dimensions[1],
                   "order-3 operand B: level-1 pos ends at %d, more fibers than %d x %d", nfib,
                   n0, B->dimensions[1]);
  const int32_t nnz = pos2[nfib];
  if (!pipeline_applies(nnz, arrays) || J <= 0) return 0;
  *applied = true;
  // the fiber level as a CSR of fibers (rows) over B's last mode
  int32_t fdims[2] = {nfib, B->dimensions[2]};
  taco_mode_t ftypes[2] = {taco_mode_dense, taco_mode_sparse};
  uint8_t* fl1[2] = {B->indices[2][0], B->indices[2][1]};
  uint8_t** fidx[2] = {nullptr, fl1};
  taco_tensor_t F{};
  F.order = 2;
  F.dimensions = fdims;
  F.csize = B->csize;
  F.mode_types = ftypes;
  F.indices = fidx;
  F.vals = B->vals;
  void* T = stage_buffer(40, (size_t)nfib * J * vb + 64);
  if (!T) return TACOGB_ERR_ALLOC;
  FiberSpmmChunks fibers;
  if (int rc = csr_product_pipelined("order-3 operand B level 2", &F, vt, nfib, B->dimensions[2],
                                     nnz, D->vals, (size_t)B->dimensions[2] * J * vb, J, vt,
                                     nullptr, (size_t)J * vb, fibers, nullptr, 0, false, T))
    return rc;
  cudaStream_t st = lib_stream();
  tacogb_csf3 b;
  if (int rc = csf3_operand(B, 30, st, b, false)) return rc;
  b.nnz = nnz;
  Operand oc;
  if (int rc = stage_in(oc, C->vals, (size_t)C->dimensions[0] * J * vb, 37, st)) return rc;
  const size_t abytes = (size_t)A->dimensions[0] * J * vb;
  void* adev = stage_buffer(39, abytes + 64);
  if (!adev) return TACOGB_ERR_ALLOC;
  if (abytes) TACOGB_CUDA_TRY(cudaMemsetAsync(adev, 0, abytes, st));
  if (int rc = mttkrp_combine_launch(&b, J, oc.dev, T, adev, st)) return rc;
  if (abytes) TACOGB_CUDA_TRY(cudaMemcpyAsync(A->vals, adev, abytes, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return consume_device_status();
}

int tacogb_mttkrp_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (int rc = check_mttkrp(A, B, C, D)) return rc;
  const size_t vb = vbytes_of(B);
  const int32_t J = A->dimensions[1];
  {
    bool applied = false;
    const int rc = mttkrp_pipelined(A, B, C, D, J, value_type_of_csize(B->csize), &applied);
    if (applied || rc) return rc;
  }
  taco_tensor_t* ops[2] = {C, D};
  const size_t ob[2] = {(size_t)C->dimensions[0] * J * vb, (size_t)D->dimensions[0] * J * vb};
  return t3_compute(A, B, (size_t)A->dimensions[0] * J * vb, 2, ops, ob,
                    [J](const tacogb_csf3& b, const void* const* d, void* a, cudaStream_t st) {
                      return mttkrp_run(&b, J, d[0], d[1], a, TACOGB_VARIANT_AUTO, st);
                    });
}
int tacogb_mttkrp_evaluate(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C,
                           taco_tensor_t* D) {
  if (int rc = tacogb_mttkrp_assemble(A, B, C, D)) return rc;
  return tacogb_mttkrp_compute(A, B, C, D);
}

#define TACOGB_SHIM3(name)                                                                \
  int _shim_tacogb_##name(void** a) {                                                     \
    return tacogb_##name((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2]); \
  }
#define TACOGB_SHIM4(name)                                                                \
  int _shim_tacogb_##name(void** a) {                                                     \
    return tacogb_##name((taco_tensor_t*)a[0], (taco_tensor_t*)a[1], (taco_tensor_t*)a[2], \
                         (taco_tensor_t*)a[3]);                                           \
  }
TACOGB_SHIM3(ttv_assemble)
TACOGB_SHIM3(ttv_compute)
TACOGB_SHIM3(ttv_evaluate)
TACOGB_SHIM3(ttm_assemble)
TACOGB_SHIM3(ttm_compute)
TACOGB_SHIM3(ttm_evaluate)
TACOGB_SHIM4(mttkrp_assemble)
TACOGB_SHIM4(mttkrp_compute)
TACOGB_SHIM4(mttkrp_evaluate)
#undef TACOGB_SHIM3
#undef TACOGB_SHIM4

// ------------------------------------------------------------------ formats ---------------

int tacogb_spmv_dcsr(const tacogb_dcsr* A, const void* x, void* y, int32_t dense_y, void* stream) {
  return spmv_dcsr_run(A, x, y, dense_y != 0, (cudaStream_t)stream);
}
int tacogb_spmm_dcsr(const tacogb_dcsr* A, int32_t N, const void* B, void* C, void* stream) {
  return spmm_dcsr_run(A, N, B, C, (cudaStream_t)stream);
}
int tacogb_spmv_csc(const tacogb_csr* A, const void* x, void* y, void* stream) {
  return spmv_csc_run(A, x, y, (cudaStream_t)stream);
}
int tacogb_csc_to_csr(int32_t rows, int32_t cols, int64_t nnz, const int32_t* colpos,
                      const int32_t* rowidx, const void* vals, int32_t vtype, int32_t* pos,
                      int32_t* crd, void* out_vals, void* stream) {
  return csc_to_csr_run(rows, cols, nnz, colpos, rowidx, vals, vtype, pos, crd, out_vals,
                        (cudaStream_t)stream);
}
int tacogb_densify(int32_t n, int64_t k, const int32_t* idx, const void* vals, int32_t vtype,
                   void* out, void* stream) {
  return densify_run(n, k, idx, vals, vtype, out, (cudaStream_t)stream);
}

}  // extern "C"
