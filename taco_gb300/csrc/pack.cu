// COO -> CSR packing on the GPU: the sort + pack that taco runs on the host when a tensor with
// inserted coordinates is first used (TensorBase::pack, src/tensor.cpp:295-463: permute the
// coordinates to the mode ordering, qsort them lexicographically (:420-422), then the generated
// "pack" merges the sorted coordinate buffer into the target format, summing duplicates
// (src/tensor.cpp:303-311 and the COO-buffer assembly lowered at :935-1020)).
//
// Here the (row, col) pairs, in any order and with duplicates, are sorted by a stable LSD
// radix sort (8-bit digits over the column bits, then the row bits) that carries each entry's
// original index; duplicates therefore meet in input order and are summed in that order, so
// the result is deterministic (taco's qsort is not stable: for values whose sum depends on the
// order, taco's last bits are arbitrary).  Each run of equal keys becomes one CSR entry; row
// starts are scattered into pos.  Explicit zeros (including duplicates that cancel) are kept,
// as taco's pack keeps them.

#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace tacogb {

namespace {

constexpr int kPkThreads = 256;
constexpr int kPkRounds = 8;                        // items per thread per tile
constexpr int kPkTile = kPkThreads * kPkRounds;     // 2048 items per block
constexpr int kPkWarps = kPkThreads / 32;
constexpr int kRadix = 256;

// Per-tile digit histogram, stored digit-major (hist[d * nblocks + b]) so that one exclusive
// scan of the whole array gives every (digit, tile) its global output offset in stable order.
__global__ void __launch_bounds__(kPkThreads)
pk_hist(const uint32_t* __restrict__ keys, int64_t n, int shift, int32_t* __restrict__ hist,
        int32_t nblocks) {
  __shared__ int32_t h[kRadix];
  const int tid = threadIdx.x;
  h[tid] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kPkTile;
#pragma unroll 4
  for (int j = 0; j < kPkRounds; j++) {
    const int64_t i = base + j * kPkThreads + tid;
    if (i < n) atomicAdd(&h[(__ldg(keys + i) >> shift) & (kRadix - 1)], 1);
  }
  __syncthreads();
  hist[(int64_t)tid * nblocks + blockIdx.x] = h[tid];
}

// Stable scatter of one tile by the digit at `shift` of `keys`: the tile's records are ranked
// (record j*256 + t of the tile follows every earlier record of the same digit), reordered by
// digit in shared memory, then written out so that each digit's records of the tile form one
// contiguous run at offs[d][block] (coalesced writes instead of one 4-byte store per record
// into a different place).  The rank inside a round of 256 records comes from
// __match_any_sync within each warp and per-warp digit counts; run[d] carries earlier rounds.
// idx_in == nullptr means identity indices (the first pass).
__global__ void __launch_bounds__(kPkThreads)
pk_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ other,
           const int32_t* __restrict__ idx_in, uint32_t* __restrict__ keys_out,
           uint32_t* __restrict__ other_out, int32_t* __restrict__ idx_out, int64_t n, int shift,
           const int32_t* __restrict__ offs, int32_t nblocks) {
  __shared__ uint32_t s_key[kPkTile], s_oth[kPkTile];
  __shared__ int32_t s_idx[kPkTile];
  __shared__ int32_t loc[kRadix + 1];  // tile-local start of every digit
  __shared__ int32_t run[kRadix];
  __shared__ int32_t wcnt[kPkWarps][kRadix];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * kPkTile;
  const int cnt = (int)(n - base < kPkTile ? n - base : kPkTile);
  uint32_t k[kPkRounds], o[kPkRounds];
  int32_t x[kPkRounds];
  run[tid] = 0;
#pragma unroll
  for (int w = 0; w < kPkWarps; w++) wcnt[w][tid] = 0;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kPkRounds; j++) {
    const int i = j * kPkThreads + tid;
    if (i < cnt) {
      k[j] = keys[base + i];
      o[j] = other[base + i];
      x[j] = idx_in ? idx_in[base + i] : (int32_t)(base + i);
      atomicAdd(&run[(k[j] >> shift) & (kRadix - 1)], 1);
    }
  }
  __syncthreads();
  if (tid == 0) {  // exclusive scan of the tile's 256 digit counts
    int acc = 0;
    for (int d = 0; d < kRadix; d++) {
      loc[d] = acc;
      acc += run[d];
    }
    loc[kRadix] = acc;
  }
  __syncthreads();
  run[tid] = loc[tid];
  __syncthreads();
  const unsigned lt = (1u << lane) - 1;
#pragma unroll
  for (int j = 0; j < kPkRounds; j++) {
    const int i = j * kPkThreads + tid;
    const bool valid = i < cnt;
    const int d = valid ? (int)((k[j] >> shift) & (kRadix - 1)) : kRadix;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int intra = __popc(peers & lt);
    if (valid && intra == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pre = 0;
      for (int w = 0; w < warp; w++) pre += wcnt[w][d];
      const int p = run[d] + pre + intra;
      s_key[p] = k[j];
      s_oth[p] = o[j];
      s_idx[p] = x[j];
    }
    __syncthreads();
    int add = 0;
#pragma unroll
    for (int w = 0; w < kPkWarps; w++) {
      add += wcnt[w][tid];
      wcnt[w][tid] = 0;
    }
    run[tid] += add;
    __syncthreads();
  }
  for (int p = tid; p < cnt; p += kPkThreads) {
    const uint32_t kk = s_key[p];
    const int d = (int)((kk >> shift) & (kRadix - 1));
    const int64_t dst = (int64_t)offs[(int64_t)d * nblocks + blockIdx.x] + (p - loc[d]);
    keys_out[dst] = kk;
    other_out[dst] = s_oth[p];
    idx_out[dst] = s_idx[p];
  }
}

// ---- exclusive scan of int32 counts (totals below 2^31) ------------------------------------

constexpr int kScanItems = 1024;  // per block: 256 threads x 4

__global__ void __launch_bounds__(256)
pk_scan_partials(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ partial) {
  __shared__ int64_t s[256];
  const int64_t base = (int64_t)blockIdx.x * kScanItems;
  int64_t v = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int64_t i = base + threadIdx.x * 4 + j;
    if (i < n) v += in[i];
  }
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// One block: exclusive scan of the block partials, in place.
__global__ void __launch_bounds__(1024) pk_scan_top(int64_t* __restrict__ partial, int64_t nb) {
  __shared__ int64_t s[1024];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    const int64_t v = i < nb ? partial[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
      const int64_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) partial[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += s[1023];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256)
pk_scan_apply(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ partial,
              int32_t* __restrict__ out) {
  __shared__ int64_t s[256];
  const int64_t base = (int64_t)blockIdx.x * kScanItems;
  int32_t v[4];
  int64_t t = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int64_t i = base + threadIdx.x * 4 + j;
    v[j] = i < n ? in[i] : 0;
    t += v[j];
  }
  s[threadIdx.x] = t;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const int64_t u = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += u;
    __syncthreads();
  }
  int64_t run = partial[blockIdx.x] + s[threadIdx.x] - t;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int64_t i = base + threadIdx.x * 4 + j;
    if (i < n) out[i] = (int32_t)run;
    run += v[j];
  }
}

// ---- runs of equal keys -> CSR --------------------------------------------------------------

// head[i] = 1 where a run of equal (row, col) starts; *bad = 1 for a coordinate out of range.
__global__ void pk_heads(const uint32_t* __restrict__ r, const uint32_t* __restrict__ c, int64_t n,
                         uint32_t rows, uint32_t cols, int32_t* __restrict__ head,
                         int* __restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t ri = r[i], ci = c[i];
  if (ri >= rows || ci >= cols) *bad = 1;
  head[i] = (i == 0 || ri != r[i - 1] || ci != c[i - 1]) ? 1 : 0;
}

// Thread i at the head of a run writes its CSR entry (column, and the sum of the run's values in
// input order) at slot opos[i], and the starts of the rows from the previous entry's row + 1 up
// to its own; the last entry also closes the remaining rows.  Every index written is checked
// against its array, so out-of-range coordinates (reported by pk_heads) cannot write outside.
template <typename V>
__global__ void pk_emit(const uint32_t* __restrict__ r, const uint32_t* __restrict__ c,
                        const int32_t* __restrict__ idx, const int32_t* __restrict__ head,
                        const int32_t* __restrict__ opos, int64_t n, const V* __restrict__ vin,
                        uint32_t rows, int32_t* __restrict__ pos, int32_t* __restrict__ crd,
                        V* __restrict__ vout) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t ri = r[i];
  if (head[i]) {
    const int32_t o = opos[i];
    const uint32_t ci = c[i];
    V sum = vin[idx[i]];
    for (int64_t j = i + 1; j < n && r[j] == ri && c[j] == ci; j++) sum += vin[idx[j]];
    crd[o] = (int32_t)ci;
    vout[o] = sum;
    const int64_t rp = (i == 0) ? -1 : (int64_t)r[i - 1];
    if ((int64_t)ri != rp) {
      const int64_t hi = min((int64_t)ri, (int64_t)rows);
      for (int64_t q = rp + 1; q <= hi; q++) pos[q] = o;
    }
  }
  if (i == n - 1) {
    const int32_t total = opos[i] + head[i];
    for (int64_t q = min((int64_t)ri, (int64_t)rows) + 1; q <= rows; q++) pos[q] = total;
  }
}

inline int bits_for(uint32_t extent) {  // bits that hold 0 .. extent-1
  int b = 1;
  while (b < 32 && (extent - 1) >> b) b++;
  return b;
}

}  // namespace

int pack_csr(int32_t rows, int32_t cols, int64_t n, const int32_t* coord_rows,
             const int32_t* coord_cols, const void* vals, int32_t vtype, int32_t* pos,
             int32_t* crd, void* out_vals, int64_t* nnz, cudaStream_t st) {
  TACOGB_CHECK_ARG(rows >= 0 && cols >= 0 && n >= 0, "pack: negative size");
  TACOGB_CHECK_ARG(n < (1ll << 31), "pack: %lld coordinates exceed int32 positions", (long long)n);
  TACOGB_CHECK_ARG(vtype == TACOGB_F64 || vtype == TACOGB_F32, "pack: value type %d", vtype);
  TACOGB_CHECK_ARG(pos != nullptr && nnz != nullptr, "pack: null pos or nnz");
  TACOGB_CHECK_ARG(n == 0 || (coord_rows && coord_cols && vals && crd && out_vals),
                   "pack: null coordinate, value or output array");
  if (n > 0) TACOGB_CHECK_ARG(rows > 0 && cols > 0, "pack: coordinates of an empty matrix");
  if (n == 0) {
    TACOGB_CUDA_TRY(cudaMemsetAsync(pos, 0, ((size_t)rows + 1) * sizeof(int32_t), st));
    *nnz = 0;
    return 0;
  }
  const int32_t nblocks = (int32_t)((n + kPkTile - 1) / kPkTile);
  const int64_t hist_n = (int64_t)kRadix * nblocks;
  const int64_t scan_n = std::max<int64_t>(hist_n, n);
  const int64_t nparts = (scan_n + kScanItems - 1) / kScanItems;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t a4 = al((size_t)n * 4);
  const size_t need = 6 * a4 + al((size_t)hist_n * 4) + al((size_t)nparts * 8) + 2 * a4 + 256;
  unsigned char* ws = (unsigned char*)scratch(need, 5);
  if (!ws) return last_code();
  uint32_t* rA = (uint32_t*)ws;
  uint32_t* rB = (uint32_t*)(ws + a4);
  uint32_t* cA = (uint32_t*)(ws + 2 * a4);
  uint32_t* cB = (uint32_t*)(ws + 3 * a4);
  int32_t* xA = (int32_t*)(ws + 4 * a4);
  int32_t* xB = (int32_t*)(ws + 5 * a4);
  int32_t* hist = (int32_t*)(ws + 6 * a4);
  int64_t* parts = (int64_t*)(ws + 6 * a4 + al((size_t)hist_n * 4));
  int32_t* head = (int32_t*)((unsigned char*)parts + al((size_t)nparts * 8));
  int32_t* opos = (int32_t*)((unsigned char*)head + a4);
  int* bad = (int*)((unsigned char*)opos + a4);
  TACOGB_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));

  auto scan = [&](const int32_t* in, int64_t m, int32_t* out) -> int {
    const int64_t nb = (m + kScanItems - 1) / kScanItems;
    TACOGB_LAUNCH("pack_scan_partials", st,
                  pk_scan_partials<<<(unsigned)nb, 256, 0, st>>>(in, m, parts));
    TACOGB_LAUNCH("pack_scan_top", st, pk_scan_top<<<1, 1024, 0, st>>>(parts, nb));
    TACOGB_LAUNCH("pack_scan_apply", st,
                  pk_scan_apply<<<(unsigned)nb, 256, 0, st>>>(in, m, parts, out));
    return 0;
  };
  // LSD passes: column digits, then row digits.  Each pass reads (src_r, src_c, src_x) and
  // writes the other buffer of the pair; the first reads the caller's arrays (src_x null:
  // identity indices).
  const uint32_t* src_r = (const uint32_t*)coord_rows;
  const uint32_t* src_c = (const uint32_t*)coord_cols;
  const int32_t* src_x = nullptr;
  int buf = 0;
  auto pass = [&](bool by_col, int shift) -> int {
    uint32_t* dr = buf ? rB : rA;
    uint32_t* dc = buf ? cB : cA;
    int32_t* dx = buf ? xB : xA;
    const uint32_t* key = by_col ? src_c : src_r;
    const uint32_t* oth = by_col ? src_r : src_c;
    TACOGB_LAUNCH("pack_hist", st,
                  pk_hist<<<(unsigned)nblocks, kPkThreads, 0, st>>>(key, n, shift, hist, nblocks));
    if (int rc = scan(hist, hist_n, hist)) return rc;
    TACOGB_LAUNCH("pack_scatter", st,
                  pk_scatter<<<(unsigned)nblocks, kPkThreads, 0, st>>>(
                      key, oth, src_x, by_col ? dc : dr, by_col ? dr : dc, dx, n, shift, hist,
                      nblocks));
    src_r = dr;
    src_c = dc;
    src_x = dx;
    buf ^= 1;
    return 0;
  };
  const int cbits = bits_for((uint32_t)cols), rbits = bits_for((uint32_t)rows);
  for (int shift = 0; shift < cbits; shift += 8)
    if (int rc = pass(true, shift)) return rc;
  for (int shift = 0; shift < rbits; shift += 8)
    if (int rc = pass(false, shift)) return rc;
  const uint32_t* rcur = src_r;
  const uint32_t* ccur = src_c;
  const int32_t* xcur = src_x;
  const unsigned eb = (unsigned)((n + 255) / 256);
  TACOGB_LAUNCH("pack_heads", st,
                pk_heads<<<eb, 256, 0, st>>>(rcur, ccur, n, (uint32_t)rows, (uint32_t)cols, head,
                                             bad));
  if (int rc = scan(head, n, opos)) return rc;
  if (vtype == TACOGB_F64)
    TACOGB_LAUNCH("pack_emit", st,
                  pk_emit<double><<<eb, 256, 0, st>>>(rcur, ccur, xcur, head, opos, n,
                                                      (const double*)vals, (uint32_t)rows, pos,
                                                      crd, (double*)out_vals));
  else
    TACOGB_LAUNCH("pack_emit", st,
                  pk_emit<float><<<eb, 256, 0, st>>>(rcur, ccur, xcur, head, opos, n,
                                                     (const float*)vals, (uint32_t)rows, pos, crd,
                                                     (float*)out_vals));
  int32_t h[2] = {0, 0};
  int hbad = 0;
  TACOGB_CUDA_TRY(cudaMemcpyAsync(&h[0], opos + n - 1, 4, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaMemcpyAsync(&h[1], head + n - 1, 4, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  TACOGB_CHECK_ARG(hbad == 0, "pack: a coordinate lies outside the %d x %d matrix", rows, cols);
  *nnz = (int64_t)h[0] + h[1];
  return 0;
}

}  // namespace tacogb

namespace tacogb {
namespace {

// taco's coordinate buffer (n records of int32 row, int32 column, value) -> separate arrays.
template <typename V>
__global__ void pk_split_records(const unsigned char* __restrict__ buf, int64_t n,
                                 int32_t* __restrict__ r, int32_t* __restrict__ c,
                                 V* __restrict__ v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned char* rec = buf + i * (int64_t)(8 + sizeof(V));
  r[i] = *reinterpret_cast<const int32_t*>(rec);
  c[i] = *reinterpret_cast<const int32_t*>(rec + 4);
  v[i] = *reinterpret_cast<const V*>(rec + 8);
}

}  // namespace

int pack_split_records(const void* buf, int64_t n, int32_t vtype, int32_t* r, int32_t* c,
                       void* v, cudaStream_t st) {
  if (n == 0) return 0;
  const unsigned g = (unsigned)((n + 255) / 256);
  if (vtype == TACOGB_F64)
    TACOGB_LAUNCH("pack_split_records", st,
                  pk_split_records<double><<<g, 256, 0, st>>>((const unsigned char*)buf, n, r, c,
                                                              (double*)v));
  else
    TACOGB_LAUNCH("pack_split_records", st,
                  pk_split_records<float><<<g, 256, 0, st>>>((const unsigned char*)buf, n, r, c,
                                                             (float*)v));
  return 0;
}

}  // namespace tacogb

extern "C" int tacogb_pack_csr(int32_t rows, int32_t cols, int64_t n, const int32_t* coord_rows,
                               const int32_t* coord_cols, const void* vals, int32_t vtype,
                               int32_t* pos, int32_t* crd, void* out_vals, int64_t* nnz,
                               void* stream) {
  return tacogb::pack_csr(rows, cols, n, coord_rows, coord_cols, vals, vtype, pos, crd, out_vals,
                          nnz, (cudaStream_t)stream);
}

