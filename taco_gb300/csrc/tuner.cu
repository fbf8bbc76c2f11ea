// Sparsity features and the MLP cost model that picks each batched matrix's work-unit kind.
//
// Features (one CTA per matrix; all statistics exact except the Gini coefficient, which is taken
// over a row-length histogram with exact bins below 2048 and 16 bins per octave above):
//   0 log2(rows+1)   1 log2(nnz+1)   2 log2(mean+1)   3 std/mean of row lengths
//   4 log2(max+1)    5 Gini of row lengths            6 max |j-i| / cols (bandwidth)
//   7 mean |j-i| / cols                8 fraction of empty rows   9 log2(cols+1)
//
// The model: F=10 inputs (z-scored with the training set's statistics) -> 32 ReLU -> 32 ReLU ->
// K=6 outputs, one per kind: the predicted log2 of the kind's SM cycles per (row + nonzero).
// Training minimises the masked mean squared error with Adam.  Gradients are deterministic: each
// block keeps its samples' activations in shared memory and reduces every parameter's gradient
// over its samples in a fixed order; a second kernel sums the block partials in block order.
// The model only chooses which kernel runs; the arithmetic of every kind is the same.

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace tacogb {
namespace {

constexpr int F = TACOGB_MLP_FEATURES;
constexpr int H = TACOGB_MLP_HIDDEN;
constexpr int K = TACOGB_MLP_KINDS;
// parameter layout: W1[H][F] b1[H] W2[H][H] b2[H] W3[K][H] b3[K]
constexpr int OW1 = 0, OB1 = OW1 + H * F, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H,
              OB3 = OW3 + K * H, NPARAM = OB3 + K;

// ------------------------------------------------------------------------- features ------

constexpr int kExactBins = 2048;
constexpr int kLogBins = 20 * 16;  // octaves 2^11 .. 2^30, 16 bins each
constexpr int kBins = kExactBins + kLogBins;
constexpr int kFeatBlock = 256;

__device__ __forceinline__ int len_bin(uint32_t L) {
  if (L < (uint32_t)kExactBins) return (int)L;
  const int e = 31 - __clz((int)L);  // 11..30 (row lengths are int32)
  const int sub = (int)((L >> (e - 4)) & 15u);
  const int b = kExactBins + (min(e, 30) - 11) * 16 + sub;
  return b;
}

struct FeatDesc {
  const int32_t* pos;
  const int32_t* crd;
  int32_t rows, cols, nnz, pad;
};

__global__ void __launch_bounds__(kFeatBlock)
batch_features(const FeatDesc* __restrict__ desc, float* __restrict__ out) {
  __shared__ uint32_t cnt[kBins];
  __shared__ unsigned long long lsum[kLogBins];
  __shared__ unsigned long long s_sq, s_band_sum;
  __shared__ int s_max, s_band_max, s_empty;
  const FeatDesc d = desc[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int b = tid; b < kBins; b += kFeatBlock) cnt[b] = 0;
  for (int b = tid; b < kLogBins; b += kFeatBlock) lsum[b] = 0;
  if (tid == 0) {
    s_sq = 0;
    s_band_sum = 0;
    s_max = 0;
    s_band_max = 0;
    s_empty = 0;
  }
  __syncthreads();
  // row lengths: one thread per row
  unsigned long long sq = 0;
  int mx = 0, empty = 0;
  for (int i = tid; i < d.rows; i += kFeatBlock) {
    const uint32_t L = (uint32_t)(__ldg(d.pos + i + 1) - __ldg(d.pos + i));
    sq += (unsigned long long)L * L;
    mx = max(mx, (int)L);
    empty += (L == 0);
    const int b = len_bin(L);
    atomicAdd(&cnt[b], 1u);
    if (b >= kExactBins) atomicAdd(&lsum[b - kExactBins], (unsigned long long)L);
  }
  // distances |j - i|: one warp per row
  unsigned long long bsum = 0;
  int bmax = 0;
  for (int i = warp; i < d.rows; i += kFeatBlock / 32) {
    const int p1 = __ldg(d.pos + i + 1);
    for (int p = __ldg(d.pos + i) + lane; p < p1; p += 32) {
      const int dist = abs(__ldg(d.crd + p) - i);
      bsum += (unsigned long long)dist;
      bmax = max(bmax, dist);
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
    bsum += __shfl_xor_sync(0xffffffffu, bsum, o);
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bmax = max(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
    empty += __shfl_xor_sync(0xffffffffu, empty, o);
  }
  if (lane == 0) {
    atomicAdd(&s_sq, sq);
    atomicAdd(&s_band_sum, bsum);
    atomicMax(&s_max, mx);
    atomicMax(&s_band_max, bmax);
    atomicAdd(&s_empty, empty);
  }
  __syncthreads();
  if (tid != 0) return;
  const double n = (double)d.rows, S = (double)d.nnz;
  const double mean = d.rows > 0 ? S / n : 0.0;
  const double var = d.rows > 0 ? fmax((double)s_sq / n - mean * mean, 0.0) : 0.0;
  // Gini over the histogram in ascending order: sum_b sum_b * (2 r_b + c_b - n) / (n S)
  double g = 0.0;
  if (d.nnz > 0) {
    double r = 0.0;
    for (int b = 0; b < kBins; b++) {
      const double c = (double)cnt[b];
      if (c == 0.0) continue;
      const double sb = b < kExactBins ? c * (double)b : (double)lsum[b - kExactBins];
      g += sb * (2.0 * r + c - n);
      r += c;
    }
    g /= n * S;
  }
  const double cols = d.cols > 0 ? (double)d.cols : 1.0;
  float* o = out + (size_t)blockIdx.x * F;
  o[0] = (float)log2(n + 1.0);
  o[1] = (float)log2(S + 1.0);
  o[2] = (float)log2(mean + 1.0);
  o[3] = mean > 0.0 ? (float)(sqrt(var) / mean) : 0.0f;
  o[4] = (float)log2((double)s_max + 1.0);
  o[5] = (float)g;
  o[6] = d.nnz > 0 ? (float)((double)s_band_max / cols) : 0.0f;
  o[7] = d.nnz > 0 ? (float)((double)s_band_sum / S / cols) : 0.0f;
  o[8] = d.rows > 0 ? (float)((double)s_empty / n) : 0.0f;
  o[9] = (float)log2((double)d.cols + 1.0);
}

// ------------------------------------------------------------------------------ MLP -----

constexpr int kMlpBlock = 128;  // samples per block
constexpr int XS = F + 1, HS = H + 1, KS = K + 1;  // padded strides: conflict-free both ways
constexpr int kMlpSmemFloats = NPARAM + kMlpBlock * (XS + 4 * HS + KS);

__device__ __forceinline__ void mlp_load_params(float* sp, const float* __restrict__ params) {
  for (int p = threadIdx.x; p < NPARAM; p += blockDim.x) sp[p] = params[p];
}

// Forward pass of one sample; x already z-scored.  h1, h2 may be strided shared rows.
__device__ __forceinline__ void mlp_forward_one(const float* __restrict__ P, const float* x,
                                                float* h1, float* h2, float* y) {
  for (int j = 0; j < H; j++) {
    float a = P[OB1 + j];
#pragma unroll
    for (int f = 0; f < F; f++) a = fmaf(P[OW1 + j * F + f], x[f], a);
    h1[j] = fmaxf(a, 0.0f);
  }
  for (int j = 0; j < H; j++) {
    float a = P[OB2 + j];
#pragma unroll 8
    for (int i = 0; i < H; i++) a = fmaf(P[OW2 + j * H + i], h1[i], a);
    h2[j] = fmaxf(a, 0.0f);
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    float a = P[OB3 + k];
#pragma unroll 8
    for (int i = 0; i < H; i++) a = fmaf(P[OW3 + k * H + i], h2[i], a);
    y[k] = a;
  }
}

__device__ __forceinline__ void load_features(const float* __restrict__ X,
                                              const float* __restrict__ norm, int s, float* x) {
#pragma unroll
  for (int f = 0; f < F; f++) x[f] = (X[(size_t)s * F + f] - norm[f]) / norm[F + f];
}

// Predictions (n x K, optional) and the argmin kind of each sample (optional).
__global__ void __launch_bounds__(kMlpBlock)
mlp_predict(const float* __restrict__ params, const float* __restrict__ norm,
            const float* __restrict__ X, int n, float* __restrict__ pred,
            int32_t* __restrict__ kinds) {
  __shared__ float sp[NPARAM];
  __shared__ float sh[2][kMlpBlock * HS];
  mlp_load_params(sp, params);
  __syncthreads();
  const int s = blockIdx.x * kMlpBlock + threadIdx.x;
  if (s >= n) return;
  float x[F], y[K];
  load_features(X, norm, s, x);
  mlp_forward_one(sp, x, sh[0] + threadIdx.x * HS, sh[1] + threadIdx.x * HS, y);
  int best = 0;
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (pred) pred[(size_t)s * K + k] = y[k];
    if (y[k] < y[best]) best = k;
  }
  if (kinds) kinds[s] = best;
}

// Per-block gradient partials of sum_s sum_k M (y - Y)^2 (unnormalised), the block's loss sum
// and mask count.  part: gridDim.x rows of NPARAM + 2 floats.
__global__ void __launch_bounds__(kMlpBlock)
mlp_grad_partial(const float* __restrict__ params, const float* __restrict__ norm,
                 const float* __restrict__ X, const float* __restrict__ Y,
                 const float* __restrict__ M, int n, float* __restrict__ part) {
  extern __shared__ float smem[];
  float* sp = smem;
  float* sx = sp + NPARAM;                 // [s][XS]
  float* s1 = sx + kMlpBlock * XS;         // h1 [s][HS]
  float* s2 = s1 + kMlpBlock * HS;         // h2
  float* g1 = s2 + kMlpBlock * HS;         // dL/d(pre-activation 1)
  float* g2 = g1 + kMlpBlock * HS;         // dL/d(pre-activation 2)
  float* g3 = g2 + kMlpBlock * HS;         // dL/dy [s][KS]
  __shared__ float s_loss[kMlpBlock], s_mask[kMlpBlock];
  mlp_load_params(sp, params);
  __syncthreads();
  const int t = threadIdx.x, s = blockIdx.x * kMlpBlock + t;
  float* x = sx + t * XS;
  float* h1 = s1 + t * HS;
  float* h2 = s2 + t * HS;
  float* d1 = g1 + t * HS;
  float* d2 = g2 + t * HS;
  float* d3 = g3 + t * KS;
  float loss = 0.0f, msum = 0.0f;
  if (s < n) {
    load_features(X, norm, s, x);
    float y[K];
    mlp_forward_one(sp, x, h1, h2, y);
#pragma unroll
    for (int k = 0; k < K; k++) {
      const float m = M[(size_t)s * K + k], e = y[k] - Y[(size_t)s * K + k];
      d3[k] = 2.0f * m * e;
      loss = fmaf(m * e, e, loss);
      msum += m;
    }
    for (int i = 0; i < H; i++) {
      float a = 0.0f;
#pragma unroll
      for (int k = 0; k < K; k++) a = fmaf(sp[OW3 + k * H + i], d3[k], a);
      d2[i] = h2[i] > 0.0f ? a : 0.0f;
    }
    for (int i = 0; i < H; i++) {
      float a = 0.0f;
#pragma unroll 8
      for (int j = 0; j < H; j++) a = fmaf(sp[OW2 + j * H + i], d2[j], a);
      d1[i] = h1[i] > 0.0f ? a : 0.0f;
    }
  } else {
    for (int f = 0; f < F; f++) x[f] = 0.0f;
    for (int i = 0; i < H; i++) h1[i] = h2[i] = d1[i] = d2[i] = 0.0f;
    for (int k = 0; k < K; k++) d3[k] = 0.0f;
  }
  s_loss[t] = loss;
  s_mask[t] = msum;
  __syncthreads();
  const int ns = min(kMlpBlock, n - (int)blockIdx.x * kMlpBlock);
  float* out = part + (size_t)blockIdx.x * (NPARAM + 2);
  for (int p = t; p < NPARAM; p += kMlpBlock) {
    const float *a, *b;  // gradient = sum_s a[s*sa] * (b ? b[s*sb] : 1)
    int sa, sb;
    if (p < OB1) { const int j = (p - OW1) / F, f = (p - OW1) % F; a = g1 + j; sa = HS; b = sx + f; sb = XS; }
    else if (p < OW2) { a = g1 + (p - OB1); sa = HS; b = nullptr; sb = 0; }
    else if (p < OB2) { const int j = (p - OW2) / H, i = (p - OW2) % H; a = g2 + j; sa = HS; b = s1 + i; sb = HS; }
    else if (p < OW3) { a = g2 + (p - OB2); sa = HS; b = nullptr; sb = 0; }
    else if (p < OB3) { const int k = (p - OW3) / H, i = (p - OW3) % H; a = g3 + k; sa = KS; b = s2 + i; sb = HS; }
    else { a = g3 + (p - OB3); sa = KS; b = nullptr; sb = 0; }
    float acc = 0.0f;
    if (b) {
      for (int q = 0; q < ns; q++) acc = fmaf(a[q * sa], b[q * sb], acc);
    } else {
      for (int q = 0; q < ns; q++) acc += a[q * sa];
    }
    out[p] = acc;
  }
  if (t == 0) {
    float l = 0.0f, m = 0.0f;
    for (int q = 0; q < kMlpBlock; q++) {
      l += s_loss[q];
      m += s_mask[q];
    }
    out[NPARAM] = l;
    out[NPARAM + 1] = m;
  }
}

// Sums the block partials in block order and normalises by the mask count.  With grad, writes
// the gradient; with params, takes one Adam step (beta1 0.9, beta2 0.999, eps 1e-8); with loss,
// writes the mean loss of the evaluated parameters.
__global__ void mlp_reduce_step(const float* __restrict__ part, int nblk,
                                float* __restrict__ grad, float* __restrict__ params,
                                float* __restrict__ m1, float* __restrict__ m2, int step,
                                float lr, float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > NPARAM) return;
  float msum = 0.0f;
  for (int b = 0; b < nblk; b++) msum += part[(size_t)b * (NPARAM + 2) + NPARAM + 1];
  const float inv = msum > 0.0f ? 1.0f / msum : 0.0f;
  if (p == NPARAM) {
    if (loss) {
      float l = 0.0f;
      for (int b = 0; b < nblk; b++) l += part[(size_t)b * (NPARAM + 2) + NPARAM];
      *loss = l * inv;
    }
    return;
  }
  float g = 0.0f;
  for (int b = 0; b < nblk; b++) g += part[(size_t)b * (NPARAM + 2) + p];
  g *= inv;
  if (grad) grad[p] = g;
  if (params) {
    const float a = 0.9f * m1[p] + 0.1f * g;
    const float v = 0.999f * m2[p] + 0.001f * g * g;
    m1[p] = a;
    m2[p] = v;
    const float ah = a / (1.0f - powf(0.9f, (float)step));
    const float vh = v / (1.0f - powf(0.999f, (float)step));
    params[p] -= lr * ah / (sqrtf(vh) + 1e-8f);
  }
}

}  // namespace
}  // namespace tacogb

using namespace tacogb;

namespace {

int mlp_check(const float* params, const float* norm, const float* X, int32_t n) {
  TACOGB_CHECK_ARG(params != nullptr && norm != nullptr, "mlp: null parameters");
  TACOGB_CHECK_ARG(n >= 0 && (n == 0 || X != nullptr), "mlp: bad sample count or features");
  return 0;
}

// One evaluation of the block partials for (params, X, Y, M) into part (device scratch).
int mlp_partials(const float* params, const float* norm, const float* X, const float* Y,
                 const float* M, int32_t n, float* part, cudaStream_t st) {
  const int nblk = (n + kMlpBlock - 1) / kMlpBlock;
  const size_t smem = sizeof(float) * kMlpSmemFloats;
  TACOGB_CUDA_TRY(cudaFuncSetAttribute(mlp_grad_partial,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  mlp_grad_partial<<<nblk, kMlpBlock, smem, st>>>(params, norm, X, Y, M, n, part);
  count_launch();
  TACOGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace

extern "C" {

int tacogb_mlp_param_count(void) { return NPARAM; }

int tacogb_batch_features(int32_t count, const tacogb_csr* mats, float* feats, void* stream) {
  TACOGB_CHECK_ARG(count >= 0 && (count == 0 || (mats && feats)), "features: null arguments");
  if (count == 0) return 0;
  std::vector<FeatDesc> h(count);
  for (int m = 0; m < count; m++) {
    const tacogb_csr& A = mats[m];
    TACOGB_CHECK_ARG(A.rows >= 0 && A.cols >= 0 && A.nnz >= 0 && A.nnz <= INT32_MAX,
                     "features: matrix %d has a bad size", m);
    TACOGB_CHECK_ARG(A.rows == 0 || A.pos, "features: matrix %d has null pos", m);
    TACOGB_CHECK_ARG(A.nnz == 0 || A.crd, "features: matrix %d has null crd", m);
    h[m] = FeatDesc{A.pos, A.crd, A.rows, A.cols, (int32_t)A.nnz, 0};
  }
  cudaStream_t st = (cudaStream_t)stream;
  FeatDesc* d = (FeatDesc*)scratch(sizeof(FeatDesc) * count + 256 + sizeof(float) * F * count, 4);
  if (!d) return last_code();
  float* dout = (float*)((char*)d + ((sizeof(FeatDesc) * count + 255) & ~(size_t)255));
  TACOGB_CUDA_TRY(cudaMemcpyAsync(d, h.data(), sizeof(FeatDesc) * count, cudaMemcpyHostToDevice, st));
  batch_features<<<count, kFeatBlock, 0, st>>>(d, dout);
  count_launch();
  TACOGB_CUDA_TRY(cudaGetLastError());
  TACOGB_CUDA_TRY(cudaMemcpyAsync(feats, dout, sizeof(float) * F * count, cudaMemcpyDeviceToHost, st));
  TACOGB_CUDA_TRY(cudaStreamSynchronize(st));
  return 0;
}

int tacogb_mlp_predict(const float* params, const float* norm, const float* X, int32_t n,
                       float* pred, int32_t* kinds, void* stream) {
  if (int rc = mlp_check(params, norm, X, n)) return rc;
  if (n == 0) return 0;
  mlp_predict<<<(n + kMlpBlock - 1) / kMlpBlock, kMlpBlock, 0, (cudaStream_t)stream>>>(
      params, norm, X, n, pred, kinds);
  count_launch();
  TACOGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

int tacogb_mlp_grad(const float* params, const float* norm, const float* X, const float* Y,
                    const float* M, int32_t n, float* grad, float* loss, void* stream) {
  if (int rc = mlp_check(params, norm, X, n)) return rc;
  TACOGB_CHECK_ARG(n > 0 && Y && M && grad, "mlp: gradient needs samples, targets and a mask");
  cudaStream_t st = (cudaStream_t)stream;
  const int nblk = (n + kMlpBlock - 1) / kMlpBlock;
  float* part = (float*)scratch(sizeof(float) * (size_t)nblk * (NPARAM + 2), 4);
  if (!part) return last_code();
  if (int rc = mlp_partials(params, norm, X, Y, M, n, part, st)) return rc;
  mlp_reduce_step<<<(NPARAM + 1 + 255) / 256, 256, 0, st>>>(part, nblk, grad, nullptr, nullptr,
                                                             nullptr, 0, 0.0f, loss);
  count_launch();
  TACOGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

int tacogb_mlp_train(float* params, const float* norm, const float* X, const float* Y,
                     const float* M, int32_t n, int32_t steps, int32_t step0, float lr,
                     float* adam_state, float* losses, void* stream) {
  if (int rc = mlp_check(params, norm, X, n)) return rc;
  TACOGB_CHECK_ARG(n > 0 && Y && M && adam_state && steps >= 0 && step0 >= 0 && lr > 0.0f,
                   "mlp: training needs samples, targets, a mask, Adam state and lr > 0");
  cudaStream_t st = (cudaStream_t)stream;
  const int nblk = (n + kMlpBlock - 1) / kMlpBlock;
  float* part = (float*)scratch(sizeof(float) * (size_t)nblk * (NPARAM + 2), 4);
  if (!part) return last_code();
  for (int it = 0; it < steps; it++) {
    if (int rc = mlp_partials(params, norm, X, Y, M, n, part, st)) return rc;
    mlp_reduce_step<<<(NPARAM + 1 + 255) / 256, 256, 0, st>>>(
        part, nblk, nullptr, params, adam_state, adam_state + NPARAM, step0 + it + 1, lr,
        losses ? losses + it : nullptr);
    count_launch();
    TACOGB_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

int tacogb_batch_autotune(int32_t count, const tacogb_csr* mats, const void* const* x,
                          void* const* y, int32_t precision, int32_t reps, int32_t* kinds,
                          int64_t* cycles, void* stream) {
  TACOGB_CHECK_ARG(count > 0 && mats && x && y && kinds, "autotune: null arguments");
  TACOGB_CHECK_ARG(reps >= 1, "autotune: reps must be >= 1");
  TACOGB_CHECK_ARG(tacogb_batch_variant_count() == K, "autotune: kind count mismatch");
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<int64_t> best((size_t)count * K, INT64_MAX), run(count);
  std::vector<int32_t> v(count);
  for (int k = 0; k < K; k++) {
    std::fill(v.begin(), v.end(), k);
    tacogb_batch* plan = nullptr;
    if (int rc = tacogb_batch_create(count, mats, x, y, precision, v.data(), &plan)) return rc;
    int rc = tacogb_batch_run(plan, st);  // warm-up: first touch of the plan's arrays
    for (int r = 0; r < reps && rc == 0; r++) {
      rc = tacogb_batch_run(plan, st);
      if (rc == 0) rc = tacogb_batch_matrix_cycles(plan, (int64_t*)run.data(), st);
      if (rc == 0)
        for (int m = 0; m < count; m++)
          best[(size_t)m * K + k] = std::min(best[(size_t)m * K + k], run[m]);
    }
    tacogb_batch_destroy(plan);
    if (rc) return rc;
  }
  for (int m = 0; m < count; m++) {
    int b = 0;
    for (int k = 1; k < K; k++)
      if (best[(size_t)m * K + k] < best[(size_t)m * K + b]) b = k;
    kinds[m] = b;
  }
  if (cycles) std::memcpy(cycles, best.data(), sizeof(int64_t) * best.size());
  return 0;
}

int tacogb_batch_select(int32_t count, const tacogb_csr* mats, const float* params,
                        const float* norm, int32_t* kinds, void* stream) {
  TACOGB_CHECK_ARG(count > 0 && mats && params && norm && kinds, "select: null arguments");
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<float> feats((size_t)count * F);
  if (int rc = tacogb_batch_features(count, mats, feats.data(), st)) return rc;
  float* dX = nullptr;
  int32_t* dk = nullptr;
  TACOGB_CUDA_TRY(cudaMalloc(&dX, sizeof(float) * feats.size()));
  if (cudaMalloc(&dk, sizeof(int32_t) * count) != cudaSuccess) {
    cudaFree(dX);
    set_error(TACOGB_ERR_ALLOC, "select: out of device memory");
    return TACOGB_ERR_ALLOC;
  }
  cudaError_t e = cudaMemcpyAsync(dX, feats.data(), sizeof(float) * feats.size(),
                                  cudaMemcpyHostToDevice, st);
  int rc = e == cudaSuccess ? tacogb_mlp_predict(params, norm, dX, count, nullptr, dk, st) : 0;
  if (e == cudaSuccess && rc == 0)
    e = cudaMemcpyAsync(kinds, dk, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && rc == 0) e = cudaStreamSynchronize(st);
  cudaFree(dX);
  cudaFree(dk);
  if (rc) return rc;
  if (e != cudaSuccess) {
    set_error(TACOGB_ERR_CUDA, "select: %s", cudaGetErrorString(e));
    return TACOGB_ERR_CUDA;
  }
  return 0;
}

}  // extern "C"
