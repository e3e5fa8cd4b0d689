// Learned skeleton-rank predictor: inference, gradient and Adam kernels for
// the 16 -> 64 -> 64 -> 1 MLP of rank_model.hpp.  One warp per sample: lane
// l owns hidden units l and l + 32; the weights sit in shared memory, W1 and
// W2 transposed so that a warp's accesses to one input column are
// consecutive (no bank conflicts).
#include <cuda_runtime.h>

#include "common.cuh"
#include "rank_model.hpp"

namespace rskel {

namespace {

constexpr int kH = kRankHidden, kF = kRankFeatures;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kH * kF;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH;
constexpr int kWarpsPerBlock = 8;
constexpr int kMlpThreads = 32 * kWarpsPerBlock;

// Shared weights: W1T (kF x kH), W2T (kH x kH), W2 (kH x kH, for the
// backward pass), biases and output layer.
struct SharedMlp {
  float* w1t;
  float* w2t;
  float* w2;
  float* b1;
  float* b2;
  float* w3;
  float b3;
};

__device__ void load_mlp(const float* W, float* smem, SharedMlp* m, bool need_w2) {
  m->w1t = smem;
  m->w2t = m->w1t + kF * kH;
  m->w2 = m->w2t + kH * kH;
  m->b1 = m->w2 + (need_w2 ? kH * kH : 0);
  m->b2 = m->b1 + kH;
  m->w3 = m->b2 + kH;
  for (int e = threadIdx.x; e < kH * kF; e += blockDim.x) {
    const int u = e / kF, i = e % kF;
    m->w1t[i * kH + u] = W[kOffW1 + e];
  }
  for (int e = threadIdx.x; e < kH * kH; e += blockDim.x) {
    const int u = e / kH, j = e % kH;
    m->w2t[j * kH + u] = W[kOffW2 + e];
    if (need_w2) m->w2[e] = W[kOffW2 + e];
  }
  for (int u = threadIdx.x; u < kH; u += blockDim.x) {
    m->b1[u] = W[kOffB1 + u];
    m->b2[u] = W[kOffB2 + u];
    m->w3[u] = W[kOffW3 + u];
  }
  m->b3 = W[kOffB3];
}

// Forward pass of one sample by one warp; x, h1, h2 are the warp's shared
// slices (kF, kH, kH).  Returns the rank fraction y on every lane.
__device__ float forward(const SharedMlp& m, const float* x, float* h1, float* h2) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int u = lane + 32 * s;
    float a = m.b1[u];
#pragma unroll
    for (int i = 0; i < kF; ++i) a += m.w1t[i * kH + u] * x[i];
    h1[u] = a > 0.f ? a : 0.f;
  }
  __syncwarp();
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int u = lane + 32 * s;
    float a = m.b2[u];
    for (int j = 0; j < kH; ++j) a += m.w2t[j * kH + u] * h1[j];
    h2[u] = a > 0.f ? a : 0.f;
  }
  __syncwarp();
  float part = m.w3[lane] * h2[lane] + m.w3[lane + 32] * h2[lane + 32];
  part = warp_sum(part);
  const float z = part + m.b3;
  return 1.f / (1.f + __expf(-z));
}

constexpr size_t mlp_smem(bool need_w2) {
  return sizeof(float) * ((size_t)kF * kH + kH * kH + (need_w2 ? kH * kH : 0) + 3 * kH +
                          kWarpsPerBlock * (kF + 3 * kH));
}

// Sketch rows for a box from the predicted rank fraction: headroom over the
// predicted rank plus extra rows of oversampling, never more than the plain
// n + 16.
__device__ __forceinline__ int ell_from_fraction(float y, int n, float headroom, int extra) {
  const int k = (int)ceilf(y * (float)n);
  int ell = (int)ceilf(headroom * (float)k) + extra;
  if (ell < 12) ell = 12;
  if (ell > n + 16) ell = n + 16;
  return ell;
}

template <int kMode>  // 0: predict into out; 1: write tasks[i].ell and ell_by_slot
__global__ void __launch_bounds__(kMlpThreads) infer_kernel(const float* W, const float* feats,
                                                            int count, float* out,
                                                            IdTask* tasks, int* ell_by_slot,
                                                            float headroom, int extra) {
  extern __shared__ __align__(16) float smem[];
  SharedMlp m;
  load_mlp(W, smem, &m, false);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xw = m.w3 + kH + warp * (kF + 3 * kH);
  float* h1 = xw + kF;
  float* h2 = h1 + kH;
  __syncthreads();
  for (int i = blockIdx.x * kWarpsPerBlock + warp; i < count; i += gridDim.x * kWarpsPerBlock) {
    if (lane < kF) xw[lane] = feats[(size_t)i * kF + lane];
    __syncwarp();
    const float y = forward(m, xw, h1, h2);
    if (lane == 0) {
      if (kMode == 0) {
        out[i] = y;
      } else {
        const int ell = ell_from_fraction(y, tasks[i].n, headroom, extra);
        tasks[i].ell = ell;
        ell_by_slot[tasks[i].slot] = ell;
      }
    }
    __syncwarp();
  }
}

// Gradient partials, deterministic: each warp owns a private gradient in
// shared memory (within a warp every entry belongs to one lane, so no
// atomics), the block sums its warps in order into partial[block], and
// grad_reduce_kernel sums the blocks in order.  Samples go to warps by a
// fixed rule, so the result does not depend on scheduling.
constexpr int kGradBlocks = 152;
constexpr int kPartial = kRankWeights + 1;  // a block's gradient, then its squared error

__global__ void __launch_bounds__(kMlpThreads) grad_kernel(const float* W, const float* feats,
                                                           const float* targets, int count,
                                                           float* partial) {
  extern __shared__ __align__(16) float smem[];
  SharedMlp m;
  load_mlp(W, smem, &m, true);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xw = m.w3 + kH + warp * (kF + 3 * kH);
  float* h1 = xw + kF;
  float* h2 = h1 + kH;
  float* d2 = h2 + kH;  // dL/d(pre-activation of layer 2)
  float* gall = m.w3 + kH + kWarpsPerBlock * (kF + 3 * kH);  // kWarpsPerBlock gradients
  float* g = gall + (size_t)warp * kRankWeights;
  __shared__ float wl[kWarpsPerBlock];
  for (int e = threadIdx.x; e < kWarpsPerBlock * kRankWeights; e += blockDim.x) gall[e] = 0.f;
  __syncthreads();
  float lsum = 0.f;
  const float scale = 1.f / (float)count;
  for (int i = blockIdx.x * kWarpsPerBlock + warp; i < count; i += gridDim.x * kWarpsPerBlock) {
    if (lane < kF) xw[lane] = feats[(size_t)i * kF + lane];
    __syncwarp();
    const float y = forward(m, xw, h1, h2);
    const float t = targets[i];
    lsum += (y - t) * (y - t);
    const float dz = 2.f * (y - t) * y * (1.f - y) * scale;
    if (lane == 0) g[kOffB3] += dz;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int u = lane + 32 * s;
      g[kOffW3 + u] += dz * h2[u];
      const float du = h2[u] > 0.f ? dz * m.w3[u] : 0.f;
      d2[u] = du;
      g[kOffB2 + u] += du;
    }
    __syncwarp();
    // dW2[u][j] = d2[u] h1[j]: lane covers columns j = lane, lane + 32
    for (int u = 0; u < kH; ++u) {
      const float du = d2[u];
      if (du == 0.f) continue;
      g[kOffW2 + u * kH + lane] += du * h1[lane];
      g[kOffW2 + u * kH + lane + 32] += du * h1[lane + 32];
    }
    // d1[j] = sum_u W2[u][j] d2[u] (h1[j] > 0)
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = lane + 32 * s;
      float a = 0.f;
      for (int u = 0; u < kH; ++u) a += m.w2[u * kH + j] * d2[u];
      const float d1 = h1[j] > 0.f ? a : 0.f;
      g[kOffB1 + j] += d1;
#pragma unroll
      for (int q = 0; q < kF; ++q) g[kOffW1 + j * kF + q] += d1 * xw[q];
    }
    __syncwarp();
  }
  if (lane == 0) wl[warp] = lsum;  // every lane holds the warp's sum (y is on every lane)
  __syncthreads();
  float* out = partial + (size_t)blockIdx.x * kPartial;
  for (int e = threadIdx.x; e < kRankWeights; e += blockDim.x) {
    float a = 0.f;
    for (int w = 0; w < kWarpsPerBlock; ++w) a += gall[(size_t)w * kRankWeights + e];
    out[e] = a;
  }
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int w = 0; w < kWarpsPerBlock; ++w) a += wl[w];
    out[kRankWeights] = a;
  }
}

__global__ void grad_reduce_kernel(const float* partial, int blocks, float* grad,
                                   float* loss_sum) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kPartial) return;
  float a = 0.f;
  for (int b = 0; b < blocks; ++b) a += partial[(size_t)b * kPartial + e];
  if (e < kRankWeights) grad[e] = a;
  else *loss_sum = a;
}

int grad_blocks(int count) {
  const int g = (count + kWarpsPerBlock - 1) / kWarpsPerBlock;
  return g < 1 ? 1 : (g > kGradBlocks ? kGradBlocks : g);
}

__global__ void adam_kernel(float* W, const float* grad, float* m, float* v, float b1t, float b2t,
                            float lr) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kRankWeights) return;
  const float b1 = 0.9f, b2 = 0.999f;
  const float gr = grad[e];
  const float mm = b1 * m[e] + (1.f - b1) * gr;
  const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
  m[e] = mm;
  v[e] = vv;
  const float mh = mm / (1.f - b1t), vh = vv / (1.f - b2t);
  W[e] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

int grid_for(int count) {
  const int g = (count + kWarpsPerBlock - 1) / kWarpsPerBlock;
  return g < 1 ? 1 : (g > 1216 ? 1216 : g);
}

}  // namespace

cudaError_t rank_infer_ell(const float* weights, const float* features, IdTask* tasks,
                           int num_tasks, int* ell_by_slot, float headroom, int extra,
                           cudaStream_t st) {
  if (num_tasks <= 0) return cudaSuccess;
  infer_kernel<1><<<grid_for(num_tasks), kMlpThreads, mlp_smem(false), st>>>(
      weights, features, num_tasks, nullptr, tasks, ell_by_slot, headroom, extra);
  return cudaGetLastError();
}

cudaError_t rank_predict(const float* weights, const float* features, int count, float* out,
                         cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  infer_kernel<0><<<grid_for(count), kMlpThreads, mlp_smem(false), st>>>(
      weights, features, count, out, nullptr, nullptr, 0.f, 0);
  return cudaGetLastError();
}

size_t rank_gradient_scratch(int count) { return (size_t)grad_blocks(count) * kPartial; }

cudaError_t rank_gradient(const float* weights, const float* features, const float* targets,
                          int count, float* grad, float* loss_sum, float* scratch,
                          cudaStream_t st) {
  if (count <= 0) {
    cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(float) * kRankWeights, st);
    return e == cudaSuccess ? cudaMemsetAsync(loss_sum, 0, sizeof(float), st) : e;
  }
  const int blocks = grad_blocks(count);
  const size_t smem = mlp_smem(true) + sizeof(float) * kWarpsPerBlock * kRankWeights;
  set_smem_once<grad_kernel>();
  grad_kernel<<<blocks, kMlpThreads, smem, st>>>(weights, features, targets, count, scratch);
  grad_reduce_kernel<<<(kPartial + 255) / 256, 256, 0, st>>>(scratch, blocks, grad, loss_sum);
  return cudaGetLastError();
}

cudaError_t rank_adam(float* weights, const float* grad, float* m, float* v, int t, float lr,
                      cudaStream_t st) {
  const float b1t = powf(0.9f, (float)t), b2t = powf(0.999f, (float)t);
  adam_kernel<<<(kRankWeights + 255) / 256, 256, 0, st>>>(weights, grad, m, v, b1t, b2t, lr);
  return cudaGetLastError();
}

}  // namespace rskel
