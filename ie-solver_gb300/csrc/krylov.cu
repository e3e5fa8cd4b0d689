// Block-vector kernels of the flexible GMRES used for the refinement's
// correction equation (no reference counterpart: the reference solves
// directly).  A block vector holds nrhs vectors of the bordered system:
// the mu parts as a D x nrhs column-major block, then the alpha parts as an
// nb x nrhs block, so the FMM and the factorization read them in place.
// Basis vector j of a basis starts at V + j * vstride.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.hpp"

namespace rskel {

namespace {

constexpr int kKryThreads = 256;

__device__ __forceinline__ int rhs_of(size_t i, int D, int nb, int nrhs) {
  const size_t mu = (size_t)D * nrhs;
  return i < mu ? (int)(i / D) : (int)((i - mu) / nb);
}

// part[(c * gridDim.x + block) * kKrylovMaxBasis + j]: this block's share of
// <V_j, w> over right-hand side c's entries (grid: blocks x nrhs).
__global__ void __launch_bounds__(kKryThreads) mdot_partial_kernel(const double* V,
                                                                   size_t vstride, int nv,
                                                                   const double* w, int D,
                                                                   int nb, int nrhs,
                                                                   double* part) {
  const int c = blockIdx.y;
  const size_t n = (size_t)D + nb;
  double acc[kKrylovMaxBasis];
#pragma unroll
  for (int j = 0; j < kKrylovMaxBasis; ++j) acc[j] = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t i = e < (size_t)D ? (size_t)c * D + e
                                   : (size_t)D * nrhs + (size_t)c * nb + (e - D);
    const double we = w[i];
#pragma unroll
    for (int j = 0; j < kKrylovMaxBasis; ++j)
      if (j < nv) acc[j] += V[j * vstride + i] * we;
  }
  __shared__ double red[kKryThreads / 32][kKrylovMaxBasis];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kKrylovMaxBasis; ++j) {
    if (j >= nv) break;
    const double v = warp_sum(acc[j]);
    if (lane == 0) red[warp][j] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < nv) {
    double s = 0.0;
    for (int wp = 0; wp < kKryThreads / 32; ++wp) s += red[wp][threadIdx.x];
    part[((size_t)c * gridDim.x + blockIdx.x) * kKrylovMaxBasis + threadIdx.x] = s;
  }
}

// h[c * kKrylovMaxBasis + j] = sum over blocks, in block order.
__global__ void mdot_final_kernel(const double* part, int nv, int nrhs, int nblk, double* h) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv * nrhs) return;
  const int c = t / nv, j = t % nv;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += part[((size_t)c * nblk + b) * kKrylovMaxBasis + j];
  h[c * kKrylovMaxBasis + j] = s;
}

// w += sign * sum_j h[c][j] V_j over every entry (c = the entry's rhs).
__global__ void maxpy_kernel(double* w, const double* V, size_t vstride, int nv, const double* h,
                             double sign, int D, int nb, int nrhs) {
  const size_t total = ((size_t)D + nb) * nrhs;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int c = rhs_of(i, D, nb, nrhs);
    double acc = 0.0;
    for (int j = 0; j < nv; ++j) acc += h[c * kKrylovMaxBasis + j] * V[j * vstride + i];
    w[i] += sign * acc;
  }
}

// w = x * s[c] (s: nrhs scale factors on the device).
__global__ void kscale_kernel(double* w, const double* x, const double* s, int D, int nb,
                              int nrhs) {
  const size_t total = ((size_t)D + nb) * nrhs;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x)
    w[i] = x[i] * s[rhs_of(i, D, nb, nrhs)];
}

unsigned grid_for(size_t n) {
  const size_t g = (n + kKryThreads - 1) / kKryThreads;
  return (unsigned)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

}  // namespace

int krylov_dot_blocks(int D, int nb) {
  const size_t n = (size_t)D + nb;
  const size_t b = (n + 4 * kKryThreads - 1) / (4 * kKryThreads);
  return (int)(b < 1 ? 1 : (b > 64 ? 64 : b));
}

void launch_mdot(const double* V, size_t vstride, int nv, const double* w, int D, int nb, int nrhs,
                 double* part, double* h, cudaStream_t st) {
  if (nv <= 0 || nrhs <= 0) return;
  const int nblk = krylov_dot_blocks(D, nb);
  mdot_partial_kernel<<<dim3(nblk, nrhs), kKryThreads, 0, st>>>(V, vstride, nv, w, D, nb, nrhs,
                                                                part);
  mdot_final_kernel<<<(nv * nrhs + 127) / 128, 128, 0, st>>>(part, nv, nrhs, nblk, h);
}

void launch_maxpy(double* w, const double* V, size_t vstride, int nv, const double* h, double sign,
                  int D, int nb, int nrhs, cudaStream_t st) {
  if (nv <= 0) return;
  maxpy_kernel<<<grid_for(((size_t)D + nb) * nrhs), kKryThreads, 0, st>>>(w, V, vstride, nv, h,
                                                                         sign, D, nb, nrhs);
}

void launch_kscale(double* w, const double* x, const double* s, int D, int nb, int nrhs,
                   cudaStream_t st) {
  kscale_kernel<<<grid_for(((size_t)D + nb) * nrhs), kKryThreads, 0, st>>>(w, x, s, D, nb, nrhs);
}

}  // namespace rskel
