// CUDA-core FMA peak of the current GPU, FP32 and FP64: the roofline
// denominators for the solver's kernels, which are bound by CUDA-core FMA
// (small pivoted factorizations) rather than by tensor cores or HBM.
// Built as its own library (lib/libfmapeak.so) for the benchmark; it is not
// part of the solver's C ABI.
#include <cuda_runtime.h>

namespace {

// Eight independent FMA chains per thread keep the pipes full.
template <class T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b;
    x1 = x1 * a + b;
    x2 = x2 * a + b;
    x3 = x3 * a + b;
    x4 = x4 * a + b;
    x5 = x5 * a + b;
    x6 = x6 * a + b;
    x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
int time_chains(int blocks, int threads, int iters, T* out, double* tflops) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return 1;
  fma_chains<T><<<blocks, threads>>>(out, 16, (T)0.999, (T)1e-3);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)1e-3);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

// Measures both peaks on `device` (a few tens of milliseconds); 0 on success.
extern "C" int fma_peak_tflops(int device, double* fp32_tflops, double* fp64_tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return 1;
  const int blocks = nsm * 8, threads = 256;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return 1;
  int rc = time_chains<float>(blocks, threads, 50000, reinterpret_cast<float*>(out), fp32_tflops);
  rc |= time_chains<double>(blocks, threads, 1000, out, fp64_tflops);
  cudaFree(out);
  return rc;
}
