// Minimal owning device buffer.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstring>

namespace rskel {

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;  // elements

  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }

  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  // Grows to at least n elements; contents are discarded on growth.
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    release();
    size_t want = n + n / 4 + 64;
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e != cudaSuccess) { p = nullptr; return e; }
    cap = want;
    return cudaSuccess;
  }
  // Grows to at least n elements keeping the first `used` elements.
  cudaError_t ensure_keep(size_t n, size_t used, cudaStream_t st) {
    if (n <= cap && p) return cudaSuccess;
    size_t want = n + n / 2 + 1024;
    T* q = nullptr;
    cudaError_t e = cudaMalloc(&q, want * sizeof(T));
    if (e != cudaSuccess) return e;
    if (p && used) {
      e = cudaMemcpyAsync(q, p, used * sizeof(T), cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) { cudaFree(q); return e; }
      cudaStreamSynchronize(st);
    }
    release();
    p = q;
    cap = want;
    return cudaSuccess;
  }
};

// Pinned host staging buffer.
template <class T>
struct HostBuf {
  T* p = nullptr;
  size_t cap = 0;
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  ~HostBuf() { release(); }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
  cudaError_t ensure(size_t n) {
    if (n <= cap && p) return cudaSuccess;
    release();
    size_t want = n + n / 4 + 64;
    cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
    if (e != cudaSuccess) { p = nullptr; return e; }
    cap = want;
    return cudaSuccess;
  }
};

}  // namespace rskel
