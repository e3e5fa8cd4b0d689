// rs_id_noalloc: one FP64 interpolative decomposition (ie_Mat::id,
// ie_mat.cpp:548-588) of a matrix that is already on the device, without any
// device allocation.
//
// The ID kernel's column-pivoted QR runs on the whole m x n matrix held in a
// global-memory tile (the same "direct" mode the FP64 factorization uses for
// its boxes).  Here that tile, and the one-task descriptor the kernel reads,
// live in file-scope __device__ arrays of fixed size instead of buffers from
// cudaMalloc, so a call costs two kernel launches on the caller's stream and
// nothing else.
//
// Set-up: the first call on a device (with that device current) looks up the
// arrays' device addresses with cudaGetSymbolAddress and sets the kernel's
// shared-memory attribute; make that first call before any stream capture.
// The addresses are kept for the life of the process, so a process that
// resets a device (cudaDeviceReset) must not call this entry point on that
// device afterwards: the kept addresses belong to the destroyed context.
//
// Errors: a CUDA error already pending in the calling thread (left by the
// caller's earlier work) is reported as RS_ERR_CUDA without being cleared,
// and nothing is launched; each of this call's two launches is checked on
// its own right after it.
//
// Sharing: every call on a device uses the same arrays, so calls that overlap
// in time (on different streams, or from different host threads) race and
// must be serialised by the caller.  Nothing in the arrays needs to start at
// zero: each call writes the descriptor and every tile row and reflector
// entry it later reads.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/rskel.h"
#include "kernels.hpp"
#include "plan.hpp"

namespace rskel {
namespace {

// 4 MiB of FP64 scratch: the m x n tile (rows padded to 64, leading
// dimension n + up to 31) plus the m-entry reflector.
constexpr size_t kNoAllocScratchDoubles = size_t(1) << 19;
constexpr size_t kNoAllocSmemMax = 227 * 1024;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_id_scratch[kNoAllocScratchDoubles];
static __device__ __align__(256) IdTask g_id_task;

__global__ void put_task_kernel(IdTask t, IdTask* dst) { *dst = t; }

struct DeviceSlots {
  bool ready = false;
  double* scratch = nullptr;
  IdTask* task = nullptr;
};

std::mutex g_setup_mu;
DeviceSlots g_slots[kMaxDevices];

// Once per device, with that device current.
rs_status setup_device(int dev, DeviceSlots** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSlots& d = g_slots[dev];
  if (!d.ready) {
    void* ps = nullptr;
    void* pt = nullptr;
    if (cudaGetSymbolAddress(&ps, g_id_scratch) != cudaSuccess) return RS_ERR_CUDA;
    if (cudaGetSymbolAddress(&pt, g_id_task) != cudaSuccess) return RS_ERR_CUDA;
    d.scratch = static_cast<double*>(ps);
    d.task = static_cast<IdTask*>(pt);
    if (id_noalloc_prepare() != cudaSuccess) return RS_ERR_CUDA;
    d.ready = true;
  }
  *out = &d;
  return RS_OK;
}

}  // namespace
}  // namespace rskel

extern "C" rs_status rs_id_noalloc(int m, int n, const double* A, double tol, int* rank, int* perm,
                                   double* Z, void* stream) {
  using namespace rskel;
  if (m < 1 || n < 1 || !A || !rank || !perm || !Z || !(tol > 0)) return RS_ERR_ARG;
  if (id_direct_tile(m, n) > kNoAllocScratchDoubles ||
      id_kernel_smem(n, false, false) > kNoAllocSmemMax)
    return RS_ERR_CAPACITY;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return RS_ERR_NO_DEVICE;
  if (dev >= kMaxDevices) return RS_ERR_CAPACITY;
  DeviceSlots* d = nullptr;
  rs_status rc = setup_device(dev, &d);
  if (rc != RS_OK) return rc;
  // not this call's error: leave it pending for its owner, launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return RS_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  IdTask t{};
  t.n = n;
  t.act_off = 0;
  t.slot = 0;
  t.fac_off = 0;
  t.scratch_off = 0;
  t.dense_off = 0;
  t.m_dense = m;
  put_task_kernel<<<1, 1, 0, st>>>(t, d->task);
  if (cudaGetLastError() != cudaSuccess) return RS_ERR_CUDA;
  IdParams ip{};
  ip.sd = 1;
  ip.npp = 1;
  ip.tol = tol;
  ip.tasks = d->task;
  ip.ranks = rank;
  ip.perm = perm;
  ip.fac = Z;
  ip.scratch = d->scratch;
  ip.dense = A;
  ip.phase_clk = nullptr;
  ip.direct = 1;
  launch_id(ip, 1, n, id_kernel_smem(n, false, false), false, st);
  return cudaGetLastError() == cudaSuccess ? RS_OK : RS_ERR_CUDA;
}
