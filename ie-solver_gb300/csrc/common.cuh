// Device helpers shared by the factorization and solve kernels.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include "plan.hpp"

namespace rskel {

constexpr int kThreads = 256;              // threads per box (8 warps)
constexpr int kSmemOptIn = 227 * 1024;     // opt-in dynamic shared memory per CTA

// Raises a kernel's dynamic shared-memory limit to the opt-in maximum once
// per process (a driver call per launch would sit on every level's path).
// (One flag per kernel: the kernel is a template argument.)
template <auto Kernel>
inline void set_smem_once() {
  static bool done = false;
  if (!done) {
    // The limit covers static plus dynamic shared memory.
    cudaFuncAttributes a{};
    size_t stat = 0;
    if (cudaFuncGetAttributes(&a, Kernel) == cudaSuccess) stat = a.sharedSizeBytes;
    cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kSmemOptIn - stat));
    done = true;
  }
}
constexpr int kWarps = kThreads / 32;

// Programmatic dependent launch.  A kernel launched with launch_pdl may be
// scheduled while the previous kernel on its stream still runs, once every
// CTA of that kernel has called pdl_launch_dependents (or exited); it does
// its prologue (reads of data written before that kernel) and calls
// pdl_wait before its first read of the previous kernel's output, which
// returns once that kernel has completed and its writes are visible.  In a
// kernel launched without the attribute both are no-ops.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch with programmatic stream serialisation; a plain launch if the
// attribute is refused.
template <class... Params, class... Args>
inline void launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, kernel, args...) != cudaSuccess) {
    (void)cudaGetLastError();
    kernel<<<grid, block, smem, st>>>(args...);
  }
}

// The elements e = threadIdx.x, threadIdx.x + blockDim.x, ... of a
// column-major rows x cols tile as (i, j) = (e % rows, e / rows), stepped
// without an integer division per element (a division by a runtime value
// is a long ALU sequence, and the kernels' tile loops run once per step).
// rows must be positive.
struct TileWalk {
  int i, j, di, dj, rows;
  __device__ __forceinline__ explicit TileWalk(int rows_) : rows(rows_) {
    i = (int)threadIdx.x % rows;
    j = (int)threadIdx.x / rows;
    di = (int)blockDim.x % rows;
    dj = (int)blockDim.x / rows;
  }
  __device__ __forceinline__ int e() const { return i + rows * j; }
  __device__ __forceinline__ void next() {
    i += di;
    j += dj;
    if (i >= rows) {
      i -= rows;
      ++j;
    }
  }
};

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide argmax of val over [lo, hi) (ties -> smallest index), result in
// *out_idx for every thread.  scratch needs 2 * kWarps entries.
__device__ __forceinline__ int block_argmax(const double* val, int lo, int hi, double* sv,
                                            int* si) {
  double best = -1.0;
  int bi = hi;
  for (int c = lo + threadIdx.x; c < hi; c += blockDim.x) {
    double v = val[c];
    if (v > best || (v == best && c < bi)) { best = v; bi = c; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, best, o);
    int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sv[warp] = best; si[warp] = bi; }
  __syncthreads();
  if (warp == 0) {
    int nw = blockDim.x >> 5;
    best = lane < nw ? sv[lane] : -1.0;
    bi = lane < nw ? si[lane] : hi;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) si[0] = bi;
  }
  __syncthreads();
  int r = si[0];
  __syncthreads();
  return r;
}

// Per-DOF boundary data staged in shared memory (structure of arrays).
template <class Real>
struct DofSoA {
  Real *x, *y, *nx, *ny, *w, *kap;
  int* comp;
};

template <class Real>
__device__ __forceinline__ Real* carve(unsigned char*& p, int count) {
  Real* r = reinterpret_cast<Real*>(p);
  size_t bytes = sizeof(Real) * (size_t)count;
  p += (bytes + 15) & ~size_t(15);
  return r;
}

template <class Real>
__device__ __forceinline__ DofSoA<Real> carve_dofs(unsigned char*& p, int count) {
  DofSoA<Real> d;
  d.x = carve<Real>(p, count);
  d.y = carve<Real>(p, count);
  d.nx = carve<Real>(p, count);
  d.ny = carve<Real>(p, count);
  d.w = carve<Real>(p, count);
  d.kap = carve<Real>(p, count);
  d.comp = carve<int>(p, count);
  return d;
}

template <class Real>
__host__ __device__ constexpr size_t dofs_bytes(int count) {
  return 6 * ((sizeof(Real) * (size_t)count + 15) & ~size_t(15)) +
         ((sizeof(int) * (size_t)count + 15) & ~size_t(15));
}

// Loads DOF data for dofs[0..cnt) into slots [0..cnt) of d.  Coordinates are
// shifted by (ox, oy) in double before rounding to Real.
template <class Real>
__device__ __forceinline__ void load_dof(const Geo<double>& g, int sd, int dof, double ox,
                                         double oy, DofSoA<Real>& d, int slot) {
  int p = sd == 1 ? dof : (dof >> 1);
  // all six loads before any store: the stores go through generic pointers
  // that the compiler cannot tell apart from the geometry, so interleaved
  // they would make six dependent global round trips
  const double gx = g.x[p], gy = g.y[p], gnx = g.nx[p], gny = g.ny[p], gw = g.w[p];
  const double gk = g.kap[p];
  d.x[slot] = (Real)(gx - ox);
  d.y[slot] = (Real)(gy - oy);
  d.nx[slot] = (Real)gnx;
  d.ny[slot] = (Real)gny;
  d.w[slot] = (Real)gw;
  d.kap[slot] = (Real)gk;
  d.comp[slot] = dof - p * sd;
}

// y[i ys] -= a x[i xs] for i < cnt (x and y disjoint), four loads of each
// ahead of their stores: in a plain loop every load waits behind the
// previous store, which the compiler cannot prove distinct, so the loop is a
// chain of shared-memory round trips.  Each element is the same fused
// multiply-add as in the plain loop.
template <class T>
__device__ __forceinline__ void axpy_sub(T* y, int ys, const T* x, int xs, T a, int cnt) {
  int i = 0;
  for (; i + 4 <= cnt; i += 4) {
    const T y0 = y[i * ys], y1 = y[(i + 1) * ys], y2 = y[(i + 2) * ys], y3 = y[(i + 3) * ys];
    const T x0 = x[i * xs], x1 = x[(i + 1) * xs], x2 = x[(i + 2) * xs], x3 = x[(i + 3) * xs];
    y[i * ys] = y0 - a * x0;
    y[(i + 1) * ys] = y1 - a * x1;
    y[(i + 2) * ys] = y2 - a * x2;
    y[(i + 3) * ys] = y3 - a * x3;
  }
  for (; i < cnt; ++i) y[i * ys] -= a * x[i * xs];
}

// dst[e] = src[e] for e < n, over `nthreads` threads (this one is `tid`),
// eight loads in flight per thread before their stores: a plain copy loop
// through generic pointers keeps each load behind the previous store (the
// compiler cannot rule out that they alias), one global round trip per
// element.
template <class T>
__device__ __forceinline__ void batched_copy(T* dst, const T* src, int n, int tid, int nthreads) {
  for (int e0 = tid; e0 < n; e0 += 8 * nthreads) {
    T v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * nthreads;
      if (e < n) v[q] = src[e];
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * nthreads;
      if (e < n) dst[e] = v[q];
    }
  }
}

// Reciprocal: correctly rounded single-precision reciprocal; for double, a
// single-precision seed refined by two Newton-Raphson steps
// y <- y + y (1 - d y) (quadratic convergence: 2^-23 -> 2^-46 -> below one
// ulp), which costs four FP64 FMAs instead of a full-precision division.
__device__ __forceinline__ float rcp(float d) { return __frcp_rn(d); }
__device__ __forceinline__ double rcp(double d) {
  const double ad = fabs(d);
  if (!(ad > 1e-30 && ad < 1e30)) return 1.0 / d;
  double y = (double)__frcp_rn((float)d);
  double e = fma(-d, y, 1.0);
  y = fma(y, e, y);
  e = fma(-d, y, 1.0);
  return fma(y, e, y);
}

// Double-layer kernel entries (ie_solver/kernel/kernel.cpp:29-91, 123-290).
// Target (tx, ty, tn) component ta; source (sx, sy, sn, sw, skap) component sb.
template <class Real>
__device__ __forceinline__ Real kernel_entry(int pde, Real tx, Real ty, Real tnx, Real tny,
                                             int ta, Real sx, Real sy, Real snx, Real sny,
                                             Real sw, Real skap, int sb) {
  if (pde == kLaplace) {
    const Real scale = (Real)(1.0 / (2.0 * CUDART_PI));
    if (tx == sx && ty == sy) return (Real)0.5 + (Real)0.5 * skap * sw * scale;
    Real r0 = tx - sx, r1 = ty - sy;
    return -sw * scale * (r0 * snx + r1 * sny) * rcp(r0 * r0 + r1 * r1);
  }
  if (pde == kStokes) {
    const Real scale = (Real)(1.0 / CUDART_PI);
    Real tn_a = ta == 0 ? tnx : tny;
    Real sn_b = sb == 0 ? snx : sny;
    if (tx == sx && ty == sy) {
      Real pot = (Real)-0.5 * skap * sw * scale;
      // tangent t = (-sn_y, sn_x): -0.5 delta_ab + pot t_a t_b + w n_a n_b
      Real t_a = ta == 0 ? -sny : snx;
      Real t_b = sb == 0 ? -sny : snx;
      Real v = pot * t_a * t_b + sw * tn_a * sn_b;
      return ta == sb ? (Real)-0.5 + v : v;
    }
    Real r0 = tx - sx, r1 = ty - sy;
    Real d = r0 * r0 + r1 * r1;
    const Real id = rcp(d);
    Real pot = sw * scale * (r0 * snx + r1 * sny) * (id * id);
    Real ra = ta == 0 ? r0 : r1;
    Real rb = sb == 0 ? r0 : r1;
    return pot * ra * rb + sw * tn_a * sn_b;
  }
  // Laplace-Neumann (kernel.cpp:80-91)
  const Real scale = (Real)(1.0 / (2.0 * CUDART_PI));
  if (tx == sx && ty == sy) return sw - (Real)0.5 + (Real)0.5 * skap * sw * scale;
  Real r0 = tx - sx, r1 = ty - sy;
  return sw + sw * scale * (r0 * tnx + r1 * tny) * rcp(r0 * r0 + r1 * r1);
}

template <class Real>
__device__ __forceinline__ Real kernel_dofs(int pde, const DofSoA<Real>& t, int i,
                                            const DofSoA<Real>& s, int j) {
  return kernel_entry<Real>(pde, t.x[i], t.y[i], t.nx[i], t.ny[i], t.comp[i], s.x[j], s.y[j],
                            s.nx[j], s.ny[j], s.w[j], s.kap[j], s.comp[j]);
}

}  // namespace rskel
