// Domain evaluation: the solution at points off the boundary,
//   u(x) = sum_j K_domain(x, y_j) mu_j + U_forward(x) alpha,
// as boundary_integral_solve assembles it (linear_solve.cpp:140-154,
// 188-266) from Initialization::InitializeDomainKernel
// (initialization.cpp:11-135) and initialize_U_mat at the targets
// (linear_solve.cpp:20-64).  Targets outside the domain (per the caller's
// flags, Boundary::is_in_domain in the reference) get zero.
//
// Kernels of a domain target x and a boundary source y (no diagonal term;
// kernel.cpp:29-104 with tgt.is_boundary false):
//   Laplace          -(w / 2pi) (r . n_y) / |r|^2
//   Stokes           (w / pi) (r . n_y) / |r|^4  r r^T
//   Laplace-Neumann  (w / 2pi) log |r|
// One thread per target, FP64; source tiles of the boundary staged in
// shared memory.
#include <cuda_runtime.h>
#include <math_constants.h>

#include "common.cuh"
#include "domain.hpp"

namespace rskel {

namespace {

constexpr int kTile = 128;
constexpr int kRhs = 8;  // right-hand sides per pass

__global__ void __launch_bounds__(kTile) domain_eval_kernel(DomainParams p, int q0, int nq) {
  extern __shared__ __align__(16) double sm[];
  double* sx = sm;
  double* sy = sx + kTile;
  double* snx = sy + kTile;
  double* sny = snx + kTile;
  double* sw = sny + kTile;
  double* smu = sw + kTile;  // kTile x sd x nq
  const int sd = p.sd;
  const int t = blockIdx.x * kTile + threadIdx.x;
  const bool act = t < p.nt;
  const bool inside = act && (p.mask == nullptr || p.mask[t] != 0);
  const double tx = act ? p.tx[t] : 0.0, ty = act ? p.ty[t] : 0.0;
  double acc[2][kRhs];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int q = 0; q < kRhs; ++q) acc[a][q] = 0.0;
  const double i2pi = 1.0 / (2.0 * CUDART_PI), ipi = 1.0 / CUDART_PI;
  for (int j0 = 0; j0 < p.n; j0 += kTile) {
    const int jc = p.n - j0 < kTile ? p.n - j0 : kTile;
    __syncthreads();
    for (int j = threadIdx.x; j < jc; j += blockDim.x) {
      sx[j] = p.g.x[j0 + j];
      sy[j] = p.g.y[j0 + j];
      snx[j] = p.g.nx[j0 + j];
      sny[j] = p.g.ny[j0 + j];
      sw[j] = p.g.w[j0 + j];
    }
    for (int e = threadIdx.x; e < jc * sd * nq; e += blockDim.x) {
      const int j = e % (jc * sd), q = e / (jc * sd);
      smu[e] = p.mu[(size_t)j0 * sd + j + (size_t)p.ldmu * (q0 + q)];
    }
    __syncthreads();
    if (!inside) continue;
    for (int j = 0; j < jc; ++j) {
      const double rx = tx - sx[j], ry = ty - sy[j];
      const double r2 = rx * rx + ry * ry;
      if (r2 == 0.0) continue;  // a target on a boundary node: no domain kernel there
      if (p.pde == kStokes) {
        const double ir2 = rcp(r2);
        const double c = sw[j] * ipi * (rx * snx[j] + ry * sny[j]) * ir2 * ir2;
#pragma unroll
        for (int q = 0; q < kRhs; ++q) {
          if (q < nq) {
            const double m0 = smu[2 * j + jc * sd * q], m1 = smu[2 * j + 1 + jc * sd * q];
            const double d = c * (rx * m0 + ry * m1);
            acc[0][q] += rx * d;
            acc[1][q] += ry * d;
          }
        }
      } else {
        const double c = p.pde == kLaplace
                             ? -sw[j] * i2pi * (rx * snx[j] + ry * sny[j]) * rcp(r2)
                             : sw[j] * i2pi * 0.5 * log(r2);
#pragma unroll
        for (int q = 0; q < kRhs; ++q)
          if (q < nq) acc[0][q] += c * smu[j + jc * q];
      }
    }
  }
  if (!act) return;
  // U_forward alpha: the hole columns at the target
  if (inside && p.nh > 0 && p.alpha != nullptr) {
    for (int h = 0; h < p.nh; ++h) {
      const double rx = tx - p.hc[2 * h], ry = ty - p.hc[2 * h + 1];
      const double r2 = rx * rx + ry * ry;
      if (p.pde == kLaplace) {
        const double u = 0.5 * log(r2);
#pragma unroll
        for (int q = 0; q < kRhs; ++q)
          if (q < nq) acc[0][q] += u * p.alpha[h + (size_t)p.ldal * (q0 + q)];
      } else if (p.pde == kStokes) {
        const double s = 1.0 / (4.0 * CUDART_PI), ir2 = rcp(r2), lg = -0.5 * log(r2);
#pragma unroll
        for (int q = 0; q < kRhs; ++q) {
          if (q < nq) {
            const double* a = p.alpha + 3 * h + (size_t)p.ldal * (q0 + q);
            acc[0][q] += s * ((lg + rx * rx * ir2) * a[0] + rx * ry * ir2 * a[1] + ry * ir2 * a[2]);
            acc[1][q] += s * (rx * ry * ir2 * a[0] + (lg + ry * ry * ir2) * a[1] - rx * ir2 * a[2]);
          }
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kRhs; ++q) {
    if (q < nq)
      for (int a = 0; a < sd; ++a)
        p.out[(size_t)t * sd + a + (size_t)p.ldo * (q0 + q)] = inside ? acc[a][q] : 0.0;
  }
}

}  // namespace

cudaError_t launch_domain_eval(const DomainParams& p, int nrhs, cudaStream_t st) {
  if (p.nt <= 0 || nrhs <= 0) return cudaSuccess;
  for (int q0 = 0; q0 < nrhs; q0 += kRhs) {
    const int nq = nrhs - q0 < kRhs ? nrhs - q0 : kRhs;
    const size_t smem = sizeof(double) * (5 * kTile + (size_t)kTile * p.sd * nq);
    domain_eval_kernel<<<(p.nt + kTile - 1) / kTile, kTile, smem, st>>>(p, q0, nq);
  }
  return cudaGetLastError();
}

}  // namespace rskel
