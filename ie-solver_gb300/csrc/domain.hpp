// Domain evaluation (boundary_integral_solve, linear_solve.cpp:188-266).
#pragma once

#include <cuda_runtime.h>

#include "plan.hpp"

namespace rskel {

struct DomainParams {
  Geo<double> g;                 // boundary nodes (device SoA)
  int n, sd, pde;
  const double *tx, *ty;         // targets (device)
  const unsigned char* mask;     // 1 = inside the domain; null = all inside
  int nt;
  const double* mu;              // (n sd) x nrhs, leading dimension ldmu
  int ldmu;
  const double* alpha;           // hole unknowns, leading dimension ldal (may be null)
  int ldal;
  const double* hc;              // hole centres, interleaved
  int nh;
  double* out;                   // (nt sd) x nrhs, leading dimension ldo
  int ldo;
};

cudaError_t launch_domain_eval(const DomainParams& p, int nrhs, cudaStream_t st);

}  // namespace rskel
