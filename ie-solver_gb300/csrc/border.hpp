// Bordered-system helper kernels (border_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace rskel {

// out(i, j) = sum_l mask[l] A(l, i) B(l, j) for A (D x na), B (D x nb),
// in FP64; part: masked_cross_scratch(na, nb, D) doubles of scratch.
template <class Real>
void masked_cross(const Real* A, int lda, int na, const Real* B, int ldb, int nb,
                  const unsigned char* mask, int D, double* out, int ldo, double* part,
                  cudaStream_t st);
size_t masked_cross_scratch(int na, int nb, int D);
template <class Real>
void assemble_s(Real* S, int ns, int nb, const Real* root, const Real* mU, const Real* mP, int D,
                const int* allskel, const double* G, cudaStream_t st);
template <class Real>
void border_rhs(Real* M, int ns, int nb, const Real* x, const int* allskel, const double* g1,
                cudaStream_t st);
template <class Real>
void border_sub(Real* nv, const Real* x, const Real* mU, int D, int nb, const Real* alpha,
                const unsigned char* red_mask, cudaStream_t st);
template <class Real>
void border_merge(Real* x, const Real* nv, const unsigned char* red_mask, int D, const int* allskel,
                  const Real* y, int ns, cudaStream_t st);
template <class Real>
void transpose_to(const double* in, int rows, int cols, Real* out, cudaStream_t st);
// U (D x nb) and Psi^T (D x nb), both column major, for h holes with centres
// hc (2h) and radii hr (h) on the device: initialize_U_mat and
// initialize_Psi_mat (linear_solve.cpp:20-112).  pde: 0 Laplace, 2 Stokes.
void border_fill(const double* px, const double* py, const double* w, int n, int pde,
                 const double* hc, const double* hr, int h, double* U, double* PsiT,
                 cudaStream_t st);
template <class Real>
void convert_from_double(const double* in, Real* out, size_t n, cudaStream_t st);
template <class Real>
void convert_to_double(const Real* in, double* out, size_t n, cudaStream_t st);

}  // namespace rskel
