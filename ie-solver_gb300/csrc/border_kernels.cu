// Kernels of the bordered (multiply connected) system, restating
// SkelFactorization::skeletonize :188-305 and multiply_connected_solve
// :596-777 (ie_solver/skel_factorization/skel_factorization.cpp).  The
// redundant / skeleton partition is carried as a per-DOF mask instead of the
// reference's gathered index maps.
#include "border.hpp"
#include "common.cuh"

namespace rskel {

// out(i, j) = sum_l mask[l] * A[l, i] * B[l, j]  (A: D x na, B: D x nb).
// The sum over l (all DOFs, up to millions) is split into chunks: CTA
// (i, group of 8 columns j, chunk) writes its partial sums, and a second
// pass adds the chunks in order (the result does not depend on
// scheduling).  Sums are FP64; in the FP32 variant the products of eight
// consecutive terms of a thread are first added in FP32, so that FP64
// additions (one FP64 instruction per 16 cycles per SM on this GPU) are an
// eighth of the terms.
constexpr int kCrossChunk = 16384;

template <class Real>
__global__ void __launch_bounds__(256) masked_cross_part_kernel(const Real* A, int lda,
                                                                const Real* B, int ldb, int nb,
                                                                const unsigned char* mask, int D,
                                                                double* part) {
  const int i = blockIdx.x, j0 = blockIdx.y * 8, na = gridDim.x;
  const int l0 = blockIdx.z * kCrossChunk, l1 = min(D, l0 + kCrossChunk);
  const int jn = min(8, nb - j0);
  const Real* Ai = A + (size_t)lda * i;
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0;
  if constexpr (sizeof(Real) == 4) {
    float f[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) f[q] = 0.f;
    int run = 0;
    for (int l = l0 + threadIdx.x; l < l1; l += blockDim.x) {
      const float a = mask[l] ? Ai[l] : 0.f;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < jn) f[q] += a * B[l + (size_t)ldb * (j0 + q)];
      if (++run == 8) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          acc[q] += (double)f[q];
          f[q] = 0.f;
        }
        run = 0;
      }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] += (double)f[q];
  } else {
    for (int l = l0 + threadIdx.x; l < l1; l += blockDim.x) {
      const double a = mask[l] ? (double)Ai[l] : 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < jn) acc[q] += a * (double)B[l + (size_t)ldb * (j0 + q)];
    }
  }
  __shared__ double red[8][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    double v = warp_sum(acc[q]);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < jn) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
    part[((size_t)blockIdx.z * na + i) * nb + j0 + threadIdx.x] = v;
  }
}

__global__ void masked_cross_sum_kernel(const double* part, int chunks, int na, int nb,
                                        double* out, int ldo) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= na * nb) return;
  const int i = e % na, j = e / na;
  double v = 0.0;
  for (int c = 0; c < chunks; ++c) v += part[((size_t)c * na + i) * nb + j];
  out[i + (size_t)ldo * j] = v;
}

size_t masked_cross_scratch(int na, int nb, int D) {
  return (size_t)((D + kCrossChunk - 1) / kCrossChunk) * na * nb;
}

template <class Real>
void masked_cross(const Real* A, int lda, int na, const Real* B, int ldb, int nb,
                  const unsigned char* mask, int D, double* out, int ldo, double* part,
                  cudaStream_t st) {
  if (na <= 0 || nb <= 0) return;
  const int chunks = (D + kCrossChunk - 1) / kCrossChunk;
  dim3 grid(na, (nb + 7) / 8, chunks);
  masked_cross_part_kernel<Real><<<grid, 256, 0, st>>>(A, lda, B, ldb, nb, mask, D, part);
  masked_cross_sum_kernel<<<(na * nb + 127) / 128, 128, 0, st>>>(part, chunks, na, nb, out, ldo);
}
template void masked_cross<double>(const double*, int, int, const double*, int, int,
                                   const unsigned char*, int, double*, int, double*, cudaStream_t);
template void masked_cross<float>(const float*, int, int, const float*, int, int,
                                  const unsigned char*, int, double*, int, double*, cudaStream_t);

// S = [Ktilde_root, mU(allskel, :); mP(allskel, :)^T, -I - G], SN = ns + nb.
template <class Real>
__global__ void assemble_s_kernel(Real* S, int ns, int nb, const Real* root, const Real* mU,
                                  const Real* mP, int D, const int* allskel, const double* G) {
  const int SN = ns + nb;
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)SN * SN) return;
  const int i = (int)(e % SN), j = (int)(e / SN);
  Real v;
  if (i < ns && j < ns) v = root[i + (size_t)ns * j];
  else if (i < ns) v = mU[allskel[i] + (size_t)D * (j - ns)];
  else if (j < ns) v = mP[allskel[j] + (size_t)D * (i - ns)];
  else v = (Real)((i == j ? -1.0 : 0.0) - G[(i - ns) + (size_t)nb * (j - ns)]);
  S[e] = v;
}

template <class Real>
void assemble_s(Real* S, int ns, int nb, const Real* root, const Real* mU, const Real* mP, int D,
                const int* allskel, const double* G, cudaStream_t st) {
  size_t tot = (size_t)(ns + nb) * (ns + nb);
  assemble_s_kernel<Real><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(S, ns, nb, root, mU, mP,
                                                                         D, allskel, G);
}
template void assemble_s<double>(double*, int, int, const double*, const double*, const double*,
                                 int, const int*, const double*, cudaStream_t);
template void assemble_s<float>(float*, int, int, const float*, const float*, const float*, int,
                                const int*, const double*, cudaStream_t);

// M[0:ns] = x[allskel]; M[ns + i] = -G1[i]  (G1 = masked_cross(mP, Dw))
template <class Real>
__global__ void border_rhs_kernel(Real* M, int ns, int nb, const Real* x, const int* allskel,
                                  const double* g1) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ns) M[i] = x[allskel[i]];
  else if (i < ns + nb) M[i] = (Real)(-g1[i - ns]);
}

template <class Real>
void border_rhs(Real* M, int ns, int nb, const Real* x, const int* allskel, const double* g1,
                cudaStream_t st) {
  int tot = ns + nb;
  if (tot > 0) border_rhs_kernel<Real><<<(tot + 255) / 256, 256, 0, st>>>(M, ns, nb, x, allskel, g1);
}
template void border_rhs<double>(double*, int, int, const double*, const int*, const double*,
                                 cudaStream_t);
template void border_rhs<float>(float*, int, int, const float*, const int*, const double*,
                                cudaStream_t);

// For redundant l: nv[l] = x[l] - sum_j mU[l, j] alpha[j]; skeleton rows copy x.
template <class Real>
__global__ void border_sub_kernel(Real* nv, const Real* x, const Real* mU, int D, int nb,
                                  const Real* alpha, const unsigned char* red_mask) {
  size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (l >= (size_t)D) return;
  Real v = x[l];
  if (red_mask[l]) {
    double acc = 0.0;
    for (int j = 0; j < nb; ++j) acc += (double)mU[l + (size_t)D * j] * (double)alpha[j];
    v = (Real)((double)v - acc);
  }
  nv[l] = v;
}

template <class Real>
void border_sub(Real* nv, const Real* x, const Real* mU, int D, int nb, const Real* alpha,
                const unsigned char* red_mask, cudaStream_t st) {
  if (D > 0)
    border_sub_kernel<Real><<<(D + 255) / 256, 256, 0, st>>>(nv, x, mU, D, nb, alpha, red_mask);
}
template void border_sub<double>(double*, const double*, const double*, int, int, const double*,
                                 const unsigned char*, cudaStream_t);
template void border_sub<float>(float*, const float*, const float*, int, int, const float*,
                                const unsigned char*, cudaStream_t);

// x[l] = red ? nv[l] : x[l]; then x[allskel[i]] = y[i].
template <class Real>
__global__ void border_merge_kernel(Real* x, const Real* nv, const unsigned char* red_mask, int D) {
  size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (l < (size_t)D && red_mask[l]) x[l] = nv[l];
}
template <class Real>
__global__ void scatter_kernel(Real* x, const int* idx, const Real* y, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[idx[i]] = y[i];
}

template <class Real>
void border_merge(Real* x, const Real* nv, const unsigned char* red_mask, int D, const int* allskel,
                  const Real* y, int ns, cudaStream_t st) {
  if (D > 0) border_merge_kernel<Real><<<(D + 255) / 256, 256, 0, st>>>(x, nv, red_mask, D);
  if (ns > 0) scatter_kernel<Real><<<(ns + 255) / 256, 256, 0, st>>>(x, allskel, y, ns);
}
template void border_merge<double>(double*, const double*, const unsigned char*, int, const int*,
                                   const double*, int, cudaStream_t);
template void border_merge<float>(float*, const float*, const unsigned char*, int, const int*,
                                  const float*, int, cudaStream_t);

template <class Real>
__global__ void transpose_kernel(const double* in, int rows, int cols, Real* out) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)rows * cols) return;
  int i = (int)(e % rows), j = (int)(e / rows);
  out[j + (size_t)cols * i] = (Real)in[e];
}
template <class Real>
void transpose_to(const double* in, int rows, int cols, Real* out, cudaStream_t st) {
  size_t tot = (size_t)rows * cols;
  if (tot) transpose_kernel<Real><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(in, rows, cols, out);
}
template void transpose_to<double>(const double*, int, int, double*, cudaStream_t);
template void transpose_to<float>(const double*, int, int, float*, cudaStream_t);

template <class Real>
__global__ void convert_kernel(const double* in, Real* out, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (Real)in[i];
}
template <class Real>
void convert_from_double(const double* in, Real* out, size_t n, cudaStream_t st) {
  if (n) convert_kernel<Real><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
}
template void convert_from_double<double>(const double*, double*, size_t, cudaStream_t);
template void convert_from_double<float>(const double*, float*, size_t, cudaStream_t);

template <class Real>
__global__ void to_double_kernel(const Real* in, double* out, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}
template <class Real>
void convert_to_double(const Real* in, double* out, size_t n, cudaStream_t st) {
  if (n) to_double_kernel<Real><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
}
template void convert_to_double<double>(const double*, double*, size_t, cudaStream_t);
template void convert_to_double<float>(const float*, double*, size_t, cudaStream_t);

// One thread per point: the point's rows of U for every hole, and its Psi
// entries for the first hole whose circle (radius + 1e-8) holds it.
__global__ void border_fill_kernel(const double* px, const double* py, const double* w, int n,
                                   int pde, const double* hc, const double* hr, int h, double* U,
                                   double* PsiT) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool stokes = pde == 2;
  const size_t D = stokes ? 2 * (size_t)n : (size_t)n;
  const double x0 = px[i], x1 = py[i];
  int member = -1;
  for (int hi = 0; hi < h; ++hi) {
    const double r0 = x0 - hc[2 * hi], r1 = x1 - hc[2 * hi + 1];
    const double r2 = r0 * r0 + r1 * r1, rn = sqrt(r2);
    if (member < 0 && rn < hr[hi] + 1e-8) member = hi;
    if (!stokes) {
      U[i + D * hi] = log(rn);
      PsiT[i + D * hi] = 0.0;
      continue;
    }
    // Stokeslet (two columns) and rotlet about the hole centre
    const double scale = 1.0 / (4.0 * CUDART_PI), lg = log(1.0 / rn), ir2 = 1.0 / r2;
    const size_t c0 = D * (3 * (size_t)hi), c1 = c0 + D, c2 = c1 + D;
    U[2 * i + c0] = scale * (lg + ir2 * r0 * r0);
    U[2 * i + 1 + c0] = scale * (ir2 * r1 * r0);
    U[2 * i + c1] = scale * (ir2 * r0 * r1);
    U[2 * i + 1 + c1] = scale * (lg + ir2 * r1 * r1);
    U[2 * i + c2] = r1 * (scale * ir2);
    U[2 * i + 1 + c2] = -r0 * (scale * ir2);
    PsiT[2 * i + c0] = PsiT[2 * i + 1 + c0] = 0.0;
    PsiT[2 * i + c1] = PsiT[2 * i + 1 + c1] = 0.0;
    PsiT[2 * i + c2] = PsiT[2 * i + 1 + c2] = 0.0;
  }
  if (member < 0) return;
  const double wi = w[i];
  if (!stokes) {
    PsiT[i + D * member] = wi;
  } else {
    const size_t c0 = D * (3 * (size_t)member), c1 = c0 + D, c2 = c1 + D;
    PsiT[2 * i + c0] = wi;
    PsiT[2 * i + 1 + c1] = wi;
    PsiT[2 * i + c2] = wi * x1;
    PsiT[2 * i + 1 + c2] = -wi * x0;
  }
}

void border_fill(const double* px, const double* py, const double* w, int n, int pde,
                 const double* hc, const double* hr, int h, double* U, double* PsiT,
                 cudaStream_t st) {
  if (n <= 0) return;
  border_fill_kernel<<<(n + 255) / 256, 256, 0, st>>>(px, py, w, n, pde, hc, hr, h, U, PsiT);
}

}  // namespace rskel
