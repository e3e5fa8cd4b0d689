// Batched interpolative decomposition of box ID matrices, one CTA per box.
//
// Restates, for every box of a tree level at once:
//   Kernel::get_id_mat   (ie_solver/kernel/kernel.cpp:293-423): rows
//       [K(rows, box); K(box, rows)^T; proxy rows], proxy rows from
//       get_proxy_mat (kernel.cpp:426-591);
//   ie_Mat::id           (ie_solver/ie_mat.cpp:548-588): column-pivoted QR,
//       rank k = first i >= 1 with |R_ii| < tol |R_00| (0 = no compression),
//       Z = R11^{-1} R12.
//
// GB300 layout of the work.  The m x n ID matrix (m ~ 150 .. several
// thousand rows, n <= a few hundred columns) is never stored: rows are
// generated on the fly in chunks of kChunk rows straight into shared memory
// and folded into an n x n triangular factor R by Householder reflections
// (a streamed, unpivoted QR).  Column-pivoted QR of R has exactly the same
// pivots and |R_ii| as column-pivoted QR of the full matrix (the column norms
// it pivots on are invariant under the orthogonal factor), so the pivoted
// factorization then runs on the small n x n tile only, and stops as soon as
// the rank is known.  Norms and the rank decision are accumulated in double
// for both element types.
#include <cstdio>

#include "common.cuh"
#include "kernels.hpp"

namespace rskel {

constexpr int kChunk = 64;  // rows per fold (two per lane)

template <class Real>
struct IdShared {
  Real* R;        // n x n, ld = n
  Real* C;        // kChunk x n, ld = kChunk
  Real* v;        // kChunk
  double* vn1;    // n
  double* vn2;    // n
  int* perm;      // n
  double* red_v;  // kWarps
  int* red_i;     // kWarps
  double* scal;   // [0] tau, [1] scale, [2] thresh, [3] flag
  DofSoA<Real> act;
  DofSoA<Real> row;
  int* kind;      // kChunk
};

template <class Real>
__host__ __device__ size_t id_smem_bytes(int n, bool tile_in_smem) {
  size_t b = 0;
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  if (tile_in_smem) {
    b += al(sizeof(Real) * (size_t)n * n);
    b += al(sizeof(Real) * (size_t)kChunk * n);
  }
  b += al(sizeof(Real) * kChunk);
  b += 2 * al(sizeof(double) * n);
  b += al(sizeof(int) * n);
  b += al(sizeof(double) * kWarps) + al(sizeof(int) * kWarps) + al(sizeof(double) * 4);
  b += dofs_bytes<Real>(n) + dofs_bytes<Real>(kChunk);
  b += al(sizeof(int) * kChunk);
  return b;
}

size_t id_kernel_smem(int n, bool fp32, bool tile_in_smem) {
  return fp32 ? id_smem_bytes<float>(n, tile_in_smem) : id_smem_bytes<double>(n, tile_in_smem);
}

// Fills chunk rows [c0, c0 + cnt) of the virtual ID matrix into S.C.
template <class Real>
__device__ void fill_chunk(const IdParams& p, const IdTask& t, IdShared<Real>& S, int c0,
                           int cnt, double ox, double oy) {
  const int n = t.n, q = t.q;
  const int sd = p.sd;
  const int prow = p.pde == kStokes ? 2 * p.npp : p.npp;  // rows per proxy block
  const double pw = 2.0 * CUDART_PI * t.pr / p.npp;
  if (t.dense_off >= 0) {
    const double* A = p.dense + t.dense_off;
    for (int e = threadIdx.x; e < kChunk * n; e += blockDim.x) {
      int i = e % kChunk, j = e / kChunk;
      S.C[i + (size_t)kChunk * j] = i < cnt ? (Real)A[(c0 + i) + (size_t)t.m_dense * j] : (Real)0;
    }
    __syncthreads();
    return;
  }
  // stage the "other" point of each chunk row
  for (int i = threadIdx.x; i < kChunk; i += blockDim.x) {
    int v = c0 + i;
    int kind = -1;
    if (i < cnt) {
      if (v < q) {
        kind = 0;
        load_dof<Real>(p.geo, sd, p.dofs[t.rows_off + v], ox, oy, S.row, i);
      } else if (v < 2 * q) {
        kind = 1;
        load_dof<Real>(p.geo, sd, p.dofs[t.rows_off + v - q], ox, oy, S.row, i);
      } else {
        int pp = v - 2 * q;
        kind = pp < prow ? 2 : 3;
        int loc = pp < prow ? pp : pp - prow;
        int pt = sd == 2 ? (loc >> 1) : loc;
        double c = p.pxy_cos[pt], s = p.pxy_sin[pt];
        S.row.x[i] = (Real)((t.cx + (t.pr + 0.0) * c) - ox);
        S.row.y[i] = (Real)((t.cy + (t.pr + 0.0) * s) - oy);
        S.row.nx[i] = (Real)c;
        S.row.ny[i] = (Real)s;
        S.row.w[i] = (Real)pw;
        S.row.kap[i] = (Real)0;
        S.row.comp[i] = sd == 2 ? (loc & 1) : 0;
      }
    }
    S.kind[i] = kind;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kChunk * n; e += blockDim.x) {
    int i = e % kChunk, j = e / kChunk;
    int kind = S.kind[i];
    Real val = (Real)0;
    if (kind == 0 || kind == 2) val = kernel_dofs<Real>(p.pde, S.row, i, S.act, j);
    else if (kind == 1 || kind == 3) val = kernel_dofs<Real>(p.pde, S.act, j, S.row, i);
    S.C[i + (size_t)kChunk * j] = val;
  }
  __syncthreads();
}

// Folds the chunk into R: Householder QR of [R; C] (R upper triangular).
template <class Real>
__device__ void fold_chunk(int n, IdShared<Real>& S) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Real* R = S.R;
  Real* C = S.C;
  for (int j = 0; j < n; ++j) {
    if (warp == 0) {
      Real c0 = C[lane + (size_t)kChunk * j], c1 = C[lane + 32 + (size_t)kChunk * j];
      double ss = warp_sum((double)c0 * c0 + (double)c1 * c1);
      double alpha = (double)R[j + (size_t)n * j];
      double tau = 0.0, scale = 0.0;
      if (ss > 0.0) {
        double beta = -copysign(sqrt(alpha * alpha + ss), alpha);
        tau = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
        if (lane == 0) R[j + (size_t)n * j] = (Real)beta;
      }
      S.v[lane] = (Real)(c0 * scale);
      S.v[lane + 32] = (Real)(c1 * scale);
      if (lane == 0) S.scal[0] = tau;
    }
    __syncthreads();
    const Real tau = (Real)S.scal[0];
    if (tau != (Real)0) {
      const Real v0 = S.v[lane], v1 = S.v[lane + 32];
      for (int c = j + 1 + warp; c < n; c += kWarps) {
        Real* cc = C + (size_t)kChunk * c;
        Real part = v0 * cc[lane] + v1 * cc[lane + 32];
        part = warp_sum(part);
        Real wv = R[j + (size_t)n * c] + part;
        Real tw = tau * wv;
        cc[lane] -= tw * v0;
        cc[lane + 32] -= tw * v1;
        if (lane == 0) R[j + (size_t)n * c] -= tw;
      }
    }
    __syncthreads();
  }
}

// Column-pivoted Householder QR of the n x n tile R with early stop at the
// rank (LAPACK dlaqp2 pivoting and norm downdating).  Returns k.
template <class Real>
__device__ int cpqr_rank(int n, double tol, IdShared<Real>& S) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Real* A = S.R;
  const double eps_data = sizeof(Real) == 4 ? 5.9604644775390625e-08 : 1.1102230246251565e-16;
  const double tol3z = sqrt(eps_data);
  for (int c = warp; c < n; c += kWarps) {
    double s = 0.0;
    for (int r = lane; r < n; r += 32) { double a = (double)A[r + (size_t)n * c]; s += a * a; }
    s = warp_sum(s);
    if (lane == 0) { S.vn1[c] = sqrt(s); S.vn2[c] = sqrt(s); S.perm[c] = c; }
  }
  __syncthreads();
  int k = 0;
  for (int i = 0; i < n; ++i) {
    int pvt = block_argmax(S.vn1, i, n, S.red_v, S.red_i);
    if (pvt != i) {
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        Real t = A[r + (size_t)n * pvt];
        A[r + (size_t)n * pvt] = A[r + (size_t)n * i];
        A[r + (size_t)n * i] = t;
      }
      if (threadIdx.x == 0) {
        int tp = S.perm[pvt]; S.perm[pvt] = S.perm[i]; S.perm[i] = tp;
        S.vn1[pvt] = S.vn1[i];
        S.vn2[pvt] = S.vn2[i];
      }
      __syncthreads();
    }
    if (warp == 0) {
      double xs = 0.0;
      for (int r = i + 1 + lane; r < n; r += 32) { double a = (double)A[r + (size_t)n * i]; xs += a * a; }
      xs = warp_sum(xs);
      double alpha = (double)A[i + (size_t)n * i];
      double nrm = sqrt(alpha * alpha + xs);
      int stop = 0;
      if (i == 0) {
        if (lane == 0) S.scal[2] = fabs(tol * nrm);
      } else if (nrm < S.scal[2]) {
        stop = 1;
      }
      double tau = 0.0, scale = 0.0;
      if (!stop && xs > 0.0) {
        double beta = -copysign(nrm, alpha);
        tau = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
        for (int r = i + 1 + lane; r < n; r += 32) A[r + (size_t)n * i] = (Real)((double)A[r + (size_t)n * i] * scale);
        if (lane == 0) A[i + (size_t)n * i] = (Real)beta;
      }
      if (lane == 0) { S.scal[0] = tau; S.scal[3] = stop; }
    }
    __syncthreads();
    if (S.scal[3] != 0.0) { k = i; break; }
    const Real tau = (Real)S.scal[0];
    for (int c = i + 1 + warp; c < n; c += kWarps) {
      Real* cc = A + (size_t)n * c;
      const Real* vv = A + (size_t)n * i;
      Real part = (Real)0;
      for (int r = i + 1 + lane; r < n; r += 32) part += vv[r] * cc[r];
      part = warp_sum(part);
      Real wv = cc[i] + part;
      Real tw = tau * wv;
      if (tau != (Real)0) {
        for (int r = i + 1 + lane; r < n; r += 32) cc[r] -= tw * vv[r];
      }
      __syncwarp();
      if (lane == 0 && tau != (Real)0) cc[i] -= tw;
      __syncwarp();
      // partial column norm downdate (dlaqp2)
      double v1 = S.vn1[c];
      if (v1 != 0.0) {
        double temp = fabs((double)cc[i]) / v1;
        temp = 1.0 - temp * temp;
        temp = temp < 0.0 ? 0.0 : temp;
        double ratio = v1 / S.vn2[c];
        double temp2 = temp * ratio * ratio;
        if (temp2 <= tol3z) {
          double s = 0.0;
          for (int r = i + 1 + lane; r < n; r += 32) { double a = (double)cc[r]; s += a * a; }
          s = warp_sum(s);
          if (lane == 0) { S.vn1[c] = sqrt(s); S.vn2[c] = sqrt(s); }
        } else if (lane == 0) {
          S.vn1[c] = v1 * sqrt(temp);
        }
      }
    }
    __syncthreads();
  }
  return k;
}

template <class Real>
__global__ void __launch_bounds__(kThreads) id_kernel(IdParams p) {
  const IdTask t = p.tasks[blockIdx.x];
  const int n = t.n;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sp = smem;
  IdShared<Real> S;
  if (t.scratch_off < 0) {
    S.R = carve<Real>(sp, n * n);
    S.C = carve<Real>(sp, kChunk * n);
  } else {
    Real* g = reinterpret_cast<Real*>(p.scratch) + t.scratch_off;
    S.R = g;
    S.C = g + (size_t)n * n;
  }
  S.v = carve<Real>(sp, kChunk);
  S.vn1 = carve<double>(sp, n);
  S.vn2 = carve<double>(sp, n);
  S.perm = carve<int>(sp, n);
  S.red_v = carve<double>(sp, kWarps);
  S.red_i = carve<int>(sp, kWarps);
  S.scal = carve<double>(sp, 4);
  S.act = carve_dofs<Real>(sp, n);
  S.row = carve_dofs<Real>(sp, kChunk);
  S.kind = carve<int>(sp, kChunk);

  // FP32 tiles use coordinates relative to the box centre (the differences
  // that matter are then exact to FP32 rounding); FP64 uses absolute ones,
  // as the reference does.
  const double ox = sizeof(Real) == 4 ? t.cx : 0.0;
  const double oy = sizeof(Real) == 4 ? t.cy : 0.0;
  if (t.dense_off < 0)
    for (int j = threadIdx.x; j < n; j += blockDim.x)
      load_dof<Real>(p.geo, p.sd, p.dofs[t.act_off + j], ox, oy, S.act, j);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) S.R[e] = (Real)0;
  __syncthreads();

  const int prow = p.pde == kStokes ? 2 * p.npp : p.npp;
  const int m = t.dense_off >= 0 ? t.m_dense : 2 * t.q + (t.use_proxy ? 2 * prow : 0);
  for (int c0 = 0; c0 < m; c0 += kChunk) {
    int cnt = m - c0 < kChunk ? m - c0 : kChunk;
    fill_chunk<Real>(p, t, S, c0, cnt, ox, oy);
    fold_chunk<Real>(n, S);
  }
  int k = m > 0 ? cpqr_rank<Real>(n, p.tol, S) : 0;
  if (threadIdx.x == 0) p.ranks[t.slot] = k;
  for (int j = threadIdx.x; j < n; j += blockDim.x) p.perm[t.act_off + j] = S.perm[j];
  if (k > 0) {
    // Z = R11^{-1} R12: one warp per column of R12, lanes over rows.
    const int r = n - k;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Real* T = reinterpret_cast<Real*>(p.fac) + t.fac_off + fac_T(k, r);
    for (int c = warp; c < r; c += kWarps) {
      Real* z = S.R + (size_t)n * (k + c);  // solve in place in R12's column
      for (int row = k - 1; row >= 0; --row) {
        Real zr = z[row] / S.R[row + (size_t)n * row];
        __syncwarp();
        for (int q2 = lane; q2 < row; q2 += 32) z[q2] -= zr * S.R[q2 + (size_t)n * row];
        if (lane == 0) z[row] = zr;
        __syncwarp();
      }
      for (int row = lane; row < k; row += 32) T[row + (size_t)k * c] = z[row];
    }
  }
}

void launch_id(const IdParams& p, int num_tasks, size_t smem, bool fp32, cudaStream_t st) {
  if (num_tasks <= 0) return;
  if (fp32) {
    cudaFuncSetAttribute(id_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    id_kernel<float><<<num_tasks, kThreads, smem, st>>>(p);
  } else {
    cudaFuncSetAttribute(id_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    id_kernel<double><<<num_tasks, kThreads, smem, st>>>(p);
  }
}

}  // namespace rskel
