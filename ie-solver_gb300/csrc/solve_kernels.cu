// Solve sweeps, dense LU, kernel blocks and the dense matvec.
//
// Sweeps restate SkelFactorization::apply_sweep_matrix / apply_diag_inv_matrix
// and the level loops of solve / multiply_connected_solve
// (ie_solver/skel_factorization/skel_factorization.cpp:388-426, 507-777).
// All compressed boxes of one tree level touch disjoint DOF sets, so a level
// is one launch with one CTA per box; the per-box work is a gather of the
// box's skeleton / redundant rows of x, a few small matrix products with the
// box's factors and a scatter back.
#include <algorithm>
#include <vector>

#include "../../include/rskel.h"
#include "common.cuh"
#include "kernels.hpp"

namespace rskel {

constexpr int kRhsBlock = 8;

// In-place solve of X y = b (LU with pivots) for up to kWarps columns of a
// column-major r x cb block y (ld = r), one warp per column.
template <class Real>
__device__ void lu_solve_cols(const Real* X, const int* piv, int r, Real* y, int ldy, int cb) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = warp; c < cb; c += kWarps) {
    Real* v = y + (size_t)ldy * c;
    if (lane == 0)
      for (int j = 0; j < r; ++j)
        if (piv[j] != j) { Real t = v[j]; v[j] = v[piv[j]]; v[piv[j]] = t; }
    __syncwarp();
    for (int j = 0; j < r; ++j) {
      const Real vj = v[j];
      __syncwarp();
      for (int i = j + 1 + lane; i < r; i += 32) v[i] -= X[i + (size_t)r * j] * vj;
      __syncwarp();
    }
    for (int j = r - 1; j >= 0; --j) {
      const Real vj = v[j] / X[j + (size_t)r * j];
      __syncwarp();
      for (int i = lane; i < j; i += 32) v[i] -= X[i + (size_t)r * j] * vj;
      if (lane == 0) v[j] = vj;
      __syncwarp();
    }
  }
}

template <class Real>
__global__ void __launch_bounds__(kThreads, 8) sweep_kernel(SweepParams p) {
  // Programmatic dependent launch: the next sweep may be scheduled once every
  // CTA of this one has started, and it runs its prologue (its task, factor
  // record and pivots, all written before the solve) while this one works;
  // the reads of x below wait for the previous kernel to complete and its
  // writes to be visible.  Without the launch attribute both are no-ops.
  pdl_launch_dependents();
  const SweepTask t = p.tasks[blockIdx.x];
  const int k = t.k, r = t.r;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sp = smem;
  Real* xs = carve<Real>(sp, k * kRhsBlock);
  Real* xr = carve<Real>(sp, r * kRhsBlock);
  int* piv = carve<int>(sp, r);
  int* sk = carve<int>(sp, k + r);  // the box's skeleton, then redundant, DOF indices
  int* rd = sk + k;
  const Real* fac = reinterpret_cast<const Real*>(p.fac) + t.fac_off;
  const Real* T = fac + fac_T(k, r);
  const Real* L = fac + fac_L(k, r);
  const Real* U = fac + fac_U(k, r);
  const Real* X = fac + fac_X(k, r);
  // The box's factor record (T, L, U, then X_rr: the LU factors in FP64, the
  // explicit inverse in FP32) is copied to shared memory in one coalesced
  // pass, before the wait for the previous level: the copy overlaps that
  // level's work, and the products and solves below read the record without
  // a global round trip per step.
  if (p.stage_fac) {
    const int len = (int)(fac_X(k, r) + (int64_t)r * r);
    Real* fsh = carve<Real>(sp, len);
    batched_copy(fsh, fac, len, threadIdx.x, blockDim.x);
    T = fsh + fac_T(k, r);
    L = fsh + fac_L(k, r);
    U = fsh + fac_U(k, r);
    X = fsh + fac_X(k, r);
  }
  Real* x = reinterpret_cast<Real*>(p.x);
  // pivots and the DOF indices before the wait too: after it, the gather of
  // x is one global round trip instead of two dependent ones
  for (int j = threadIdx.x; j < r; j += blockDim.x) piv[j] = p.piv[t.piv_off + j];
  for (int j = threadIdx.x; j < k; j += blockDim.x) sk[j] = p.dofs[t.skel_off + j];
  for (int j = threadIdx.x; j < r; j += blockDim.x) rd[j] = p.dofs[t.red_off + j];
  __syncthreads();
  pdl_wait();
  for (int c0 = 0; c0 < p.nrhs; c0 += kRhsBlock) {
    const int cb = p.nrhs - c0 < kRhsBlock ? p.nrhs - c0 : kRhsBlock;
    if (k > 0)
      for (TileWalk w(k); w.j < cb; w.next()) {
        const int i = w.i, c = w.j;
        xs[i + k * c] = x[sk[i] + (size_t)p.ld * (c0 + c)];
      }
    if (r > 0)
      for (TileWalk w(r); w.j < cb; w.next()) {
        const int i = w.i, c = w.j;
        xr[i + r * c] = x[rd[i] + (size_t)p.ld * (c0 + c)];
      }
    __syncthreads();
    if (p.mode == kUpSolve || p.mode == kUpPlain || p.mode == kUpTransU) {
      if (r > 0)
        for (TileWalk w(r); w.j < cb; w.next()) {  // x_r -= T^T x_s
          const int i = w.i, c = w.j;
          Real acc = 0;
          for (int l = 0; l < k; ++l) acc += T[l + (size_t)k * i] * xs[l + k * c];
          xr[i + r * c] -= acc;
        }
      __syncthreads();
      if (k > 0)
        for (TileWalk w(k); w.j < cb; w.next()) {
          const int i = w.i, c = w.j;
          Real acc = 0;
          if (p.mode == kUpTransU)  // x_s -= U^T x_r
            for (int l = 0; l < r; ++l) acc += U[l + (size_t)r * i] * xr[l + r * c];
          else  // x_s -= L x_r
            for (int l = 0; l < r; ++l) acc += L[i + (size_t)k * l] * xr[l + r * c];
          xs[i + k * c] -= acc;
        }
      __syncthreads();
    } else if (p.mode == kDiagOnly) {
      // (nothing before the diagonal step)
    } else {  // kDown
      if (r > 0)
        for (TileWalk w(r); w.j < cb; w.next()) {  // x_r -= U x_s
          const int i = w.i, c = w.j;
          Real acc = 0;
          for (int l = 0; l < k; ++l) acc += U[i + (size_t)r * l] * xs[l + k * c];
          xr[i + r * c] -= acc;
        }
      __syncthreads();
      if (k > 0)
        for (TileWalk w(k); w.j < cb; w.next()) {  // x_s -= T x_r
          const int i = w.i, c = w.j;
          Real acc = 0;
          for (int l = 0; l < r; ++l) acc += T[i + (size_t)k * l] * xr[l + r * c];
          xs[i + k * c] -= acc;
        }
      __syncthreads();
    }
    if (p.mode != kDiagOnly)
      if (k > 0)
        for (TileWalk w(k); w.j < cb; w.next()) {
          const int i = w.i, c = w.j;
          x[sk[i] + (size_t)p.ld * (c0 + c)] = xs[i + k * c];
        }
    // the diagonal step x_r <- X_rr^{-1} x_r (the reference's
    // apply_diag_inv_matrix, skel_factorization.cpp:419-426): an LU solve with
    // the FP64 factors, a product with the explicit inverse of the FP32 ones
    const bool diag = p.mode == kUpSolve || p.mode == kDiagOnly;
    if constexpr (sizeof(Real) == 4) {
      // each result straight to x (a thread stores the entries it sums)
      if (r > 0)
        for (TileWalk w(r); w.j < cb; w.next()) {
          const int i = w.i, c = w.j;
          Real v = xr[i + r * c];
          if (diag) {
            Real acc = 0;
            for (int l = 0; l < r; ++l) acc += X[i + (size_t)r * l] * xr[l + r * c];
            v = acc;
          }
          x[rd[i] + (size_t)p.ld * (c0 + c)] = v;
        }
    } else {
      if (diag) {
        lu_solve_cols<Real>(X, piv, r, xr, r, cb);
        __syncthreads();
      }
      if (r > 0)
        for (TileWalk w(r); w.j < cb; w.next()) {
          const int i = w.i, c = w.j;
          x[rd[i] + (size_t)p.ld * (c0 + c)] = xr[i + r * c];
        }
    }
    __syncthreads();
  }
}

void launch_sweep(const SweepParams& p, int num_tasks, int nmax, bool fp32, cudaStream_t st) {
  if (num_tasks <= 0) return;
  size_t es = fp32 ? sizeof(float) : sizeof(double);
  size_t smem = 2 * (((size_t)nmax * kRhsBlock * es + 15) & ~size_t(15)) +
                2 * ((sizeof(int) * nmax + 15) & ~size_t(15)) + 64;
  SweepParams q = p;
  // the whole record: 3 k r + r^2 <= 5 n^2 / 4
  const size_t fe = (size_t)fac_reserve(nmax);
  const size_t fb = (fe * es + 15) & ~size_t(15);
  q.stage_fac = smem + fb <= (size_t)kSmemOptIn;
  if (q.stage_fac) smem += fb;
  if (fp32) {
    set_smem_once<sweep_kernel<float>>();
    launch_pdl(sweep_kernel<float>, dim3(num_tasks), dim3(kThreads), smem, st, q);
  } else {
    set_smem_once<sweep_kernel<double>>();
    launch_pdl(sweep_kernel<double>, dim3(num_tasks), dim3(kThreads), smem, st, q);
  }
}

// ---------------------------------------------------------------------------
// Dense LU (dgetrf with partial pivoting), one CTA, matrix in global memory.
// ---------------------------------------------------------------------------
// LU with partial pivoting of one n x n block by one CTA (dgetrf as the
// reference calls it for the root, ie_mat.cpp:449-470).  With staged != 0
// the block is held in shared memory for the whole factorization.
template <class Real>
__device__ void dense_lu_body(Real* Ag, int n, int* piv, int* status, int staged,
                              unsigned char* smem) {
  __shared__ int s_piv;
  __shared__ int s_bad;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Real* A = staged ? reinterpret_cast<Real*>(smem) : Ag;
  if (staged)
    for (size_t e = threadIdx.x; e < (size_t)n * n; e += blockDim.x) A[e] = Ag[e];
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (warp == 0) {
      double best = -1.0;
      int bi = n;
      for (int i = j + lane; i < n; i += 32) {
        double v = fabs((double)A[i + (size_t)n * j]);
        if (v > best || (v == best && i < bi)) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) {
        s_piv = bi;
        piv[j] = bi;
        if (!(best > 0.0) || !isfinite(best)) s_bad = 1;
      }
    }
    __syncthreads();
    const int pj = s_piv;
    if (pj != j) {
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        Real t = A[j + (size_t)n * c];
        A[j + (size_t)n * c] = A[pj + (size_t)n * c];
        A[pj + (size_t)n * c] = t;
      }
      __syncthreads();
    }
    const Real d = A[j + (size_t)n * j];
    if (d != (Real)0) {
      const Real inv = (Real)1 / d;
      for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)n * j] *= inv;
    }
    __syncthreads();
    for (int c = j + 1 + warp; c < n; c += kWarps) {
      const Real ajc = A[j + (size_t)n * c];
      for (int i = j + 1 + lane; i < n; i += 32) A[i + (size_t)n * c] -= A[i + (size_t)n * j] * ajc;
    }
    __syncthreads();
  }
  if (staged)
    for (size_t e = threadIdx.x; e < (size_t)n * n; e += blockDim.x) Ag[e] = A[e];
  if (threadIdx.x == 0 && s_bad) atomicExch(status, 1);
}

template <class Real>
__global__ void __launch_bounds__(kThreads) dense_lu_kernel(Real* Ag, int n, int* piv,
                                                            int* status, int staged) {
  extern __shared__ __align__(16) unsigned char smem[];
  dense_lu_body<Real>(Ag, n, piv, status, staged, smem);
}

// One root block per CTA (a forest's trees); a block is staged in shared
// memory when it fits in the launch's allocation.
template <class Real>
__global__ void __launch_bounds__(kThreads) dense_lu_batched_kernel(Real* base,
                                                                    const RootTask* tasks,
                                                                    int* piv, int* status,
                                                                    size_t smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const RootTask t = tasks[blockIdx.x];
  const int staged = sizeof(Real) * (size_t)t.n * t.n <= smem_bytes;
  dense_lu_body<Real>(base + t.a_off, t.n, piv + t.piv_off, status, staged, smem);
}

template <class Real>
static void launch_dense_lu_t(Real* a, int n, int* piv, int* status, cudaStream_t st) {
  if (n <= 0) return;
  const size_t bytes = sizeof(Real) * (size_t)n * n;
  const int staged = bytes + 1024 <= (size_t)kSmemOptIn;  // room for the static variables
  set_smem_once<dense_lu_kernel<Real>>();
  dense_lu_kernel<Real><<<1, kThreads, staged ? bytes : 0, st>>>(a, n, piv, status, staged);
}
void launch_dense_lu(double* a, int n, int* piv, int* status, cudaStream_t st) {
  launch_dense_lu_t<double>(a, n, piv, status, st);
}
void launch_dense_lu_f32(float* a, int n, int* piv, int* status, cudaStream_t st) {
  launch_dense_lu_t<float>(a, n, piv, status, st);
}

void launch_dense_lu_batched(void* base, bool fp32, const RootTask* tasks, int count, int nmax,
                             int* piv, int* status, cudaStream_t st) {
  if (count <= 0 || nmax <= 0) return;
  const size_t es = fp32 ? 4 : 8;
  size_t smem = es * (size_t)nmax * nmax;
  if (smem + 1024 > (size_t)kSmemOptIn) smem = (size_t)kSmemOptIn - 1024;
  if (fp32) {
    set_smem_once<dense_lu_batched_kernel<float>>();
    dense_lu_batched_kernel<float><<<count, kThreads, smem, st>>>((float*)base, tasks, piv, status,
                                                                  smem);
  } else {
    set_smem_once<dense_lu_batched_kernel<double>>();
    dense_lu_batched_kernel<double><<<count, kThreads, smem, st>>>((double*)base, tasks, piv,
                                                                   status, smem);
  }
}

// x[idx, c] = LU^{-1} x[idx, c] for the root block (dgetrs), up to kWarps
// columns per CTA, one warp per column.  staged: 0 = work on x and LU in
// global memory; 1 = gathered columns in shared memory (n x cols); 2 = the
// LU factors in shared memory too.
template <class Real>
__device__ void dense_solve_body(const Real* LUg, int n, const int* piv, const int* idx, Real* x,
                                 int ld, int nrhs, int staged, unsigned char* smem) {
  Real* sx = reinterpret_cast<Real*>(smem);
  Real* sl = sx + (size_t)n * nrhs;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Real* LU = LUg;
  if (staged) {
    for (int e = threadIdx.x; e < n * nrhs; e += blockDim.x) {
      const int i = e % n, c = e / n;
      sx[e] = x[(idx ? idx[i] : i) + (size_t)ld * c];
    }
    if (staged == 2) {
      for (size_t e = threadIdx.x; e < (size_t)n * n; e += blockDim.x) sl[e] = LUg[e];
      LU = sl;
    }
    __syncthreads();
  }
  for (int c = warp; c < nrhs; c += kWarps) {
    Real* v = staged ? sx + (size_t)n * c : x + (size_t)ld * c;
    const int* ix = staged ? nullptr : idx;
    auto at = [&](int i) -> Real& { return v[ix ? ix[i] : i]; };
    if (lane == 0)
      for (int j = 0; j < n; ++j)
        if (piv[j] != j) { Real t = at(j); at(j) = at(piv[j]); at(piv[j]) = t; }
    __syncwarp();
    for (int j = 0; j < n; ++j) {
      const Real vj = at(j);
      __syncwarp();
      for (int i = j + 1 + lane; i < n; i += 32) at(i) -= LU[i + (size_t)n * j] * vj;
      __syncwarp();
    }
    for (int j = n - 1; j >= 0; --j) {
      const Real vj = at(j) / LU[j + (size_t)n * j];
      __syncwarp();
      for (int i = lane; i < j; i += 32) at(i) -= LU[i + (size_t)n * j] * vj;
      if (lane == 0) at(j) = vj;
      __syncwarp();
    }
  }
  if (staged) {
    __syncthreads();
    for (int e = threadIdx.x; e < n * nrhs; e += blockDim.x) {
      const int i = e % n, c = e / n;
      x[(idx ? idx[i] : i) + (size_t)ld * c] = sx[e];
    }
  }
}

template <class Real>
__global__ void __launch_bounds__(kThreads) dense_solve_kernel(const Real* LUg, int n,
                                                               const int* piv, const int* idx,
                                                               Real* x, int ld, int nrhs,
                                                               int staged) {
  extern __shared__ __align__(16) unsigned char smem[];
  dense_solve_body<Real>(LUg, n, piv, idx, x, ld, nrhs, staged, smem);
}

// One root block per CTA, all right-hand sides in chunks of kWarps columns,
// each chunk staged as far as the launch's allocation allows.
template <class Real>
__global__ void __launch_bounds__(kThreads) dense_solve_batched_kernel(const Real* base,
                                                                       const RootTask* tasks,
                                                                       const int* piv,
                                                                       const int* dofs, Real* x,
                                                                       int ld, int nrhs,
                                                                       size_t smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const RootTask t = tasks[blockIdx.x];
  for (int c0 = 0; c0 < nrhs; c0 += kWarps) {
    const int cols = nrhs - c0 < kWarps ? nrhs - c0 : kWarps;
    const size_t xb = sizeof(Real) * (size_t)t.n * cols, lb = sizeof(Real) * (size_t)t.n * t.n;
    const int staged = xb + lb <= smem_bytes ? 2 : xb <= smem_bytes ? 1 : 0;
    dense_solve_body<Real>(base + t.a_off, t.n, piv + t.piv_off, dofs + t.idx_off,
                           x + (size_t)ld * c0, ld, cols, staged, smem);
    __syncthreads();
  }
}

void launch_dense_solve_batched(const void* base, bool fp32, const RootTask* tasks, int count,
                                int nmax, const int* piv, const int* dofs, void* x, int ld,
                                int nrhs, cudaStream_t st) {
  if (count <= 0 || nmax <= 0 || nrhs <= 0) return;
  const size_t es = fp32 ? 4 : 8;
  const int cols = nrhs < kWarps ? nrhs : kWarps;
  size_t smem = es * ((size_t)nmax * cols + (size_t)nmax * nmax);
  if (smem > (size_t)kSmemOptIn) smem = (size_t)kSmemOptIn;
  if (fp32) {
    set_smem_once<dense_solve_batched_kernel<float>>();
    dense_solve_batched_kernel<float><<<count, kThreads, smem, st>>>(
        (const float*)base, tasks, piv, dofs, (float*)x, ld, nrhs, smem);
  } else {
    set_smem_once<dense_solve_batched_kernel<double>>();
    dense_solve_batched_kernel<double><<<count, kThreads, smem, st>>>(
        (const double*)base, tasks, piv, dofs, (double*)x, ld, nrhs, smem);
  }
}

// ---------------------------------------------------------------------------
// FP32 root blocks by explicit inverse.  The LU solve above is 2n dependent
// steps per column on every application of the factorization; with the
// inverse formed once per factorization, each application is one product.
// Gauss-Jordan elimination with partial pivoting, one CTA per block, the
// block in registers: thread (tc, ti) = (tid / 16, tid % 16) owns rows
// ti + 16a and columns tc + 16b (a, b < 8), so a column's 128 rows sit in
// one half-warp and its pivot search needs no barrier.  Rows are not
// swapped: step j takes the unused row p_j with the largest |A(p_j, j)|
// (the first on ties), and the in-place update leaves M with
// A^{-1}(j, p_c) = M(p_j, c), which is written out unpermuted.
// ---------------------------------------------------------------------------
constexpr int kInvG = 16;             // thread grid 16 x 16
constexpr int kInvR = kRootInvMax / kInvG;  // rows and columns per thread

__global__ void __launch_bounds__(kInvG * kInvG) root_inverse_kernel(float* base,
                                                                   const RootTask* tasks,
                                                                   int* status) {
  const RootTask t = tasks[blockIdx.x];
  const int n = t.n;
  float* Ag = base + t.a_off;
  const int tid = threadIdx.x, tc = tid >> 4, ti = tid & 15;
  __shared__ float colbuf[2][kRootInvMax];
  __shared__ float rowbuf[2][kRootInvMax];
  __shared__ int s_p[kRootInvMax];
  __shared__ int s_pinv[kRootInvMax];
  __shared__ float s_piv[2];
  __shared__ int s_bad;
  float M[kInvR][kInvR];
#pragma unroll
  for (int a = 0; a < kInvR; ++a)
#pragma unroll
    for (int b = 0; b < kInvR; ++b) {
      const int i = ti + kInvG * a, c = tc + kInvG * b;
      M[a][b] = i < n && c < n ? Ag[i + (size_t)n * c] : 0.f;
    }
  if (tid == 0) s_bad = 0;
  unsigned used = 0;  // bit a: row ti + 16a has been a pivot row
  const unsigned half = 0xffffu << (16 * (tc & 1));
  for (int j = 0; j < n; ++j) {
    const int buf = j & 1, jb = j >> 4;
    if (tc == (j & 15)) {
      // this half-warp holds column j: publish it and pick the pivot row
      float best = -1.f, bv = 0.f;
      int bi = kRootInvMax;
#pragma unroll
      for (int a = 0; a < kInvR; ++a) {
        float v = 0.f;
#pragma unroll
        for (int b = 0; b < kInvR; ++b)
          if (b == jb) v = M[a][b];
        const int i = ti + kInvG * a;
        colbuf[buf][i] = v;
        if (i < n && !((used >> a) & 1u) && fabsf(v) > best) {
          best = fabsf(v);
          bv = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(half, best, o);
        const float ov = __shfl_xor_sync(half, bv, o);
        const int oi = __shfl_xor_sync(half, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bv = ov;
          bi = oi;
        }
      }
      if (ti == 0) {
        const bool ok = best > 0.f && isfinite(best) && bi < n;
        s_p[j] = ok ? bi : 0;
        s_piv[buf] = ok ? bv : 1.f;
        if (!ok) s_bad = 1;
      }
    }
    __syncthreads();
    const int p = s_p[j];
    const float piv = s_piv[buf];
    if (ti == (p & 15)) {
      // the owners of row p publish it scaled by the pivot
      const int pa = p >> 4;
      const float inv = 1.f / piv;
      used |= 1u << pa;
#pragma unroll
      for (int b = 0; b < kInvR; ++b) {
        float v = 0.f;
#pragma unroll
        for (int a = 0; a < kInvR; ++a)
          if (a == pa) v = M[a][b];
        const int c = tc + kInvG * b;
        rowbuf[buf][c] = c == j ? inv : v * inv;
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < kInvR; ++a) {
      const int i = ti + kInvG * a;
      const float ci = colbuf[buf][i];
#pragma unroll
      for (int b = 0; b < kInvR; ++b) {
        const int c = tc + kInvG * b;
        const float rc = rowbuf[buf][c];
        const float m = c == j ? 0.f : M[a][b];
        M[a][b] = i == p ? rc : m - ci * rc;
      }
    }
  }
  __syncthreads();
  // (a singular block repeats pivot rows: the map then stays in range)
  for (int r = tid; r < kRootInvMax; r += blockDim.x) s_pinv[r] = r;
  __syncthreads();
  for (int j = tid; j < n; j += blockDim.x) s_pinv[s_p[j]] = j;
  __syncthreads();
#pragma unroll
  for (int a = 0; a < kInvR; ++a)
#pragma unroll
    for (int b = 0; b < kInvR; ++b) {
      const int r = ti + kInvG * a, c = tc + kInvG * b;
      if (r < n && c < n) Ag[s_pinv[r] + (size_t)n * s_p[c]] = M[a][b];
    }
  if (tid == 0 && s_bad) atomicExch(status, 1);
}

// x[idx, c] <- A^{-1} x[idx, c] per root block, with the explicit inverse:
// one warp per row of the inverse (rows strided over the CTA's warps), a
// CTA per root.  Each lane holds its share of its rows (four entries per
// row, n <= 128) in registers, loaded before the wait for the up sweep, so
// after it the only global round trips are the gather of x and the stores.
// Every row's sum runs over l in the same order for every launch.
constexpr int kRootApplyWarps = 32;
constexpr int kRootRowsPerWarp = kRootInvMax / kRootApplyWarps;

__global__ void __launch_bounds__(32 * kRootApplyWarps) root_apply_kernel(
    const float* base, const RootTask* tasks, const int* dofs, float* x, int ld, int nrhs) {
  pdl_launch_dependents();
  const RootTask t = tasks[blockIdx.x];
  const int n = t.n;
  const float* Ai = base + t.a_off;
  const int* idx = dofs + t.idx_off;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ float sx[kRootInvMax * kRhsBlock];
  __shared__ int sidx[kRootInvMax];
  float a[kRootRowsPerWarp][4];
#pragma unroll
  for (int q = 0; q < kRootRowsPerWarp; ++q) {
    const int i = warp + kRootApplyWarps * q;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int l = lane + 32 * h;
      a[q][h] = i < n && l < n ? Ai[i + (size_t)n * l] : 0.f;
    }
  }
  for (int e = threadIdx.x; e < n; e += blockDim.x) sidx[e] = idx[e];
  __syncthreads();
  pdl_wait();
  for (int c0 = 0; c0 < nrhs; c0 += kRhsBlock) {
    const int cb = nrhs - c0 < kRhsBlock ? nrhs - c0 : kRhsBlock;
    for (int e = threadIdx.x; e < n * cb; e += blockDim.x) {
      const int i = e % n, c = e / n;
      sx[i + n * c] = x[sidx[i] + (size_t)ld * (c0 + c)];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kRootRowsPerWarp; ++q) {
      const int i = warp + kRootApplyWarps * q;
      if (i >= n) break;
      float acc[kRhsBlock];
#pragma unroll
      for (int c = 0; c < kRhsBlock; ++c) acc[c] = 0.f;
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int l = lane + 32 * h;
        if (l < n)
#pragma unroll
          for (int c = 0; c < kRhsBlock; ++c)
            if (c < cb) acc[c] += a[q][h] * sx[l + n * c];
      }
#pragma unroll
      for (int c = 0; c < kRhsBlock; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
      if (lane < cb) {
        float v = acc[0];
#pragma unroll
        for (int c = 1; c < kRhsBlock; ++c)
          if (lane == c) v = acc[c];
        x[sidx[i] + (size_t)ld * (c0 + lane)] = v;
      }
    }
    __syncthreads();
  }
}

void launch_root_inverse(float* base, const RootTask* tasks, int count, int* status,
                         cudaStream_t st) {
  if (count <= 0) return;
  root_inverse_kernel<<<count, kInvG * kInvG, 0, st>>>(base, tasks, status);
}

void launch_root_apply(const float* base, const RootTask* tasks, int count, const int* dofs,
                       float* x, int ld, int nrhs, cudaStream_t st) {
  if (count <= 0 || nrhs <= 0) return;
  launch_pdl(root_apply_kernel, dim3(count), dim3(32 * kRootApplyWarps), 0, st, base, tasks, dofs,
             x, ld, nrhs);
}

// ---------------------------------------------------------------------------
// Explicit inverse of one large block (the bordered system's S, about 1500
// DOFs for 16 holes), FP32 or FP64, by all SMs.  One CTA doing the whole LU in global
// memory was most of a bordered solve's time.  Gauss-Jordan with partial
// pivoting, the columns split over the CTAs of a cooperative launch: at step
// j every CTA reads column j and picks the pivot row itself (the same
// choice everywhere: the unused row with the largest |A(i, j)|, the first
// on ties), reads the pivot row for its own columns, and after a grid
// barrier updates its own columns; a second barrier closes the step.  Rows
// are not moved, so A ends as M with A^{-1}(a, b) = M(piv[a], pinv[b]),
// which the CTAs write out unpermuted.  Data other CTAs wrote are read past
// L1 (ld.global.cg).  The grid barriers spin a bounded number of times:
// on a timeout the kernel raises err and every CTA returns.
// ---------------------------------------------------------------------------
constexpr int kCoopThreads = 256;
constexpr unsigned kBarrierSpins = 1u << 22;

__device__ bool grid_barrier(unsigned* count, unsigned target, int* err,
                             unsigned max_spins = kBarrierSpins) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(count, 1u);
    unsigned spins = 0;
    int ok = 1;
    while (*reinterpret_cast<volatile unsigned*>(count) < target) {
      if (*reinterpret_cast<volatile int*>(err) != 0 || ++spins > max_spins) {
        atomicExch(err, 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Self-test of the bounded grid barrier: `rounds` barriers over a
// cooperative grid of one CTA per SM.  CTA `skip` (none when skip < 0)
// returns before its first arrival, so the other CTAs' waits run out after
// `spins` polls; they raise *err and return.  passed[b] = the barriers CTA b
// got through (the skipped CTA writes nothing).
__global__ void __launch_bounds__(128) barrier_probe_kernel(unsigned* bar, int* err, int skip,
                                                            unsigned spins, int rounds,
                                                            int* passed) {
  if ((int)blockIdx.x == skip) return;  // block-uniform
  int k = 0;
  for (int r = 0; r < rounds; ++r) {
    if (!grid_barrier(bar, (unsigned)(r + 1) * gridDim.x, err, spins)) break;
    ++k;
  }
  if (threadIdx.x == 0) passed[blockIdx.x] = k;
}

size_t coop_inverse_smem(int n, int grid, size_t es) {
  const int cols = (n + grid - 1) / grid;
  return es * (size_t)n + 2 * sizeof(int) * (size_t)n + es * (size_t)cols + 16;
}

template <class Real>
__global__ void __launch_bounds__(kCoopThreads) coop_inverse_kernel(Real* A, int n, Real* Ainv,
                                                                    unsigned* bar, int* err,
                                                                    int* status) {
  extern __shared__ __align__(16) unsigned char smem[];
  Real* col = reinterpret_cast<Real*>(smem);        // column j, all rows
  Real* rowv = col + n;                             // scaled pivot row, own columns
  const int per = (n + gridDim.x - 1) / gridDim.x;
  int* used = reinterpret_cast<int*>(rowv + per);   // row -> 1 once a pivot (then pinv)
  int* piv = used + n;                              // step -> pivot row
  __shared__ Real red_v[kCoopThreads / 32];
  __shared__ int red_i[kCoopThreads / 32];
  __shared__ int s_p;
  __shared__ Real s_inv;
  const int G = gridDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c0 = blockIdx.x * per, c1 = min(n, c0 + per);
  for (int i = tid; i < n; i += blockDim.x) used[i] = 0;
  unsigned epoch = 0;
  for (int j = 0; j < n; ++j) {
    for (int i = tid; i < n; i += blockDim.x) col[i] = __ldcg(A + i + (size_t)n * j);
    __syncthreads();
    Real best = -1;
    int bi = n;
    for (int i = tid; i < n; i += blockDim.x) {
      const Real v = fabs(col[i]);
      if (!used[i] && v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const Real ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { red_v[warp] = best; red_i[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < kCoopThreads / 32; ++w)
        if (red_v[w] > best || (red_v[w] == best && red_i[w] < bi)) { best = red_v[w]; bi = red_i[w]; }
      const bool ok = best > (Real)0 && isfinite(best) && bi < n;
      if (!ok) {  // singular: flagged, continue with the first unused row
        if (blockIdx.x == 0) atomicExch(status, 1);
        bi = 0;
        while (bi < n - 1 && used[bi]) ++bi;
      }
      s_p = bi;
      const Real d = col[bi];
      s_inv = d != (Real)0 ? (Real)1 / d : (Real)0;
    }
    __syncthreads();
    const int p = s_p;
    const Real inv = s_inv;
    for (int c = c0 + tid; c < c1; c += blockDim.x)
      rowv[c - c0] = c == j ? inv : __ldcg(A + p + (size_t)n * c) * inv;
    // every CTA has read column j and its part of row p
    if (!grid_barrier(bar, ++epoch * (unsigned)G, err)) return;
    if (tid == 0) {
      used[p] = 1;
      piv[j] = p;
    }
    for (int c = c0; c < c1; ++c) {
      Real* Ac = A + (size_t)n * c;
      const Real rc = rowv[c - c0];
      for (int i = tid; i < n; i += blockDim.x) {
        const Real m = c == j ? (Real)0 : Ac[i];
        Ac[i] = i == p ? rc : m - col[i] * rc;
      }
    }
    if (!grid_barrier(bar, ++epoch * (unsigned)G, err)) return;
  }
  // pinv over used[] (no longer needed), then the own columns of A^{-1}
  int* pinv = used;
  for (int i = tid; i < n; i += blockDim.x) pinv[i] = i;  // a singular block repeats rows
  __syncthreads();
  for (int j = tid; j < n; j += blockDim.x) pinv[piv[j]] = j;
  __syncthreads();
  for (int b = c0; b < c1; ++b) {
    const Real* Mc = A + (size_t)n * pinv[b];
    for (int a = tid; a < n; a += blockDim.x) Ainv[a + (size_t)n * b] = __ldcg(Mc + piv[a]);
  }
}

// y[a] = sum_b Ainv(a, b) x[b], one thread per row, x staged in shared
// memory a chunk at a time.
template <class Real>
__global__ void __launch_bounds__(128) dense_gemv_kernel(const Real* Ainv, int n, const Real* x,
                                                         Real* y) {
  __shared__ Real xs[1024];
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  Real acc = 0;
  for (int b0 = 0; b0 < n; b0 += 1024) {
    const int nb = min(1024, n - b0);
    __syncthreads();
    for (int e = threadIdx.x; e < nb; e += blockDim.x) xs[e] = x[b0 + e];
    __syncthreads();
    if (a < n)
#pragma unroll 4
      for (int b = 0; b < nb; ++b) acc += Ainv[a + (size_t)n * (b0 + b)] * xs[b];
  }
  if (a < n) y[a] = acc;
}

// CTAs of the cooperative launch: up to two per SM, as many as fit with the
// shared memory n needs (0: n too large for it).
template <class Real>
int coop_inverse_grid(int n) {
  int dev = 0, sms = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  // at least what any grid of >= sms CTAs needs
  const size_t smem = coop_inverse_smem(n, sms, sizeof(Real));
  if (smem + 1024 > (size_t)kSmemOptIn) return 0;
  if (cudaFuncSetAttribute(coop_inverse_kernel<Real>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, coop_inverse_kernel<Real>, kCoopThreads,
                                                    smem) != cudaSuccess ||
      occ < 1)
    return 0;
  return sms * (occ < 2 ? occ : 2);
}

template <class Real>
static cudaError_t launch_coop_inverse_t(Real* a, int n, Real* ainv, unsigned* bar, int* err,
                                         int* status, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int grid = coop_inverse_grid<Real>(n);
  if (grid <= 0) return cudaErrorInvalidValue;
  if (grid > n) grid = n;
  const size_t smem = coop_inverse_smem(n, grid, sizeof(Real));
  cudaError_t e = cudaFuncSetAttribute(coop_inverse_kernel<Real>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(bar, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
  void* args[] = {&a, &n, &ainv, &bar, &err, &status};
  return cudaLaunchCooperativeKernel((const void*)coop_inverse_kernel<Real>, dim3(grid),
                                     dim3(kCoopThreads), args, smem, st);
}
cudaError_t launch_coop_inverse(float* a, int n, float* ainv, unsigned* bar, int* err,
                                int* status, cudaStream_t st) {
  return launch_coop_inverse_t<float>(a, n, ainv, bar, err, status, st);
}
cudaError_t launch_coop_inverse(double* a, int n, double* ainv, unsigned* bar, int* err,
                                int* status, cudaStream_t st) {
  return launch_coop_inverse_t<double>(a, n, ainv, bar, err, status, st);
}

void launch_dense_gemv(const float* ainv, int n, const float* x, float* y, cudaStream_t st) {
  if (n <= 0) return;
  dense_gemv_kernel<float><<<(n + 127) / 128, 128, 0, st>>>(ainv, n, x, y);
}
void launch_dense_gemv(const double* ainv, int n, const double* x, double* y, cudaStream_t st) {
  if (n <= 0) return;
  dense_gemv_kernel<double><<<(n + 127) / 128, 128, 0, st>>>(ainv, n, x, y);
}

template <class Real>
static void launch_dense_solve_t(const Real* lu, int n, const int* piv, const int* idx, Real* x,
                                 int ld, int nrhs, cudaStream_t st) {
  set_smem_once<dense_solve_kernel<Real>>();
  for (int c0 = 0; c0 < nrhs; c0 += kWarps) {
    const int cols = nrhs - c0 < kWarps ? nrhs - c0 : kWarps;
    const size_t xb = sizeof(Real) * (size_t)n * cols, lb = sizeof(Real) * (size_t)n * n;
    const int staged = xb + lb <= (size_t)kSmemOptIn ? 2 : xb <= (size_t)kSmemOptIn ? 1 : 0;
    const size_t smem = staged == 2 ? xb + lb : staged == 1 ? xb : 0;
    dense_solve_kernel<Real><<<1, kThreads, smem, st>>>(lu, n, piv, idx, x + (size_t)ld * c0, ld,
                                                        cols, staged);
  }
}

void launch_dense_solve_gather(const void* lu, bool fp32, int n, const int* piv,
                               const int* idx, void* x, int ld, int nrhs, cudaStream_t st) {
  if (n <= 0 || nrhs <= 0) return;
  if (fp32)
    launch_dense_solve_t<float>((const float*)lu, n, piv, idx, (float*)x, ld, nrhs, st);
  else
    launch_dense_solve_t<double>((const double*)lu, n, piv, idx, (double*)x, ld, nrhs, st);
}

// ---------------------------------------------------------------------------
// Kernel blocks and the dense FP64 matvec
// ---------------------------------------------------------------------------
__device__ __forceinline__ double kernel_gdof(const Geo<double>& g, int pde, int sd, int ti,
                                              int sj) {
  int tp = sd == 1 ? ti : ti >> 1, spt = sd == 1 ? sj : sj >> 1;
  return kernel_entry<double>(pde, g.x[tp], g.y[tp], g.nx[tp], g.ny[tp], ti - tp * sd, g.x[spt],
                              g.y[spt], g.nx[spt], g.ny[spt], g.w[spt], g.kap[spt], sj - spt * sd);
}

__global__ void kernel_block_kernel(Geo<double> g, int pde, int sd, const int* I, int nI,
                                    const int* J, int nJ, double* out) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nI * nJ) return;
  int i = (int)(e % nI), j = (int)(e / nI);
  out[e] = kernel_gdof(g, pde, sd, I[i], J[j]);
}

void launch_kernel_block(const Geo<double>& g, int pde, int sd, const int* I, int nI,
                         const int* J, int nJ, double* out, cudaStream_t st) {
  size_t tot = (size_t)nI * nJ;
  if (!tot) return;
  kernel_block_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(g, pde, sd, I, nI, J, nJ, out);
}

constexpr int kMvTargets = 64;
constexpr int kMvSplit = 4;
constexpr int kMvTile = 256;

// y = K x: CTA per 64 target DOFs, 4 source lanes per target, FP64.
__global__ void __launch_bounds__(kMvTargets * kMvSplit) matvec_kernel(Geo<double> g, int pde,
                                                                       int sd, int D,
                                                                       const double* x, int nrhs,
                                                                       double* y) {
  __shared__ double sx[kMvTile], sy[kMvTile], snx[kMvTile], sny[kMvTile], sw[kMvTile],
      sk[kMvTile];
  __shared__ int sc[kMvTile];
  __shared__ double part[kMvSplit][kMvTargets][kRhsBlock];
  const int tl = threadIdx.x % kMvTargets, sl = threadIdx.x / kMvTargets;
  const int ti = blockIdx.x * kMvTargets + tl;
  const bool valid = ti < D;
  int tp = 0, ta = 0;
  double tx = 0, ty = 0, tnx = 0, tny = 0;
  if (valid) {
    tp = sd == 1 ? ti : ti >> 1;
    ta = ti - tp * sd;
    tx = g.x[tp]; ty = g.y[tp]; tnx = g.nx[tp]; tny = g.ny[tp];
  }
  for (int c0 = 0; c0 < nrhs; c0 += kRhsBlock) {
    const int cb = nrhs - c0 < kRhsBlock ? nrhs - c0 : kRhsBlock;
    double acc[kRhsBlock];
#pragma unroll
    for (int c = 0; c < kRhsBlock; ++c) acc[c] = 0.0;
    for (int s0 = 0; s0 < D; s0 += kMvTile) {
      __syncthreads();
      for (int q = threadIdx.x; q < kMvTile; q += blockDim.x) {
        int sj = s0 + q;
        if (sj < D) {
          int spt = sd == 1 ? sj : sj >> 1;
          sx[q] = g.x[spt]; sy[q] = g.y[spt]; snx[q] = g.nx[spt]; sny[q] = g.ny[spt];
          sw[q] = g.w[spt]; sk[q] = g.kap[spt]; sc[q] = sj - spt * sd;
        }
      }
      __syncthreads();
      if (valid) {
        const int lim = D - s0 < kMvTile ? D - s0 : kMvTile;
        for (int q = sl; q < lim; q += kMvSplit) {
          double kv = kernel_entry<double>(pde, tx, ty, tnx, tny, ta, sx[q], sy[q], snx[q],
                                           sny[q], sw[q], sk[q], sc[q]);
#pragma unroll
          for (int c = 0; c < kRhsBlock; ++c)
            if (c < cb) acc[c] += kv * x[s0 + q + (size_t)D * (c0 + c)];
        }
      }
    }
#pragma unroll
    for (int c = 0; c < kRhsBlock; ++c) part[sl][tl][c] = acc[c];
    __syncthreads();
    if (sl == 0 && valid)
      for (int c = 0; c < cb; ++c) {
        double s = 0.0;
        for (int q = 0; q < kMvSplit; ++q) s += part[q][tl][c];
        y[ti + (size_t)D * (c0 + c)] = s;
      }
    __syncthreads();
  }
}

void launch_matvec(const Geo<double>& g, int pde, int sd, int npts, const double* x, int nrhs,
                   double* y, cudaStream_t st) {
  int D = npts * sd;
  if (D <= 0 || nrhs <= 0) return;
  matvec_kernel<<<(D + kMvTargets - 1) / kMvTargets, kMvTargets * kMvSplit, 0, st>>>(g, pde, sd,
                                                                                   D, x, nrhs, y);
}

// ---------------------------------------------------------------------------
// elementwise
// ---------------------------------------------------------------------------
__global__ void d2f_kernel(const double* in, float* out, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}
__global__ void add_f2d_kernel(double* acc, const float* inc, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) acc[i] += (double)inc[i];
}
__global__ void axpby_kernel(double* y, const double* x, double a, double b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

void launch_d2f(const double* in, float* out, size_t n, cudaStream_t st) {
  if (n) d2f_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
}
void launch_add_f2d(double* acc, const float* inc, size_t n, cudaStream_t st) {
  if (n) add_f2d_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(acc, inc, n);
}
__global__ void f2d_kernel(const float* in, double* out, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}
void launch_f2d(const float* in, double* out, size_t n, cudaStream_t st) {
  if (n) f2d_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
}
void launch_axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st) {
  if (n) axpby_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, x, a, b, n);
}

}  // namespace rskel

namespace rskel {

// out[c] = || x[:, c] ||_2
// Two passes with a fixed summation order (the convergence test must not
// depend on scheduling): kNormBlocks partial sums per column, then one
// warp per column adds them.
constexpr int kNormBlocks = 64;
__global__ void col_norms_partial_kernel(const double* x, int rows, double* part) {
  const int c = blockIdx.y, b = blockIdx.x;
  double s = 0.0;
  for (int i = b * blockDim.x + threadIdx.x; i < rows; i += kNormBlocks * blockDim.x) {
    const double v = x[i + (size_t)rows * c];
    s += v * v;
  }
  s = warp_sum(s);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    part[b + kNormBlocks * (size_t)c] = t;
  }
}

__global__ void col_norms_final_kernel(const double* part, int cols, double* out) {
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= cols) return;
  double s = 0.0;
  for (int b = lane; b < kNormBlocks; b += 32) s += part[b + kNormBlocks * (size_t)c];
  s = warp_sum(s);
  if (lane == 0) out[c] = sqrt(s);
}

// out[c] = ||x[:, c]||_2; out must hold cols + kNormBlocks * cols doubles
// (the tail holds the partial sums).
void launch_col_norms(const double* x, int rows, int cols, double* out, cudaStream_t st) {
  if (cols <= 0) return;
  double* part = out + cols;
  col_norms_partial_kernel<<<dim3(kNormBlocks, cols), 256, 0, st>>>(x, rows, part);
  col_norms_final_kernel<<<(cols + 7) / 8, 256, 0, st>>>(part, cols, out);
}

// out[q + np * c] = |x[seg[q] .. seg[q + 1]), column c|_2: the norm of each
// boundary's part of a batch (one CTA per boundary and column).
__global__ void seg_norms_kernel(const double* x, int rows, const int* seg, int np, double* out) {
  __shared__ double red[kThreads / 32];
  const int q = blockIdx.x, c = blockIdx.y;
  double acc = 0.0;
  for (int i = seg[q] + threadIdx.x; i < seg[q + 1]; i += blockDim.x) {
    const double v = x[i + (size_t)rows * c];
    acc += v * v;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
    out[q + (size_t)np * c] = sqrt(t);
  }
}

void launch_seg_norms(const double* x, int rows, int cols, const int* seg, int np, double* out,
                      cudaStream_t st) {
  if (cols <= 0 || np <= 0) return;
  seg_norms_kernel<<<dim3(np, cols), kThreads, 0, st>>>(x, rows, seg, np, out);
}

// r[l] -= sum_j U[l, j] a[j]
__global__ void gemv_sub_kernel(double* r, const double* U, const double* a, int D, int nb) {
  size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (l >= (size_t)D) return;
  double acc = 0.0;
  for (int j = 0; j < nb; ++j) acc += U[l + (size_t)D * j] * a[j];
  r[l] -= acc;
}

void launch_gemv_sub(double* r, const double* U, const double* a, int D, int nb, cudaStream_t st) {
  if (D > 0) gemv_sub_kernel<<<(D + 255) / 256, 256, 0, st>>>(r, U, a, D, nb);
}

}  // namespace rskel

// ---------------------------------------------------------------------------
// C ABI: rs_barrier_selftest (include/rskel.h)
// ---------------------------------------------------------------------------
extern "C" rs_status rs_barrier_selftest(int device, int skip_block, unsigned spins, int rounds,
                                         int* err, int* passed_min, int* passed_max, float* ms) {
  using namespace rskel;
  if (!err || !passed_min || !passed_max || !ms || rounds < 1 || rounds > 64 || spins < 1 ||
      spins > kBarrierSpins)
    return RS_ERR_ARG;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return RS_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return RS_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return RS_ERR_CUDA;
  int grid = 0;
  if (cudaDeviceGetAttribute(&grid, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return RS_ERR_CUDA;
  if (skip_block >= grid) return RS_ERR_ARG;
  unsigned* bar = nullptr;
  int* d_err = nullptr;
  int* passed = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  rs_status rc = RS_ERR_CUDA;
  std::vector<int> h(grid);
  void* args[] = {&bar, &d_err, &skip_block, &spins, &rounds, &passed};
  if (cudaMalloc(&bar, sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&d_err, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&passed, sizeof(int) * grid) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
      cudaMemset(bar, 0, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(d_err, 0, sizeof(int)) != cudaSuccess ||
      cudaMemset(passed, 0xff, sizeof(int) * grid) != cudaSuccess)
    goto done;
  if (cudaEventRecord(e0, nullptr) != cudaSuccess ||
      cudaLaunchCooperativeKernel((const void*)barrier_probe_kernel, dim3(grid), dim3(128), args,
                                  0, nullptr) != cudaSuccess ||
      cudaEventRecord(e1, nullptr) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(err, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(h.data(), passed, sizeof(int) * grid, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)
    goto done;
  *passed_min = rounds;
  *passed_max = 0;
  for (int b = 0; b < grid; ++b)
    if (b != skip_block) {
      *passed_min = std::min(*passed_min, h[b]);
      *passed_max = std::max(*passed_max, h[b]);
    }
  rc = RS_OK;
done:
  if (rc != RS_OK) (void)cudaGetLastError();
  cudaFree(bar);
  cudaFree(d_err);
  cudaFree(passed);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return rc;
}
