// Batched Schur-complement elimination of compressed boxes, one CTA per box.
//
// Restates SkelFactorization::decouple (ie_solver/skel_factorization/
// skel_factorization.cpp:77-128) with the descendant updates of
// get_all_schur_updates (:323-381) folded in differently: under weak
// admissibility every Schur update of a box's descendants lives inside one
// child's DOF set, so the updated matrix of a box is the kernel everywhere
// except on the children's diagonal blocks, which are the children's own
// Schur-complemented blocks E_child (k x k for a compressed child, its whole
// assembled block otherwise).  Each box therefore assembles
//     Ktilde = [E_c1  K(c1,c2) ...; K(c2,c1)  E_c2 ...; ...]
// in shared memory directly in skeleton-first order (s = p[0:k], r = p[k:]),
// and writes its own E = Ktilde(s,s) - L K_r_sn for its parent.  Boxes that
// are not compressed write E = Ktilde.
//
// With T the ID interpolation matrix (k x r):
//   K_r_sn = Ktilde(r,s) - T^T Ktilde(s,s)
//   X_rr   = Ktilde(r,r) - T^T Ktilde(s,r) - K_r_sn T
//   K_sn_r = Ktilde(s,r) - Ktilde(s,s) T
//   X_rr = P^T L U (partial pivoting), U_f = X_rr^{-1} K_r_sn,
//   L_f = K_sn_r X_rr^{-1},  E = Ktilde(s,s) - K_sn_r U_f  (= L_f K_r_sn).
#include "common.cuh"
#include "kernels.hpp"

namespace rskel {

template <class Real>
__host__ __device__ size_t dec_smem_bytes(int n, bool tile_in_smem) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  size_t b = 0;
  if (tile_in_smem) {
    b += al(sizeof(Real) * (size_t)n * (n | 1));  // M (leading dimension n | 1)
    b += al(sizeof(Real) * (size_t)(n / 2 + 1) * (n - n / 2 + 1));  // T (k*r <= n^2/4)
  }
  b += dofs_bytes<Real>(n);
  b += 3 * al(sizeof(int) * n);                   // child, idx, ld
  b += al(sizeof(int64_t) * n);                   // e_base
  b += 2 * al(sizeof(int) * n);                   // order, piv
  b += al(sizeof(double) * 4);
  return b;
}

size_t decouple_kernel_smem(int n, bool fp32, bool tile_in_smem) {
  return fp32 ? dec_smem_bytes<float>(n, tile_in_smem) : dec_smem_bytes<double>(n, tile_in_smem);
}

template <class Real>
__global__ void __launch_bounds__(kThreads) decouple_kernel(DecoupleParams p) {
  const DecoupleTask t = p.tasks[blockIdx.x];
  const int n = t.n;
  const int k = t.slot >= 0 ? p.ranks[t.slot] : 0;
  const int r = n - k;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sp = smem;
  Real *M, *T;
  if (t.scratch_off < 0) {
    M = carve<Real>(sp, n * (n | 1));
    T = carve<Real>(sp, (n / 2 + 1) * (n - n / 2 + 1));
  } else {
    M = reinterpret_cast<Real*>(p.scratch) + t.scratch_off;
    T = M + (size_t)n * (n | 1);
  }
  DofSoA<Real> act = carve_dofs<Real>(sp, n);
  int* bchild = carve<int>(sp, n);
  int* bidx = carve<int>(sp, n);
  int* bld = carve<int>(sp, n);
  int64_t* bbase = carve<int64_t>(sp, n);
  int* order = carve<int>(sp, n);
  int* piv = carve<int>(sp, n);
  double* scal = carve<double>(sp, 4);

  const Real* E_in = reinterpret_cast<const Real*>(p.epool);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    load_dof<Real>(p.geo, p.sd, p.dofs[t.act_off + j], 0.0, 0.0, act, j);
    int c = 0;
    while (c < 3 && j >= t.cstart[c + 1]) ++c;  // the run of active position j
    bchild[j] = c;
    bidx[j] = j - t.cstart[c];
    bld[j] = t.cld[c];
    bbase[j] = t.ce[c];
    order[j] = k > 0 ? p.perm[t.perm_off + j] : j;
  }
  __syncthreads();
  // Assemble Ktilde in skeleton-first order.
  if (n > 0)
    for (TileWalk w(n); w.j < n; w.next()) {
      const int a = w.i, b = w.j;
      const int ia = order[a], ib = order[b];
      Real val;
      if (bchild[ia] == bchild[ib] && bbase[ia] >= 0) {
        val = E_in[bbase[ia] + bidx[ia] + (int64_t)bld[ia] * bidx[ib]];
      } else {
        val = kernel_dofs<Real>(p.pde, act, ia, act, ib);
      }
      M[a + (size_t)(n | 1) * b] = val;
    }
  __syncthreads();
  Real* E_out = reinterpret_cast<Real*>(p.epool) + t.e_off;
  if (k == 0) {
    for (TileWalk w(n); w.j < n; w.next()) E_out[w.e()] = M[w.i + (size_t)(n | 1) * w.j];
    return;
  }
  Real* fac = reinterpret_cast<Real*>(p.fac) + t.fac_off;
  // T (k x r, column major in the record) is held transposed, Tt(i, l) =
  // T(l, i) at Tt[i + r l]: the products below walk i across the threads,
  // which then read consecutive words
  for (int e = threadIdx.x; e < k * r; e += blockDim.x) {
    const int l = e % k, i = e / k;
    T[i + (size_t)r * l] = fac[fac_T(k, r) + e];
  }
  __syncthreads();
  // an odd leading dimension: walks along a row (threads across columns)
  // then hit distinct banks
  const size_t ld = n | 1;
  Real* Mss = M;
  Real* Msr = M + ld * k;
  Real* Mrs = M + k;
  Real* Mrr = M + k + ld * k;
  // 1) K_r_sn = Mrs - T^T Mss  (r x k), in place
  if (r > 0)
    for (TileWalk w(r); w.j < k; w.next()) {
      const int i = w.i, j = w.j;
      Real acc = Mrs[i + ld * j];
      for (int l = 0; l < k; ++l) acc -= T[i + (size_t)r * l] * Mss[l + ld * j];
      Mrs[i + ld * j] = acc;
    }
  __syncthreads();
  // 2) X_rr = Mrr - T^T Msr - K_r_sn T  (r x r), in place
  if (r > 0)
    for (TileWalk w(r); w.j < r; w.next()) {
      const int i = w.i, j = w.j;
      Real a1 = 0, a2 = 0;
      for (int l = 0; l < k; ++l) {
        a1 += T[i + (size_t)r * l] * Msr[l + ld * j];
        a2 += Mrs[i + ld * l] * T[j + (size_t)r * l];
      }
      Mrr[i + ld * j] = (Mrr[i + ld * j] - a1) - a2;
    }
  __syncthreads();
  // 3) K_sn_r = Msr - Mss T  (k x r), in place
  if (k > 0)
    for (TileWalk w(k); w.j < r; w.next()) {
      const int i = w.i, j = w.j;
      Real acc = Msr[i + ld * j];
      for (int l = 0; l < k; ++l) acc -= Mss[i + ld * l] * T[j + (size_t)r * l];
      Msr[i + ld * j] = acc;
    }
  __syncthreads();
  if (threadIdx.x == 0) scal[0] = 0.0;
  if constexpr (sizeof(Real) == 4) {
    // FP32 factorization: X_rr is inverted explicitly (Gauss-Jordan with
    // partial pivoting), so that U_f, L_f and the solve's diagonal step are
    // matrix products spread over the whole CTA instead of one warp-serial
    // triangular solve per column.  The refinement absorbs the explicit
    // inverse's slightly larger rounding error.  Rows are not moved: step j
    // takes the row piv[j] with the largest |X(piv[j], j)| among those not
    // yet pivot rows, and the in-place update leaves M with
    // X^{-1}(a, b) = M(piv[a], pinv[b]).  Ties go to the row that
    // dgetrf-style row interchanges would hold at the smallest position
    // (pos[] tracks those positions), so the pivot sequence is that of
    // elimination with explicit swaps.  Column j + 1 and the scaled pivot row
    // go through double buffers, so a step takes two CTA barriers.  The
    // assembly's index arrays are free by now and hold the buffers.
    float* colbuf[2] = {reinterpret_cast<float*>(bchild), reinterpret_cast<float*>(bidx)};
    float* rowbuf[2] = {reinterpret_cast<float*>(bld), reinterpret_cast<float*>(order)};
    int* pos = reinterpret_cast<int*>(bbase);  // row -> position (>= j: not yet a pivot row)
    int* row_at = pos + n;                     // position -> row
    for (int i = threadIdx.x; i < r; i += blockDim.x) {
      colbuf[0][i] = Mrr[i];
      pos[i] = i;
      row_at[i] = i;
    }
    __syncthreads();
    for (int j = 0; j < r; ++j) {
      const int buf = j & 1;
      // every warp finds the pivot row itself (no barrier for a broadcast)
      float best = -1.f;
      int bi = r, bp = r;
      for (int i = lane; i < r; i += 32) {
        const int ps = pos[i];
        if (ps < j) continue;
        const float v = fabsf(colbuf[buf][i]);
        if (v > best || (v == best && ps < bp)) { best = v; bi = i; bp = ps; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        const int op = __shfl_xor_sync(0xffffffffu, bp, o);
        if (ov > best || (ov == best && op < bp)) { best = ov; bi = oi; bp = op; }
      }
      const bool ok = best > 0.f && isfinite(best) && bi < r;
      const int pr = ok ? bi : row_at[j];  // a singular block: any row, flagged
      if (threadIdx.x == 0) {
        piv[j] = pr;
        if (!ok) scal[0] = 1.0;
      }
      const Real d = Mrr[pr + ld * j];
      const Real inv = d != (Real)0 ? (Real)1 / d : (Real)0;
      for (int c = threadIdx.x; c < r; c += blockDim.x)
        rowbuf[buf][c] = c == j ? inv : Mrr[pr + ld * c] * inv;
      __syncthreads();
      // (every warp has read pos for this step by now): the interchange of
      // positions j and pos[pr]
      if (threadIdx.x == 0) {
        const int q = row_at[j], pp = pos[pr];
        row_at[pp] = q;
        pos[q] = pp;
        row_at[j] = pr;
        pos[pr] = j;
      }
      if (r > 0)
        for (TileWalk w(r); w.j < r; w.next()) {
          const int i = w.i, c = w.j;
          const Real m = c == j ? (Real)0 : Mrr[i + ld * c];
          const Real v = i == pr ? rowbuf[buf][c] : m - colbuf[buf][i] * rowbuf[buf][c];
          Mrr[i + ld * c] = v;
          if (c == j + 1) colbuf[buf ^ 1][i] = v;
        }
      __syncthreads();
    }
    int* pinv = bchild;
    for (int j = threadIdx.x; j < r; j += blockDim.x) pinv[j] = j;  // a singular block repeats rows
    __syncthreads();
    for (int j = threadIdx.x; j < r; j += blockDim.x) pinv[piv[j]] = j;
    __syncthreads();
    Real* Lo = fac + fac_L(k, r);
    Real* Uo = fac + fac_U(k, r);
    Real* Xo = fac + fac_X(k, r);
    // X^{-1}(a, b) = M(piv[a], pinv[b]) to the record, then back over M in
    // its own order (a CTA reads its own global writes after the barrier)
    if (r > 0)
      for (TileWalk w(r); w.j < r; w.next()) {
        const int i = w.i, j = w.j;
        const int e = w.e();
        Xo[e] = Mrr[piv[i] + ld * pinv[j]];
      }
    __syncthreads();
    if (r > 0)
      for (TileWalk w(r); w.j < r; w.next()) {
        const int i = w.i, j = w.j;
        const int e = w.e();
        Mrr[i + ld * j] = Xo[e];
      }
    __syncthreads();
    // U_f = X^{-1} K_r_sn (r x k) and L_f = K_sn_r X^{-1} (k x r), to the
    // record.  The sums run over the DOFs in their own order: in pivot order
    // the Stokes x / y pairs no longer cancel early, and the FP32
    // factorization loses accuracy.
    // (U_f also goes to T's bytes, free since step 3, for E below)
    Real* Us = T;
    if (r > 0)
      for (TileWalk w(r); w.j < k; w.next()) {
        const int i = w.i, j = w.j;
        const int e = w.e();
        Real acc = 0;
        for (int l = 0; l < r; ++l) acc += Mrr[i + ld * l] * Mrs[l + ld * j];
        Uo[e] = acc;
        Us[e] = acc;
      }
    if (k > 0)
      for (TileWalk w(k); w.j < r; w.next()) {
        const int i = w.i, j = w.j;
        const int e = w.e();
        Real acc = 0;
        for (int l = 0; l < r; ++l) acc += Msr[i + ld * l] * Mrr[l + ld * j];
        Lo[e] = acc;
      }
    __syncthreads();  // U_f is read back below (same CTA)
    // E = Mss - K_sn_r U_f  (k x k)
    if (k > 0)
      for (TileWalk w(k); w.j < k; w.next()) {
        const int i = w.i, j = w.j;
        const int e = w.e();
        Real acc = Mss[i + ld * j];
        for (int l = 0; l < r; ++l) acc -= Msr[i + ld * l] * Us[l + (size_t)r * j];
        E_out[e] = acc;
      }
    for (int j = threadIdx.x; j < r; j += blockDim.x) p.piv[t.piv_off + j] = j;
    if (threadIdx.x == 0 && scal[0] != 0.0) atomicExch(p.status, 1);
    return;
  }
  // 4) LU of X_rr with partial pivoting (dgetrf), in place.
  for (int j = 0; j < r; ++j) {
    if (warp == 0) {
      double best = -1.0;
      int bi = r;
      for (int i = j + lane; i < r; i += 32) {
        double v = fabs((double)Mrr[i + ld * j]);
        if (v > best || (v == best && i < bi)) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) {
        piv[j] = bi;
        if (!(best > 0.0) || !isfinite(best)) scal[0] = 1.0;
      }
    }
    __syncthreads();
    const int pj = piv[j];
    if (pj != j) {
      for (int c = threadIdx.x; c < r; c += blockDim.x) {
        Real tmp = Mrr[j + ld * c];
        Mrr[j + ld * c] = Mrr[pj + ld * c];
        Mrr[pj + ld * c] = tmp;
      }
      __syncthreads();
    }
    const Real d = Mrr[j + ld * j];
    if (d != (Real)0) {
      const Real inv = (Real)1 / d;
      for (int i = j + 1 + threadIdx.x; i < r; i += blockDim.x) Mrr[i + ld * j] *= inv;
    }
    __syncthreads();
    const int rem = r - j - 1;
    if (rem > 0)
      for (TileWalk w(rem); w.j < rem; w.next()) {
        const int i = j + 1 + w.i, c = j + 1 + w.j;
        Mrr[i + ld * c] -= Mrr[i + ld * j] * Mrr[j + ld * c];
      }
    __syncthreads();
  }
  // 5) U_f = X^{-1} K_r_sn, in place over Mrs (one warp per column).
  const int nwarps = blockDim.x >> 5;
  for (int c = warp; c < k; c += nwarps) {
    Real* y = Mrs + ld * c;
    if (lane == 0)
      for (int j = 0; j < r; ++j)
        if (piv[j] != j) { Real tmp = y[j]; y[j] = y[piv[j]]; y[piv[j]] = tmp; }
    __syncwarp();
    for (int j = 0; j < r; ++j) {
      const Real yj = y[j];
      __syncwarp();
      for (int i = j + 1 + lane; i < r; i += 32) y[i] -= Mrr[i + ld * j] * yj;
      __syncwarp();
    }
    for (int j = r - 1; j >= 0; --j) {
      const Real yj = y[j] / Mrr[j + ld * j];
      __syncwarp();
      for (int i = lane; i < j; i += 32) y[i] -= Mrr[i + ld * j] * yj;
      if (lane == 0) y[j] = yj;
      __syncwarp();
    }
  }
  __syncthreads();
  // 6) E = Mss - K_sn_r U_f  (k x k), in place over Mss.
  if (k > 0)
    for (TileWalk w(k); w.j < k; w.next()) {
      const int i = w.i, j = w.j;
      Real acc = 0;
      for (int l = 0; l < r; ++l) acc += Msr[i + ld * l] * Mrs[l + ld * j];
      Mss[i + ld * j] -= acc;
    }
  __syncthreads();
  // 7) L_f = K_sn_r X^{-1}: solve X^T y = K_sn_r(i,:)^T per row (one warp per row).
  for (int i = warp; i < k; i += nwarps) {
    Real* y = Msr + i;  // stride ld
    for (int j = 0; j < r; ++j) {  // U^T z = b
      const Real yj = y[ld * j] / Mrr[j + ld * j];
      __syncwarp();
      for (int q = j + 1 + lane; q < r; q += 32) y[ld * q] -= Mrr[j + ld * q] * yj;
      if (lane == 0) y[ld * j] = yj;
      __syncwarp();
    }
    for (int j = r - 1; j >= 0; --j) {  // L^T w = z (unit diagonal)
      const Real yj = y[ld * j];
      __syncwarp();
      for (int q = lane; q < j; q += 32) y[ld * q] -= Mrr[j + ld * q] * yj;
      __syncwarp();
    }
    if (lane == 0)
      for (int j = r - 1; j >= 0; --j)
        if (piv[j] != j) { Real tmp = y[ld * j]; y[ld * j] = y[ld * piv[j]]; y[ld * piv[j]] = tmp; }
    __syncwarp();
  }
  __syncthreads();
  // 8) write L_f (k x r), U_f (r x k), X_rr LU (r x r), pivots, E (k x k).
  Real* Lo = fac + fac_L(k, r);
  Real* Uo = fac + fac_U(k, r);
  Real* Xo = fac + fac_X(k, r);
  if (k > 0)
    for (TileWalk w(k); w.j < r; w.next()) {
      const int i = w.i, j = w.j;
      Lo[w.e()] = Msr[i + ld * j];
    }
  if (r > 0)
    for (TileWalk w(r); w.j < k; w.next()) {
      const int i = w.i, j = w.j;
      Uo[w.e()] = Mrs[i + ld * j];
    }
  if (r > 0)
    for (TileWalk w(r); w.j < r; w.next()) {
      const int i = w.i, j = w.j;
      const int e = w.e();
      Xo[e] = Mrr[i + ld * j];
    }
  if (k > 0)
    for (TileWalk w(k); w.j < k; w.next()) {
      const int i = w.i, j = w.j;
      const int e = w.e();
      E_out[e] = Mss[i + ld * j];
    }
  for (int j = threadIdx.x; j < r; j += blockDim.x) p.piv[t.piv_off + j] = piv[j];
  if (threadIdx.x == 0 && scal[0] != 0.0) atomicExch(p.status, 1);
}

// threads: 256 (default) or 128 per box; every loop of the kernel strides
// by blockDim.x (or its warp count).
void launch_decouple(const DecoupleParams& p, int num_tasks, size_t smem, bool fp32,
                     cudaStream_t st, int threads) {
  if (num_tasks <= 0) return;
  const int nt = threads == 128 ? 128 : kThreads;
  if (fp32) {
    set_smem_once<decouple_kernel<float>>();
    decouple_kernel<float><<<num_tasks, nt, smem, st>>>(p);
  } else {
    set_smem_once<decouple_kernel<double>>();
    decouple_kernel<double><<<num_tasks, nt, smem, st>>>(p);
  }
}

}  // namespace rskel
