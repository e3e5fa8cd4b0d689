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

// C = C0 - A B (kSub) or C = A B for an m x n result, over one CTA on 2 x 2
// register tiles {i, i + hm} x {j, j + hn} (hm = ceil(m / 2), hn =
// ceil(n / 2)): a step of the sums loads two elements of A and two of B for
// four independent multiply-adds, and the threads of a warp read
// consecutive rows of A.  A(i, l) is at A[i + al l], B(l, j) at
// B[bl l + bj j]; every element's sum runs over l in increasing order, as a
// loop of one element per thread would run it.  C0 may alias C (a thread
// reads its own tile before writing it).  The result also goes to C2 when
// it is given.
template <bool kSub, class Real>
__device__ __forceinline__ void cta_gemm(int m, int n, int kk, const Real* A, int al,
                                         const Real* B, int bl, int bj, const Real* C0, int ld0,
                                         Real* C, int ldc, Real* C2 = nullptr, int ldc2 = 0) {
  const int hm = (m + 1) >> 1, hn = (n + 1) >> 1;
  if (hm == 0 || hn == 0) return;
  for (TileWalk w(hm); w.j < hn; w.next()) {
    const int i0 = w.i, j0 = w.j;
    const bool ri = i0 + hm < m, rj = j0 + hn < n;
    const int i1 = ri ? i0 + hm : i0, j1 = rj ? j0 + hn : j0;
    Real c00 = 0, c10 = 0, c01 = 0, c11 = 0;
    if constexpr (kSub) {
      c00 = C0[i0 + ld0 * j0];
      c10 = C0[i1 + ld0 * j0];
      c01 = C0[i0 + ld0 * j1];
      c11 = C0[i1 + ld0 * j1];
    }
    const Real* a0 = A + i0;
    const Real* a1 = A + i1;
    const Real* b0 = B + bj * j0;
    const Real* b1 = B + bj * j1;
    for (int l = 0; l < kk; ++l) {
      const Real x0 = a0[al * l], x1 = a1[al * l];
      const Real y0 = b0[bl * l], y1 = b1[bl * l];
      if constexpr (kSub) {
        c00 -= x0 * y0;
        c10 -= x1 * y0;
        c01 -= x0 * y1;
        c11 -= x1 * y1;
      } else {
        c00 += x0 * y0;
        c10 += x1 * y0;
        c01 += x0 * y1;
        c11 += x1 * y1;
      }
    }
    auto put = [&](Real* D, int ld) {
      D[i0 + ld * j0] = c00;
      if (ri) D[i1 + ld * j0] = c10;
      if (rj) D[i0 + ld * j1] = c01;
      if (ri && rj) D[i1 + ld * j1] = c11;
    };
    put(C, ldc);
    if (C2 != nullptr) put(C2, ldc2);
  }
}


template <class Real>
__global__ void __launch_bounds__(kThreads) decouple_kernel(DecoupleParams p) {
  const DecoupleTask t = p.tasks[blockIdx.x];
  const int n = t.n;
  const int k = t.slot >= 0 ? p.ranks[t.slot] : 0;
  const int r = n - k;
  long long clk[5];
  clk[0] = clock64();
  auto stamp = [&](int q) { clk[q] = clock64(); };
  auto report = [&]() {
    if (p.phase_clk != nullptr && threadIdx.x == 0) {
      long long* o = p.phase_clk + 6 * (size_t)blockIdx.x;
      for (int q = 0; q < 4; ++q) o[q] = clk[q + 1] - clk[q];
      o[4] = n;
      o[5] = k;
    }
  };
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
    const int dof = p.dofs[t.act_off + j];
    const int oj = k > 0 ? p.perm[t.perm_off + j] : j;
    load_dof<Real>(p.geo, p.sd, dof, 0.0, 0.0, act, j);
    int c = 0;
    while (c < 3 && j >= t.cstart[c + 1]) ++c;  // the run of active position j
    bchild[j] = c;
    bidx[j] = j - t.cstart[c];
    bld[j] = t.cld[c];
    bbase[j] = t.ce[c];
    order[j] = oj;
  }
  __syncthreads();
  // Assemble Ktilde in skeleton-first order.
  // First the children's E-block entries, four loads in flight per thread
  // before their stores, then the kernel entries.
  if (n > 0) {
    for (TileWalk w(n); w.j < n;) {
      int dst[4];
      Real val[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        dst[q] = -1;
        if (w.j < n) {
          const int ia = order[w.i], ib = order[w.j];
          if (bchild[ia] == bchild[ib] && bbase[ia] >= 0) {
            dst[q] = w.i + (n | 1) * w.j;
            val[q] = E_in[bbase[ia] + bidx[ia] + (int64_t)bld[ia] * bidx[ib]];
          }
          w.next();
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (dst[q] >= 0) M[dst[q]] = val[q];
    }
    for (TileWalk w(n); w.j < n; w.next()) {
      const int ia = order[w.i], ib = order[w.j];
      if (!(bchild[ia] == bchild[ib] && bbase[ia] >= 0))
        M[w.i + (size_t)(n | 1) * w.j] = kernel_dofs<Real>(p.pde, act, ia, act, ib);
    }
  }
  __syncthreads();
  stamp(1);
  Real* E_out = reinterpret_cast<Real*>(p.epool) + t.e_off;
  if (k == 0) {
    for (TileWalk w(n); w.j < n; w.next()) E_out[w.e()] = M[w.i + (size_t)(n | 1) * w.j];
    stamp(2);
    stamp(3);
    stamp(4);
    report();
    return;
  }
  Real* fac = reinterpret_cast<Real*>(p.fac) + t.fac_off;
  // T (k x r, column major in the record) is held transposed, Tt(i, l) =
  // T(l, i) at Tt[i + r l]: the products below walk i across the threads,
  // which then read consecutive words
  {
    const Real* Tg = fac + fac_T(k, r);
    const int kr = k * r, nt = blockDim.x;
    for (int e0 = threadIdx.x; e0 < kr; e0 += 4 * nt) {  // four loads in flight
      Real v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (e0 + q * nt < kr) v[q] = Tg[e0 + q * nt];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = e0 + q * nt;
        if (e < kr) T[e / k + (size_t)r * (e % k)] = v[q];
      }
    }
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
  cta_gemm<true>(r, k, k, T, r, Mss, 1, (int)ld, Mrs, (int)ld, Mrs, (int)ld);
  __syncthreads();
  // 2) X_rr = Mrr - T^T Msr - K_r_sn T  (r x r), in place; the two sums are
  //    kept apart and subtracted in that order
  if (r > 0) {
    const int h = (r + 1) >> 1;
    for (TileWalk w(h); w.j < h; w.next()) {
      const int i0 = w.i, j0 = w.j;
      const bool ri = i0 + h < r, rj = j0 + h < r;
      const int i1 = ri ? i0 + h : i0, j1 = rj ? j0 + h : j0;
      Real p00 = 0, p10 = 0, p01 = 0, p11 = 0, q00 = 0, q10 = 0, q01 = 0, q11 = 0;
      for (int l = 0; l < k; ++l) {
        const Real t0 = T[i0 + (size_t)r * l], t1 = T[i1 + (size_t)r * l];
        const Real s0 = Msr[l + ld * j0], s1 = Msr[l + ld * j1];
        const Real u0 = Mrs[i0 + ld * l], u1 = Mrs[i1 + ld * l];
        const Real v0 = T[j0 + (size_t)r * l], v1 = T[j1 + (size_t)r * l];
        p00 += t0 * s0;
        p10 += t1 * s0;
        p01 += t0 * s1;
        p11 += t1 * s1;
        q00 += u0 * v0;
        q10 += u1 * v0;
        q01 += u0 * v1;
        q11 += u1 * v1;
      }
      Mrr[i0 + ld * j0] = (Mrr[i0 + ld * j0] - p00) - q00;
      if (ri) Mrr[i1 + ld * j0] = (Mrr[i1 + ld * j0] - p10) - q10;
      if (rj) Mrr[i0 + ld * j1] = (Mrr[i0 + ld * j1] - p01) - q01;
      if (ri && rj) Mrr[i1 + ld * j1] = (Mrr[i1 + ld * j1] - p11) - q11;
    }
  }
  __syncthreads();
  // 3) K_sn_r = Msr - Mss T  (k x r), in place
  cta_gemm<true>(k, r, k, Mss, (int)ld, T, r, 1, Msr, (int)ld, Msr, (int)ld);
  __syncthreads();
  stamp(2);
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
    const int hr = (r + 1) >> 1;
    // Pivot search of one step, by every warp (no barrier for a broadcast):
    // the largest |value| over rows whose position is at least j, ties to the
    // smallest position.  Non-negative floats order as their bit patterns, so
    // two warp reductions give it: the largest value, then the smallest
    // position holding it.  A NaN's pattern lies above infinity's.  val(i)
    // and pos_of(i) give a row's candidate value and position.
    auto pivot_search = [&](int j, auto val, auto pos_of, unsigned* wpos_out) -> bool {
      unsigned best = 0u, bpos = 0xffffffffu;
      for (int i = lane; i < r; i += 32) {
        const float v = val(i);  // (evaluated for every row: val may store it)
        const unsigned ps = (unsigned)pos_of(i);
        if (ps < (unsigned)j) continue;
        const unsigned u = __float_as_uint(fabsf(v));
        if (u > best || (u == best && ps < bpos)) {
          best = u;
          bpos = ps;
        }
      }
      const unsigned wbest = __reduce_max_sync(0xffffffffu, best);
      *wpos_out = __reduce_min_sync(0xffffffffu, best == wbest ? bpos : 0xffffffffu);
      return wbest != 0u && wbest < 0x7f800000u;  // non-zero and finite
    };
    // the interchange of positions j and pos[pr] (thread 0)
    auto interchange = [&](int j, int pr) {
      const int q = row_at[j], pp = pos[pr];
      row_at[pp] = q;
      pos[q] = pp;
      row_at[j] = pr;
      pos[pr] = j;
    };
    // Steps in pairs (j, j + 1): step j's pivot from column j; column j + 1
    // as step j leaves it, b'(i) = X(i, j+1) - X(i, j) R1(j+1), formed by
    // every warp (warp 0 keeps it in colb2), gives step j + 1's pivot among
    // the positions step j's interchange leaves; both scaled pivot rows R1,
    // R2 are formed before one barrier, and one pass applies both steps to
    // every element.  Each element sees the same operations in the same
    // order as two single steps would apply, so the result is the same.
    float* colb2 = T;  // (T's bytes are free until U_f is written)
    float* rb1 = rowbuf[0];
    float* rb2 = rowbuf[1];
    int cur = 0;  // colbuf[cur] holds the current column j
    int j = 0;
    for (; j + 1 < r; j += 2) {
      const float* cb = colbuf[cur];
      float* cn = colbuf[cur ^ 1];  // column j + 2 after both steps
      unsigned wpos1 = 0, wpos2 = 0;
      const bool ok1 = pivot_search(j, [&](int i) { return cb[i]; },
                                    [&](int i) { return pos[i]; }, &wpos1);
      const int p1 = ok1 ? row_at[wpos1] : row_at[j];  // a singular block: any row, flagged
      const Real d1 = Mrr[p1 + ld * j];
      const Real inv1 = d1 != (Real)0 ? (Real)1 / d1 : (Real)0;
      const Real r1n = Mrr[p1 + ld * (j + 1)] * inv1;  // R1(j + 1)
      // positions after step j's interchange
      const int q1 = row_at[j], pp1 = pos[p1];
      const bool ok2 = pivot_search(
          j + 1,
          [&](int i) {
            const float bv = i == p1 ? r1n : Mrr[i + ld * (j + 1)] - cb[i] * r1n;
            if (warp == 0) colb2[i] = bv;
            return bv;
          },
          [&](int i) { return i == p1 ? j : (i == q1 ? pp1 : pos[i]); }, &wpos2);
      const int at_j1 = j + 1 == pp1 ? q1 : row_at[j + 1];
      const int p2 = ok2 ? ((int)wpos2 == pp1 ? q1 : row_at[wpos2]) : at_j1;
      const Real d2 = Mrr[p2 + ld * (j + 1)] - cb[p2] * r1n;
      const Real inv2 = d2 != (Real)0 ? (Real)1 / d2 : (Real)0;
      if (threadIdx.x == 0) {
        piv[j] = p1;
        piv[j + 1] = p2;
        if (!ok1 || !ok2) scal[0] = 1.0;
      }
      const Real ap2 = cb[p2];
      for (int c = threadIdx.x; c < r; c += blockDim.x) {
        const Real r1c = c == j ? inv1 : Mrr[p1 + ld * c] * inv1;
        const Real m2 = (c == j ? (Real)0 : Mrr[p2 + ld * c]) - ap2 * r1c;
        rb1[c] = r1c;
        rb2[c] = c == j + 1 ? inv2 : m2 * inv2;
      }
      __syncthreads();
      // (every warp has read pos for this pair by now)
      if (threadIdx.x == 0) {
        interchange(j, p1);
        interchange(j + 1, p2);
      }
      if (r > 0)
        for (TileWalk w(hr); w.j < hr; w.next()) {
          const int i0 = w.i, c0 = w.j;
          const bool ri = i0 + hr < r, rc = c0 + hr < r;
          const int i1 = ri ? i0 + hr : i0, c1 = rc ? c0 + hr : c0;
          const Real a0 = cb[i0], a1 = cb[i1], e0 = colb2[i0], e1 = colb2[i1];
          const Real f0 = rb1[c0], f1 = rb1[c1], g0 = rb2[c0], g1 = rb2[c1];
          Real m[4] = {Mrr[i0 + ld * c0], Mrr[i1 + ld * c0], Mrr[i0 + ld * c1],
                       Mrr[i1 + ld * c1]};
          const int ii[4] = {i0, i1, i0, i1}, cc[4] = {c0, c0, c1, c1};
          const Real aa[4] = {a0, a1, a0, a1}, ee[4] = {e0, e1, e0, e1};
          const Real ff[4] = {f0, f0, f1, f1}, gg[4] = {g0, g0, g1, g1};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            Real v = cc[q] == j ? (Real)0 : m[q];
            v = ii[q] == p1 ? ff[q] : v - aa[q] * ff[q];      // step j
            v = cc[q] == j + 1 ? (Real)0 : v;
            m[q] = ii[q] == p2 ? gg[q] : v - ee[q] * gg[q];  // step j + 1
          }
          Mrr[i0 + ld * c0] = m[0];
          if (ri) Mrr[i1 + ld * c0] = m[1];
          if (rc) Mrr[i0 + ld * c1] = m[2];
          if (ri && rc) Mrr[i1 + ld * c1] = m[3];
          if (c0 == j + 2) {
            cn[i0] = m[0];
            if (ri) cn[i1] = m[1];
          }
          if (rc && c1 == j + 2) {
            cn[i0] = m[2];
            if (ri) cn[i1] = m[3];
          }
        }
      __syncthreads();
      cur ^= 1;
    }
    if (j < r) {  // the last step of an odd r, alone
      const float* cb = colbuf[cur];
      unsigned wpos = 0;
      const bool ok = pivot_search(j, [&](int i) { return cb[i]; },
                                   [&](int i) { return pos[i]; }, &wpos);
      const int pr = ok ? row_at[wpos] : row_at[j];
      if (threadIdx.x == 0) {
        piv[j] = pr;
        if (!ok) scal[0] = 1.0;
      }
      const Real d = Mrr[pr + ld * j];
      const Real inv = d != (Real)0 ? (Real)1 / d : (Real)0;
      for (int c = threadIdx.x; c < r; c += blockDim.x)
        rb1[c] = c == j ? inv : Mrr[pr + ld * c] * inv;
      __syncthreads();
      if (threadIdx.x == 0) interchange(j, pr);
      if (r > 0)
        for (TileWalk w(hr); w.j < hr; w.next()) {
          const int i0 = w.i, c0 = w.j;
          const bool ri = i0 + hr < r, rc = c0 + hr < r;
          const int i1 = ri ? i0 + hr : i0, c1 = rc ? c0 + hr : c0;
          const Real a0 = cb[i0], a1 = cb[i1], b0 = rb1[c0], b1 = rb1[c1];
          Real m00 = Mrr[i0 + ld * c0], m10 = Mrr[i1 + ld * c0];
          Real m01 = Mrr[i0 + ld * c1], m11 = Mrr[i1 + ld * c1];
          if (c0 == j) m00 = m10 = (Real)0;
          if (c1 == j) m01 = m11 = (Real)0;
          m00 = i0 == pr ? b0 : m00 - a0 * b0;
          m10 = i1 == pr ? b0 : m10 - a1 * b0;
          m01 = i0 == pr ? b1 : m01 - a0 * b1;
          m11 = i1 == pr ? b1 : m11 - a1 * b1;
          Mrr[i0 + ld * c0] = m00;
          if (ri) Mrr[i1 + ld * c0] = m10;
          if (rc) Mrr[i0 + ld * c1] = m01;
          if (ri && rc) Mrr[i1 + ld * c1] = m11;
        }
      __syncthreads();
    }
    stamp(3);
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
    cta_gemm<false>(r, k, r, Mrr, (int)ld, Mrs, 1, (int)ld, (const Real*)nullptr, 0, Uo, r, Us, r);
    cta_gemm<false>(k, r, r, Msr, (int)ld, Mrr, 1, (int)ld, (const Real*)nullptr, 0, Lo, k);
    __syncthreads();  // U_f is read back below (same CTA)
    // E = Mss - K_sn_r U_f  (k x k)
    cta_gemm<true>(k, k, r, Msr, (int)ld, Us, 1, r, Mss, (int)ld, E_out, k);
    for (int j = threadIdx.x; j < r; j += blockDim.x) p.piv[t.piv_off + j] = j;
    if (threadIdx.x == 0 && scal[0] != 0.0) atomicExch(p.status, 1);
    stamp(4);
    report();
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
  stamp(3);
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
  stamp(4);
  report();
}

// threads: 256 or 128 per box, or 0: 128 when the launch holds more boxes
// than one wave of 256-thread CTAs (every resident slot of every SM), so the
// boxes run in one wave at twice the CTAs per SM, else 256.  (512 threads
// for launches of fewer boxes than SMs made their slowest box no faster: a
// Gauss-Jordan step is bound by its two barriers and the pivot search, not
// by the r^2 update.)  Every loop of the kernel strides by blockDim.x (or
// its warp count).
void launch_decouple(const DecoupleParams& p, int num_tasks, size_t smem, bool fp32,
                     cudaStream_t st, int threads, int num_sms) {
  if (num_tasks <= 0) return;
  if (fp32)
    set_smem_once<decouple_kernel<float>>();
  else
    set_smem_once<decouple_kernel<double>>();
  int nt = threads == 128 ? 128 : kThreads;
  if (threads == 0) {
    // 256-thread CTAs per SM for this shared-memory size, from a small
    // per-thread cache (the occupancy query is a driver call per launch)
    struct Occ {
      size_t smem;
      int fp32, per_sm;
    };
    static thread_local Occ cache[16];
    static thread_local int cached = 0;
    int per_sm = -1;
    for (int q = 0; q < cached; ++q)
      if (cache[q].smem == smem && cache[q].fp32 == (int)fp32) per_sm = cache[q].per_sm;
    if (per_sm < 0) {
      const void* fn =
          fp32 ? (const void*)decouple_kernel<float> : (const void*)decouple_kernel<double>;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, smem) != cudaSuccess)
        per_sm = 0;
      cache[cached % 16] = Occ{smem, (int)fp32, per_sm};
      cached = cached < 16 ? cached + 1 : 16;
    }
    if (per_sm > 0 && num_tasks > per_sm * num_sms) nt = 128;
  }
  if (fp32)
    decouple_kernel<float><<<num_tasks, nt, smem, st>>>(p);
  else
    decouple_kernel<double><<<num_tasks, nt, smem, st>>>(p);
}

}  // namespace rskel
