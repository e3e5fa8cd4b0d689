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
// the rank is known.  The norm that decides the rank is accumulated in
// double for FP64 tiles and as a float pair (about 48 significant bits, on
// the FP32 pipes) for FP32 tiles.
#include <algorithm>
#include <cstdio>

#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.hpp"
#include "tcgen05.cuh"

namespace rskel {

constexpr int kChunk = 64;  // rows per fold

// Sums of squares for the FP32 paths' rank decisions, accumulated as an
// unevaluated float pair hi + lo (about 48 significant bits) on the FP32
// pipes: each square exactly by an FMA (p = a a, e = fma(a, a, -p)), each
// sum exactly by Knuth's two-sum.  The rank is then decided as by an FP64
// sum, without the FP64 pipe (about 1/60 of the FP32 rate on GB300), whose
// norm had been the longest link of a pivoted-QR step.  fp_add is
// commutative bit for bit (two-sum's error term is the exact rounding
// error, whatever the order), so a butterfly reduction leaves every lane
// the same pair.
struct FPair {
  float hi, lo;
};

__device__ __forceinline__ FPair fp_add(FPair a, FPair b) {
  const float s = a.hi + b.hi;
  const float bv = s - a.hi;
  const float e = (a.hi - (s - bv)) + (b.hi - bv);
  const float lo = e + (a.lo + b.lo);
  const float h = s + lo;
  return {h, lo - (h - s)};
}

__device__ __forceinline__ FPair fp_sq(float a) {
  const float p = a * a;
  return {p, fmaf(a, a, -p)};
}

__device__ __forceinline__ FPair fp_warp_sum(FPair v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = fp_add(v, FPair{__shfl_xor_sync(0xffffffffu, v.hi, o),
                        __shfl_xor_sync(0xffffffffu, v.lo, o)});
  return v;
}

// sqrt(hi + lo) to about 46 bits, as a normalised pair (hi is the float
// nearest the root): the FP32 root of hi and one Newton correction with the
// pair's residual.  Comparing two normalised pairs lexicographically
// compares their values.
__device__ __forceinline__ FPair fp_sqrt(FPair x) {
  if (!(x.hi > 0.f)) return FPair{0.f, 0.f};
  const float r0 = sqrtf(x.hi);
  const float c = (fmaf(-r0, r0, x.hi) + x.lo) / (2.f * r0);
  const float h = r0 + c;
  return FPair{h, c - (h - r0)};
}

// Thread layout inside a CTA: column c of a tile is owned by a team of TS
// consecutive threads (TS = 8, 4, 2, 1 for n <= 32, 64, 128, > 128); team
// thread t handles rows t, t + TS, ...  A Householder step then needs only
// team-local shuffles for every column's dot product and one CTA barrier
// (the reflector of step j+1 is formed by the team that just updated
// column j+1, and the reflector vector is double-buffered).
struct Layout {
  int t;       // this thread's index in its team
  int c0;      // first column owned
  int cstep;   // column stride between passes
  int ld;      // row-major leading dimension of tiles (padded)
};

// Team size for boxes of up to n DOFs.
__host__ __device__ inline int team_size(int n) { return n <= 64 ? 4 : (n <= 128 ? 2 : 1); }

// Row-major leading dimension: n padded so that ld = 32 / ts (mod 32), which
// makes a warp's (team, row) accesses hit distinct FP32 banks.
__host__ __device__ inline int layout_ld(int n, int ts) {
  const int want = (32 / ts) & 31;
  int ld = n;
  while ((ld & 31) != want) ++ld;
  return ld;
}

template <int TS>
__device__ __forceinline__ Layout make_layout(int n) {
  Layout L;
  L.t = threadIdx.x % TS;
  L.c0 = threadIdx.x / TS;
  L.cstep = blockDim.x / TS;
  L.ld = layout_ld(n, TS);
  return L;
}

// Lanes of this thread's team (teams are aligned groups of ts lanes).
__device__ __forceinline__ unsigned team_mask(int ts) {
  const int base = (threadIdx.x & 31) & ~(ts - 1);
  return ts >= 32 ? 0xffffffffu : (((1u << ts) - 1u) << base);
}

// Sum over the thread's team; teams may diverge from one another, so every
// shuffle names only the team's lanes.
template <int TS, class T>
__device__ __forceinline__ T team_sum(T v) {
  const unsigned m = team_mask(TS);
#pragma unroll
  for (int o = TS >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o);
  return v;
}

template <class Real>
struct IdShared {
  Real* R;        // n x n, row major, ld = L.ld
  Real* C;        // kChunk x n, row major, ld = L.ld
  Real* v;        // 2 x max(kChunk, n): double-buffered reflector
  double* vn1;    // n
  double* vn2;    // n
  int* perm;      // n
  double* scal;   // cpqr: [2] thresh (double)
  Real* rs;       // fold: [0..3] {tau, scale} x 2 buffers; cpqr: [0] tau
  int* is;        // cpqr: [0] stop flag, [1] pivot
  DofSoA<Real> act;
  DofSoA<Real> row;
  int* kind;      // kChunk
};

template <class Real>
__host__ __device__ size_t id_smem_bytes(int n, bool tile_in_smem) {
  size_t b = 0;
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const int ld = layout_ld(n, team_size(n));
  if (tile_in_smem) {
    b += al(sizeof(Real) * (size_t)n * ld);
    b += al(sizeof(Real) * (size_t)kChunk * ld);
  }
  b += al(sizeof(Real) * (3 * (size_t)(n > kChunk ? n : kChunk) + 3 * 32 * 32));
  b += 2 * al(sizeof(double) * n);
  b += al(sizeof(int) * n);
  b += al(sizeof(double) * 8) + al(sizeof(Real) * 8) + al(sizeof(int) * 8);
  b += dofs_bytes<Real>(n) + dofs_bytes<Real>(kChunk);
  b += al(sizeof(int) * kChunk);
  return b;
}

size_t id_direct_tile(int m, int n) {
  const size_t mp = (size_t)((m + kChunk - 1) / kChunk) * kChunk;
  return mp * (size_t)(n + 32) + mp + 64;  // tile + reflector
}

size_t id_kernel_smem(int n, bool fp32, bool tile_in_smem) {
  return fp32 ? id_smem_bytes<float>(n, tile_in_smem) : id_smem_bytes<double>(n, tile_in_smem);
}

template <class Real>
__device__ void stage_chunk_rows(const IdParams& p, const IdTask& t, IdShared<Real>& S, int c0,
                                 int cnt, double ox, double oy);

// Fills chunk rows [c0, c0 + cnt) of the virtual ID matrix into S.C (row major).
template <class Real>
__device__ void fill_chunk(const IdParams& p, const IdTask& t, IdShared<Real>& S, int ld, int c0,
                           int cnt, double ox, double oy) {
  const int n = t.n;
  if (t.dense_off >= 0) {
    const double* A = p.dense + t.dense_off;
    for (int e = threadIdx.x; e < kChunk * n; e += blockDim.x) {
      int i = e % kChunk, j = e / kChunk;
      S.C[(size_t)i * ld + j] = i < cnt ? (Real)A[(c0 + i) + (size_t)t.m_dense * j] : (Real)0;
    }
    __syncthreads();
    return;
  }
  stage_chunk_rows<Real>(p, t, S, c0, cnt, ox, oy);
  __syncthreads();
  for (TileWalk w(n); w.j < kChunk; w.next()) {  // row i = w.j, column j = w.i
    const int i = w.j, j = w.i;
    int kind = S.kind[i];
    Real val = (Real)0;
    if (kind == 0 || kind == 2) val = kernel_dofs<Real>(p.pde, S.row, i, S.act, j);
    else if (kind == 1 || kind == 3) val = kernel_dofs<Real>(p.pde, S.act, j, S.row, i);
    S.C[(size_t)i * ld + j] = val;
  }
  __syncthreads();
}

// Stages the "other" point of chunk rows [c0, c0 + cnt) of the virtual ID
// matrix (a row DOF, or a proxy point) and the row's kind in S.row / S.kind.
template <class Real>
__device__ void stage_chunk_rows(const IdParams& p, const IdTask& t, IdShared<Real>& S, int c0,
                                 int cnt, double ox, double oy) {
  const int q = t.q;
  const int sd = p.sd;
  const int prow = p.pde == kStokes ? 2 * p.npp : p.npp;  // rows per proxy block
  const double pw = 2.0 * CUDART_PI * t.pr / p.npp;
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
}

// Folds the chunk into R: Householder QR of [R; C] with R upper triangular.
// Reflector j has support {row j of R} u {all chunk rows}; its chunk part is
// column j of C itself (scaled), so nothing but two scalars is published per
// step.  The team that owns column j+1 accumulates that column's squared
// norm while applying reflector j, so forming reflector j+1 costs a few
// scalar operations between barriers.  Each team thread touches kChunk / TS
// rows (a compile-time count, fully unrolled).
template <class Real, int TS>
__device__ void fold_chunk(int n, const Layout& L, int step0, IdShared<Real>& S) {
  constexpr int kRows = kChunk / TS;
  Real* R = S.R;
  Real* C = S.C;
  Real* ssq = S.v;  // squared chunk-column norms, n entries
  const int t = L.t, ld = L.ld;
  const Real* Ct = C + (size_t)t * ld;  // this thread's first row
  const size_t rs = (size_t)TS * ld;    // stride between this thread's rows
  auto col_sq = [&](int c) {
    Real ss = 0;
#pragma unroll
    for (int q = 0; q < kRows; ++q) {
      const Real cv = Ct[q * rs + c];
      ss += cv * cv;
    }
    return team_sum<TS>(ss);
  };
  for (int c = L.c0; c < n; c += L.cstep) {
    const Real ss = col_sq(c);
    if (t == 0) ssq[c] = ss;
  }
  for (int j = 0; j < n; ++j) {
    const int buf = (step0 + j) & 1;
    Real* sc = S.rs + 2 * buf;  // {tau, scale}
    if (L.c0 == (j % L.cstep) && t == 0) {  // owner of column j forms reflector j
      const Real ss = ssq[j];
      const Real alpha = R[(size_t)j * ld + j];
      Real tau = 0, scale = 0;
      if (ss > (Real)0) {
        const Real beta = -copysign(sqrt(alpha * alpha + ss), alpha);
        tau = (beta - alpha) / beta;
        scale = (Real)1 / (alpha - beta);
        R[(size_t)j * ld + j] = beta;
      }
      sc[0] = tau;
      sc[1] = scale;
    }
    __syncthreads();
    const Real tau = sc[0];
    if (tau == (Real)0) {
      // identity reflector: column j+1 is unchanged, but its norm must be
      // current for the next step
      for (int c = L.c0; c < n; c += L.cstep)
        if (c == j + 1) {
          const Real ss = col_sq(c);
          if (t == 0) ssq[c] = ss;
        }
      continue;
    }
    const Real scale = sc[1];
    Real cj[kRows];
#pragma unroll
    for (int q = 0; q < kRows; ++q) cj[q] = Ct[q * rs + j];
    for (int c = L.c0; c < n; c += L.cstep) {
      if (c <= j) continue;
      Real* Cc = C + (size_t)t * ld + c;
      Real p4[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < kRows; ++q) p4[q & 3] += cj[q] * Cc[q * rs];
      Real part = team_sum<TS>((p4[0] + p4[1]) + (p4[2] + p4[3]));
      const Real tw = tau * (R[(size_t)j * ld + c] + part * scale);
      const Real tws = tw * scale;
      if (c == j + 1) {
        Real ss = 0;
#pragma unroll
        for (int q = 0; q < kRows; ++q) {
          const Real nv = Cc[q * rs] - tws * cj[q];
          Cc[q * rs] = nv;
          ss += nv * nv;
        }
        ss = team_sum<TS>(ss);
        if (t == 0) ssq[c] = ss;
      } else {
#pragma unroll
        for (int q = 0; q < kRows; ++q) Cc[q * rs] -= tws * cj[q];
      }
      if (t == 0) R[(size_t)j * ld + c] -= tw;
    }
  }
  __syncthreads();
}

// Column-pivoted Householder QR of the mr x n tile R (row major) with early
// stop at the rank (LAPACK dlaqp2 pivoting with its norm-downdating
// safeguard).  The partial norms that choose pivots are kept in the element
// type; the norm that sets the rank (the pivot column's trailing norm, which
// is |R_ii|) is accumulated in double.  Returns k.
template <class Real, int TS>
__device__ int cpqr_rank(int n, int mr, double tol, const Layout& L, IdShared<Real>& S,
                         long long* head_clk = nullptr) {
  Real* A = S.R;
  constexpr int ts = TS;
  const int t = L.t, ld = L.ld;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Real tol3z = sizeof(Real) == 4 ? (Real)2.44140625e-4 : (Real)1.0536712127723509e-08;
  Real* vn1 = reinterpret_cast<Real*>(S.vn1);
  Real* vn2 = reinterpret_cast<Real*>(S.vn2);
  for (int c = L.c0; c < n; c += L.cstep) {
    Real s = 0;
    for (int r = t; r < mr; r += ts) { const Real a = A[(size_t)r * ld + c]; s += a * a; }
    s = team_sum<TS>(s);
    if (t == 0) { vn1[c] = sqrt(s); vn2[c] = sqrt(s); S.perm[c] = c; }
  }
  __syncthreads();
  int k = 0;
  Real* v = S.v;
  const int kmax = n < mr ? n : mr;
  if constexpr (sizeof(Real) == 4) {
    // FP32 tiles.  Every column's norm below the current row is summed afresh
    // while its update is applied (one multiply-add per element), so a step's
    // head, which warp 0 runs while the other warps wait, only picks the
    // pivot, interchanges the columns and forms the reflector's scalars from
    // the pivot's norm and its diagonal entry: no reduction over the column
    // and no reflector vector.  The updates form v(r) = A(r, i) * scale
    // themselves, the same product the vector held.  A fresh FP32 sum of
    // squares is accurate to its own size, so |R_ii| near the rank threshold
    // is as good as the pivot column's own entries (the norm LAPACK's
    // sgeqp3 forms the same way).
    float th = 0.f;  // tol |R_00|
    for (int i = 0; i < kmax; ++i) {
      const long long t0 = head_clk != nullptr ? clock64() : 0;
      if (warp == 0) {
        unsigned bb = 0u;
        int li = n;
        for (int c = i + lane; c < n; c += 32) {
          const unsigned val = __float_as_uint(vn1[c]);
          if (li == n || val > bb) { bb = val; li = c; }
        }
        const unsigned wb = __reduce_max_sync(0xffffffffu, bb);
        const int bi =
            (int)__reduce_min_sync(0xffffffffu, li < n && bb == wb ? (unsigned)li : (unsigned)n);
        const float nrm = vn1[bi];  // |R_ii| (read before the interchange moves vn1[i])
        if (bi != i) {
          // eight rows per lane loaded before their stores (the tile may be
          // in global memory)
          for (int r0 = lane; r0 < mr; r0 += 256) {
            Real x[8], y[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int r = r0 + 32 * q;
              if (r < mr) {
                x[q] = A[(size_t)r * ld + bi];
                y[q] = A[(size_t)r * ld + i];
              }
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int r = r0 + 32 * q;
              if (r < mr) {
                A[(size_t)r * ld + bi] = y[q];
                A[(size_t)r * ld + i] = x[q];
              }
            }
          }
          if (lane == 0) {
            int tp = S.perm[bi]; S.perm[bi] = S.perm[i]; S.perm[i] = tp;
            vn1[bi] = vn1[i];
          }
        }
        __syncwarp();
        const float alpha = A[(size_t)i * ld + i];
        int stop = 0;
        if (i == 0) {
          const double td = fabs(tol * (double)nrm);
          th = (float)td;
          if (lane == 0) S.scal[2] = td;
        } else {
          stop = nrm < th ? 1 : 0;
        }
        const bool below = nrm > fabsf(alpha);  // some entry below the diagonal is non-zero
        float tau = 0.f, scale = 0.f, beta = 0.f;
        if (!stop && below) {
          beta = -copysignf(nrm, alpha);
          tau = (beta - alpha) / beta;
          scale = 1.f / (alpha - beta);
        }
        if (lane == 0) {
          if (!stop && below) A[(size_t)i * ld + i] = beta;
          S.rs[0] = tau;
          S.rs[1] = scale;
          S.is[0] = stop;
        }
      }
      __syncthreads();
      if (head_clk != nullptr) *head_clk += clock64() - t0;
      if (S.is[0] != 0) { k = i; break; }
      const float tau = S.rs[0], scale = S.rs[1];
      for (int c = L.c0; c < n; c += L.cstep) {
        if (c <= i) continue;
        float aic = A[(size_t)i * ld + c];
        float s2 = 0.f;
        const int r0 = i + 1 + t;
        if (tau != 0.f) {
          float part = 0.f;
          for (int r = r0; r < mr; r += ts) part += (A[(size_t)r * ld + i] * scale) * A[(size_t)r * ld + c];
          part = team_sum<TS>(part);
          const float tw = tau * (aic + part);
          // y(r) -= tw v(r), four rows loaded ahead of their stores, with
          // the new entries' squares summed
          int r = r0;
          for (; r + 3 * ts < mr; r += 4 * ts) {
            float y[4], x[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              y[q] = A[(size_t)(r + q * ts) * ld + c];
              x[q] = A[(size_t)(r + q * ts) * ld + i] * scale;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const float yn = y[q] - tw * x[q];
              A[(size_t)(r + q * ts) * ld + c] = yn;
              s2 += yn * yn;
            }
          }
          for (; r < mr; r += ts) {
            const float yn = A[(size_t)r * ld + c] - tw * (A[(size_t)r * ld + i] * scale);
            A[(size_t)r * ld + c] = yn;
            s2 += yn * yn;
          }
          aic -= tw;
        } else {
          for (int r = r0; r < mr; r += ts) {
            const float a = A[(size_t)r * ld + c];
            s2 += a * a;
          }
        }
        s2 = team_sum<TS>(s2);
        if (t == 0) {
          vn1[c] = sqrtf(s2);
          A[(size_t)i * ld + c] = aic;
        }
      }
      __syncthreads();
    }
    return k;
  } else {
  for (int i = 0; i < kmax; ++i) {
    const long long t0 = head_clk != nullptr ? clock64() : 0;
    // Warp 0 alone takes the pivot (first index of the largest partial
    // norm, idamax), interchanges the columns and forms the reflector of
    // column i; the other warps wait at the one barrier below.
    if (warp == 0) {
      int bi;  // the same in every lane
      if constexpr (sizeof(Real) == 4) {
        // partial norms are >= 0, so their bit patterns order as their
        // values: the largest by one warp reduction, then its first index
        unsigned bb = 0u;
        int li = n;
        for (int c = i + lane; c < n; c += 32) {
          const unsigned val = __float_as_uint(vn1[c]);
          if (li == n || val > bb) { bb = val; li = c; }
        }
        const unsigned wb = __reduce_max_sync(0xffffffffu, bb);
        bi = (int)__reduce_min_sync(0xffffffffu, li < n && bb == wb ? (unsigned)li : (unsigned)n);
      } else {
        Real best = -1;
        bi = n;
        for (int c = i + lane; c < n; c += 32) {
          const Real val = vn1[c];
          if (val > best) { best = val; bi = c; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const Real ov = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
      }
      if (bi != i) {
        // eight rows per lane loaded before their stores (the tile may be
        // in global memory)
        for (int r0 = lane; r0 < mr; r0 += 256) {
          Real x[8], y[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = r0 + 32 * q;
            if (r < mr) {
              x[q] = A[(size_t)r * ld + bi];
              y[q] = A[(size_t)r * ld + i];
            }
          }
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int r = r0 + 32 * q;
            if (r < mr) {
              A[(size_t)r * ld + bi] = y[q];
              A[(size_t)r * ld + i] = x[q];
            }
          }
        }
        if (lane == 0) {
          int tp = S.perm[bi]; S.perm[bi] = S.perm[i]; S.perm[i] = tp;
          vn1[bi] = vn1[i];
          vn2[bi] = vn2[i];
        }
      }
      __syncwarp();
      // The reflector: its norm |R_ii| sets the rank.  FP32 tiles sum it as
      // a float pair and compare it with the threshold as pairs (GB300's
      // FP64 pipe runs at about 1/60 of the FP32 rate; each FP64 warp
      // instruction in this chain costs tens of cycles); FP64 tiles in
      // double.
      const double alpha = (double)A[(size_t)i * ld + i];
      Real nrm;  // |R_ii| rounded to Real
      int stop = 0;
      bool below = false;  // some entry below the diagonal is non-zero
      if constexpr (sizeof(Real) == 4) {
        FPair xs{0.f, 0.f};
        for (int r = i + 1 + lane; r < mr; r += 32) xs = fp_add(xs, fp_sq(A[(size_t)r * ld + i]));
        xs = fp_warp_sum(xs);
        const FPair nv = fp_sqrt(fp_add(fp_sq((float)alpha), xs));
        below = xs.hi > 0.f;
        if (i == 0) {
          const double td = fabs(tol * ((double)nv.hi + (double)nv.lo));
          if (lane == 0) {
            S.scal[2] = td;
            S.rs[4] = (float)td;
            S.rs[5] = (float)(td - (double)(float)td);
          }
        } else {
          const float th = S.rs[4], tl = S.rs[5];
          stop = nv.hi < th || (nv.hi == th && nv.lo < tl) ? 1 : 0;
        }
        nrm = nv.hi;
      } else {
        double xs = 0.0;
        for (int r = i + 1 + lane; r < mr; r += 32) {
          const double a = (double)A[(size_t)r * ld + i];
          xs += a * a;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) xs += __shfl_xor_sync(0xffffffffu, xs, o);
        const double nd = sqrt(alpha * alpha + xs);
        below = xs > 0.0;
        if (i == 0) {
          if (lane == 0) S.scal[2] = fabs(tol * nd);
        } else if (nd < S.scal[2]) {
          stop = 1;
        }
        nrm = (Real)nd;
      }
      Real tau = 0, scale = 0, beta = 0;
      if (!stop && below) {
        const Real a = (Real)alpha;
        beta = -copysign(nrm, a);
        tau = (beta - a) / beta;
        scale = (Real)1 / (a - beta);
      }
      for (int r = i + 1 + lane; r < mr; r += 32) v[r] = A[(size_t)r * ld + i] * scale;
      __syncwarp();
      if (lane == 0) {
        if (!stop && below) A[(size_t)i * ld + i] = beta;
        S.rs[0] = tau;
        S.is[0] = stop;
      }
    }
    __syncthreads();
    if (head_clk != nullptr) *head_clk += clock64() - t0;
    if (S.is[0] != 0) { k = i; break; }
    const Real tau = S.rs[0];
    for (int c = L.c0; c < n; c += L.cstep) {
      if (c <= i) continue;
      Real aic = A[(size_t)i * ld + c];
      if (tau != (Real)0) {
        Real part = 0;
        for (int r = i + 1 + t; r < mr; r += ts) part += v[r] * A[(size_t)r * ld + c];
        part = team_sum<TS>(part);
        const Real tw = tau * (aic + part);
        const int r0 = i + 1 + t;
        if (r0 < mr)
          axpy_sub(A + (size_t)r0 * ld + c, ts * ld, v + r0, ts, tw, (mr - r0 + ts - 1) / ts);
        aic -= tw;
      }
      // partial norm downdate: vn1 <- sqrt(vn1^2 - a^2), recomputed when the
      // remaining fraction (vn1^2 - a^2) / vn2^2 drops below tol3z
      const Real v1 = vn1[c];
      if (v1 != (Real)0) {
        const Real v2 = vn2[c];
        Real x = v1 * v1 - aic * aic;
        x = x < (Real)0 ? (Real)0 : x;
        if (x <= tol3z * v2 * v2) {  // team-uniform decision
          Real s = 0;
          for (int r = i + 1 + t; r < mr; r += ts) { const Real a = A[(size_t)r * ld + c]; s += a * a; }
          s = team_sum<TS>(s);
          if (t == 0) { const Real q = sqrt(s); vn1[c] = q; vn2[c] = q; }
        } else if (t == 0) {
          vn1[c] = sqrt(x);
        }
      }
      __syncwarp(team_mask(ts));
      if (t == 0) A[(size_t)i * ld + c] = aic;
    }
    __syncthreads();
  }
  return k;
  }  // FP64 tiles
}

template <class Real, int TS>
__global__ void __launch_bounds__(kThreads) id_kernel(IdParams p) {
  const IdTask t = p.tasks[blockIdx.x];
  const int n = t.n;
  const Layout L = make_layout<TS>(n);
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sp = smem;
  IdShared<Real> S;
  if (p.direct) {
    S.R = nullptr;
    S.C = nullptr;
  } else if (t.scratch_off < 0) {
    S.R = carve<Real>(sp, n * L.ld);
    S.C = carve<Real>(sp, kChunk * L.ld);
  } else {
    Real* g = reinterpret_cast<Real*>(p.scratch) + t.scratch_off;
    S.R = g;
    S.C = g + (size_t)n * L.ld;
  }
  S.v = carve<Real>(sp, 3 * (n > kChunk ? n : kChunk) + 3 * 32 * 32);
  S.vn1 = carve<double>(sp, n);
  S.vn2 = carve<double>(sp, n);
  S.perm = carve<int>(sp, n);
  S.scal = carve<double>(sp, 8);
  S.rs = carve<Real>(sp, 8);
  S.is = carve<int>(sp, 8);
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
  if (!p.direct)
    for (int e = threadIdx.x; e < n * L.ld; e += blockDim.x) S.R[e] = (Real)0;
  __syncthreads();

  const int prow = p.pde == kStokes ? 2 * p.npp : p.npp;
  // direct == 2 (FP32 wide ID): a task with m_dense > 0 finds its m_dense-row
  // sketch already in its tile; the others factor their ID matrix directly
  const bool pre = p.direct == 2 && t.m_dense > 0;
  const int m = (t.dense_off >= 0 || pre) ? t.m_dense : 2 * t.q + (t.use_proxy ? 2 * prow : 0);
  int step0 = 0;
  long long clk_fill = 0, clk_fold = 0, clk0 = clock64();
  int k = 0;
  if (p.direct) {
    // Column-pivoted QR directly on the whole m x n ID matrix (held in the
    // task's global tile), stopping at the rank: dgeqp3 as the reference
    // calls it (ie_mat.cpp:556), minus the steps after the rank is known.
    Real* A = reinterpret_cast<Real*>(p.scratch) + t.scratch_off;
    Real* chunk_save = S.C;
    for (int c0 = 0; c0 < m && !pre; c0 += kChunk) {
      const int cnt = m - c0 < kChunk ? m - c0 : kChunk;
      S.C = A + (size_t)c0 * L.ld;
      fill_chunk<Real>(p, t, S, L.ld, c0, cnt, ox, oy);
    }
    S.C = chunk_save;
    S.R = A;
    S.v = A + (size_t)((m + kChunk - 1) / kChunk) * kChunk * L.ld;  // reflector (m entries)
    clk_fill = clock64() - clk0;
    clk0 = clock64();
    k = m > 0 ? cpqr_rank<Real, TS>(n, m, p.tol, L, S) : 0;
  } else {
    for (int c0 = 0; c0 < m; c0 += kChunk) {
      int cnt = m - c0 < kChunk ? m - c0 : kChunk;
      fill_chunk<Real>(p, t, S, L.ld, c0, cnt, ox, oy);
      const long long c1 = clock64();
      fold_chunk<Real, TS>(n, L, step0, S);
      const long long c2 = clock64();
      clk_fill += c1 - clk0;
      clk_fold += c2 - c1;
      clk0 = c2;
      step0 += n;
    }
    k = m > 0 ? cpqr_rank<Real, TS>(n, n, p.tol, L, S) : 0;
  }
  const long long clk_cpqr = clock64() - clk0;
  if (threadIdx.x == 0) p.ranks[t.slot] = k;
  for (int j = threadIdx.x; j < n; j += blockDim.x) p.perm[t.act_off + j] = S.perm[j];
  if (k > 0) {
    // Z = R11^{-1} R12 by back substitution, one team per column of R12.
    const int r = n - k;
    constexpr int ts = TS;
    const int tt = L.t, ld = L.ld;
    Real* T = reinterpret_cast<Real*>(p.fac) + t.fac_off + fac_T(k, r);
    for (int c = L.c0; c < r; c += L.cstep) {
      const int col = k + c;
      for (int row = k - 1; row >= 0; --row) {
        // owner thread of `row` finalises z[row]; the team then updates rows above
        Real zr = 0;
        if ((row % ts) == tt) {
          zr = S.R[(size_t)row * ld + col] * ((Real)1 / S.R[(size_t)row * ld + row]);
          S.R[(size_t)row * ld + col] = zr;
        }
        // broadcast within the team (the owner is lane (row % ts) of the team)
        const int base = (threadIdx.x & 31) - tt;
        zr = __shfl_sync(team_mask(ts), zr, base + (row % ts));
        if (tt < row)
          axpy_sub(S.R + (size_t)tt * ld + col, ts * ld, S.R + (size_t)tt * ld + row, ts * ld, zr,
                   (row - tt + ts - 1) / ts);
        __syncwarp(team_mask(ts));
      }
      for (int row = tt; row < k; row += ts) T[row + (size_t)k * c] = S.R[(size_t)row * ld + col];
    }
  }
  if (p.phase_clk != nullptr && threadIdx.x == 0) {
    long long* o = p.phase_clk + 4 * (size_t)t.slot;
    o[0] = clk_fill;
    o[1] = clk_fold;
    o[2] = clk_cpqr;
    o[3] = clock64() - clk0 - clk_cpqr;
  }
}

// ---------------------------------------------------------------------------
// FP32 randomized ID (the mixed-precision factorization's compression).
//
// The m x n ID matrix is sketched from the left, Y = Omega A with a dense
// +-1 matrix Omega of ell = n + kOversample rows (signs hashed from the
// sketch row and the global matrix row), accumulated chunk by chunk in
// register tiles: no serial chain, unlike the Householder fold.  Column-
// pivoted QR of the small ell x n sketch then picks the skeleton, the rank
// (first |R_ii| < tol |R_00|) and Z = R11^{-1} R12 -- the randomized
// interpolative decomposition (Martinsson, Rokhlin & Tygert 2011; Liberty et
// al. 2007).  Omega Q is a well-conditioned ell x n matrix for the n-column
// orthonormal factor Q of A, so the sketch's column norms track A's within a
// small factor: ranks may differ by one or two from a deterministic CPQR at
// the same tolerance and the interpolation error stays of order tol.  This
// path is only used by the FP32 factorization, whose accuracy is recovered
// by FP64 refinement; the FP64 path keeps the exact pivoted QR.
// ---------------------------------------------------------------------------
constexpr int kOversample = 16;
// 4x4 accumulator tiles per thread: 2 cover n <= 64 (team size 4), 5 cover n <= 128.
template <int TS>
constexpr int max_tiles() { return TS == 4 ? 2 : 5; }

// The sketch matrix Omega: entry (s, i) (sketch row s, ID-matrix row i) is
// +-1 from bit i % 8 of a 32-bit integer hash of (s, i / 8), so one hash
// gives a 16-byte row of eight BF16 signs for the tensor cores; the CUDA-core
// paths read the same entries one at a time.
__device__ __forceinline__ uint32_t sketch_bits8(int s, int grp) {
  unsigned x = (unsigned)s * 0x9E3779B1u ^ (unsigned)grp * 0x85EBCA77u ^ 0x6A09E667u;
  x ^= x >> 15;
  x *= 0x2C1B3C6Du;
  x ^= x >> 12;
  x *= 0x297A2D39u;
  x ^= x >> 15;
  return x >> 24;
}
__device__ __forceinline__ float sketch_sign(int s, int i) {
  return ((sketch_bits8(s, i >> 3) >> (i & 7)) & 1u) ? -1.0f : 1.0f;
}

__host__ __device__ inline int sketch_rows(int n) { return n + kOversample; }

// Sketch rows of a task: the predicted size when there is one (never above
// n + 16), the full n + 16 otherwise and in the redo pass.
__device__ __forceinline__ int task_ell(const IdParams& p, const IdTask& t) {
  const int full = sketch_rows(t.n);
  if (p.redo == nullptr || p.redo_pass || t.ell <= 0 || t.ell >= full) return full;
  return t.ell;
}

// A truncated sketch (mr = ell < m rows) settles the rank only when the rank
// rule stopped with at least `slack` rows to spare; otherwise (no stop
// within min(n, ell) pivots, or k > ell - slack) the box is redone.  Without
// the residual judge the slack is kMinSlack rows; with it, one row (the QR
// stopped before the rows ran out), since the judge's independent test rows
// then check the interpolation residual that a short sketch can
// underestimate.
constexpr int kMinSlack = 8;
__device__ __forceinline__ bool sketch_too_small(int k, int n, int m, int ell, int full,
                                                 bool judged) {
  if (ell >= full || m <= ell) return false;
  if (k == 0) return true;  // no stop: n <= ell would mean full rank, but ell < n + 16 here
  return k > ell - (judged ? 1 : kMinSlack);
}

// Test rows of the residual judge.  A learned pass's truncated sketch (fewer
// rows than the full n + 16, of a matrix taller than the sketch) is followed
// by kIdTestRows more rows of Omega (rows ell .. ell + 7, whose signs are
// independent of the sketch rows'), stored below the sketch.
__device__ __forceinline__ int task_test_rows(const IdParams& p, const IdTask& t, int ell, int m) {
  return (p.redo != nullptr && !p.redo_pass && p.judge_factor > 0.f && ell < sketch_rows(t.n) &&
          m > ell)
             ? kIdTestRows
             : 0;
}
__device__ __forceinline__ float sketch_or_test_sign(int r, int ell, int nt, int i) {
  return r < ell + nt ? sketch_sign(r, i) : 0.f;
}

// Residual estimate of an ID (k, perm, Z) from test rows Yt = Omega_t A
// (nt rows of a row-major tile at Yt, leading dimension ld, columns in A's
// order) and Z = R11^{-1} R12 (row i of Z at Z + i * ld, column c of Z at
// offset k + c).  For each redundant column c,
//   e = Yt(:, perm[k + c]) - Yt(:, perm[0..k)) Z(:, c) = Omega_t (A(:, perm[k+c]) - A(:, skel) Z(:, c)),
// and E ||Omega_t x||^2 = nt ||x||^2 for +-1 signs, so sqrt(|e|^2 / nt)
// estimates the interpolation residual of that column (Halko, Martinsson &
// Tropp 2011, sec. 4.3: a handful of random test vectors bound the residual
// with high probability).  Returns the squared estimate of the worst column
// this thread (cstep = the threads sharing the columns) covers.
__device__ __forceinline__ float judge_cols(const float* Yt, const float* Z, int ld, const int* perm,
                                            int k, int n, int nt, int c0, int cstep) {
  float mx = 0.f;
  for (int c = c0; c < n - k; c += cstep) {
    float ss = 0.f;
    for (int t = 0; t < nt; ++t) {
      const float* y = Yt + (size_t)t * ld;
      float e = y[perm[k + c]];
      for (int i = 0; i < k; ++i) e -= y[perm[i]] * Z[(size_t)i * ld + k + c];
      ss += e * e;
    }
    mx = fmaxf(mx, ss);
  }
  return mx;
}

// Redo flag of a judged box: 0 keeps it, 1 = the sketch did not settle the
// rank (sketch_too_small), 2 = the residual estimate is above the judge's
// bound.  `worst_sq` is the largest squared column estimate times nt.
__device__ __forceinline__ int judge_flag(const IdParams& p, float worst_sq, int nt, double thr_r00,
                                          int ell, int slot) {
  // thr_r00 = tol |R_00| of the ell-row sketch, and |R_00| estimates
  // sqrt(ell) ||a_max|| (the largest column of A), so the bound
  // judge_factor * tol * ||a_max|| is judge_factor * thr_r00 / sqrt(ell)
  const double est = sqrt((double)worst_sq / nt);
  const double unit = thr_r00 / sqrt((double)ell);
  if (p.judge_ratio != nullptr) p.judge_ratio[slot] = unit > 0 ? (float)(est / unit) : -1.f;
  return est > (double)p.judge_factor * unit ? 2 : 0;
}

// ---------------------------------------------------------------------------
// Tensor-core sketch (tcgen05).  Per 64-row chunk of the ID matrix, the
// sketch update Y += Omega_chunk A_chunk is one tcgen05.mma group: the MMA's
// M = sketch rows (sketch + test rows, padded to 128 per M tile), N = the
// box's columns padded to 16, K = the chunk's rows.  Omega is exact in BF16
// (+-1); the chunk of A is split in three BF16 parts, A = hi + mid + lo to
// about FP32 precision, and the three products accumulate in one FP32
// accumulator in tensor memory.  The CUDA cores form the kernel entries
// (the split and the signs are a few instructions more), write them straight
// into the operand tiles, and one thread issues the MMAs.
// ---------------------------------------------------------------------------
constexpr int kTcOmegaTile = 128 * kChunk * 2;   // bytes of one 128-row BF16 sign tile
constexpr uint32_t kTcPolls = 1u << 24;          // bound of every wait on the MMA barrier

__host__ __device__ inline int tc_npad(int n) { return (n + 15) & ~15; }
__host__ __device__ inline int tc_mtiles(int rows) { return (rows + 127) >> 7; }
// Operand tiles of a box of n columns with `rows` sketch rows: the sign tiles
// (first, so that any reading of them stays inside the region), then the
// three split tiles of the chunk.
__host__ __device__ inline size_t tc_tile_bytes(int n, int rows) {
  return (size_t)tc_mtiles(rows) * kTcOmegaTile + 3 * (size_t)tc_npad(n) * kChunk * 2;
}
__host__ __device__ inline uint32_t tc_tmem_cols(int cols) {
  uint32_t c = 32;
  while (c < (uint32_t)cols) c <<= 1;
  return c;
}

// v = hi + mid + lo with BF16 parts (each difference is exact in FP32).
__device__ __forceinline__ void split3(float v, uint16_t& h, uint16_t& m, uint16_t& l) {
  const __nv_bfloat16 bh = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(bh);
  const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(bm);
  h = __bfloat16_as_ushort(bh);
  m = __bfloat16_as_ushort(bm);
  l = __bfloat16_as_ushort(__float2bfloat16_rn(r2));
}

// Chunk rows [c0, c0 + cnt) (staged in S.row / S.kind) as the MMA operands:
// B = the chunk's entries, npad x kChunk K-major, in three split tiles at
// bt, bt + bbytes, bt + 2 bbytes; A = the signs of sketch rows [0, rows)
// (zero below), mtiles tiles of 128 x kChunk at om.  Each thread forms 8
// consecutive rows of one column (or 8 signs of one sketch row) and stores
// one 16-byte core-matrix row per tile; consecutive threads take
// consecutive columns (rows), so the stores are contiguous.
__device__ void fill_chunk_tc(const IdParams& p, const IdTask& t, const IdShared<float>& S, int c0,
                              int cnt, int npad, unsigned char* bt, uint32_t bbytes,
                              unsigned char* om, int rows, int mtiles) {
  const int n = t.n;
  const int items = npad * (kChunk / 8);
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int j = it % npad, g = it / npad;
    uint32_t w[3][4];
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
      uint16_t h[2], md[2], lo[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = 8 * g + q + u;
        float v = 0.f;
        if (j < n && i < cnt) {
          const int kind = S.kind[i];
          if (kind == 0 || kind == 2) v = kernel_dofs<float>(p.pde, S.row, i, S.act, j);
          else v = kernel_dofs<float>(p.pde, S.act, j, S.row, i);
        }
        split3(v, h[u], md[u], lo[u]);
      }
      w[0][q >> 1] = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
      w[1][q >> 1] = (uint32_t)md[0] | ((uint32_t)md[1] << 16);
      w[2][q >> 1] = (uint32_t)lo[0] | ((uint32_t)lo[1] << 16);
    }
    const uint32_t off = tc::tile_offset(j, 8 * g, npad);
#pragma unroll
    for (int x = 0; x < 3; ++x)
      *reinterpret_cast<uint4*>(bt + (size_t)x * bbytes + off) =
          make_uint4(w[x][0], w[x][1], w[x][2], w[x][3]);
  }
  const int orows = mtiles * 128;
  for (int it = threadIdx.x; it < orows * (kChunk / 8); it += blockDim.x) {
    const int sr = it % orows, g = it / orows;
    uint32_t w[4] = {0u, 0u, 0u, 0u};
    if (sr < rows) {
      const uint32_t b = sketch_bits8(sr, (c0 >> 3) + g);
#pragma unroll
      for (int q = 0; q < 8; ++q)  // BF16 +1 = 0x3F80, -1 = 0xBF80
        w[q >> 1] |= (uint32_t)(((b >> q) & 1u) ? 0xBF80u : 0x3F80u) << (16 * (q & 1));
    }
    *reinterpret_cast<uint4*>(om + (size_t)(sr >> 7) * kTcOmegaTile +
                              tc::tile_offset(sr & 127, 8 * g, 128)) =
        make_uint4(w[0], w[1], w[2], w[3]);
  }
}

size_t id_sketch_smem(int n, bool tc) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const int ld = layout_ld(n, team_size(n));
  const int ell = sketch_rows(n) + kIdTestRows;
  const int lp = (ell + 3) & ~3;
  size_t b = 0;
  b += al(sizeof(float) * (size_t)ell * ld);      // Y
  // C and the signs, or (tensor cores) the operand tiles in the same bytes
  const size_t cs = al(sizeof(float) * (size_t)kChunk * ld) + al(sizeof(float) * (size_t)kChunk * lp);
  b += tc ? std::max(cs, al(tc_tile_bytes(n, ell))) : cs;
  b += al(sizeof(float) * (3 * (size_t)(ell > kChunk ? ell : kChunk) + 3 * 32 * 32));
  b += 2 * al(sizeof(double) * n);
  b += al(sizeof(int) * n);
  b += al(sizeof(double) * 8) + al(sizeof(float) * 8) + al(sizeof(int) * 8);
  b += dofs_bytes<float>(n) + dofs_bytes<float>(kChunk);
  b += al(sizeof(int) * kChunk);
  return b;
}

// Leading dimension of a sketch held by one warp: n rounded up to 1 mod 32,
// so that a column walk (fixed column, rows across lanes) and a row walk
// (fixed row, columns across lanes) are both free of bank conflicts.
__host__ __device__ inline int warp_ld(int n) { return n + (33 - n % 32) % 32; }

size_t id_sketch_y_size(int n) { return (size_t)(sketch_rows(n) + kIdTestRows) * warp_ld(n); }

// Shared memory of the sketch-only variant (no Y tile, no QR workspace).
size_t id_sketch_split_smem(int n, bool tc) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const int ld = layout_ld(n, team_size(n));
  const int lp = (sketch_rows(n) + kIdTestRows + 3) & ~3;
  size_t b = 0;
  const size_t cs = al(sizeof(float) * (size_t)kChunk * ld) + al(sizeof(float) * (size_t)kChunk * lp);
  b += tc ? std::max(cs, al(tc_tile_bytes(n, sketch_rows(n) + kIdTestRows))) : cs;
  b += dofs_bytes<float>(n) + dofs_bytes<float>(kChunk);
  b += al(sizeof(int) * kChunk);
  return b;
}

// kSplit = false: sketch, pivoted QR and Z in one CTA per box.
// kSplit = true: the sketch only, written to p.sketch_y (row major, leading
// dimension warp_ld(n)) for id_cpqr_warp_kernel.
// kTC: the sketch on the tensor cores (tcgen05), the rest unchanged.
template <int TS, bool kSplit, bool kTC>
__global__ void __launch_bounds__(kThreads) id_sketch_kernel(IdParams p) {
  using Real = float;
  const IdTask t = p.tasks[blockIdx.x];
  if (p.redo_pass && p.redo[t.slot] == 0) return;  // block-uniform
  const int n = t.n;
  const Layout L = make_layout<TS>(n);
  const int ld = L.ld;
  const int ell = task_ell(p, t);
  const int prow = p.pde == kStokes ? 2 * p.npp : p.npp;
  const int m = 2 * t.q + (t.use_proxy ? 2 * prow : 0);
  const int nt = task_test_rows(p, t, ell, m);  // judge's test rows below the sketch
  const int lp = (ell + nt + 3) & ~3;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sp = smem;
  IdShared<Real> S;
  Real* sg;
  unsigned char* reg;  // S.C and the signs, or (kTC) the tensor cores' operand tiles
  // the operand tiles share the bytes of S.C and the signs (small matrices
  // use S.C, sketched ones the tiles)
  auto union_tiles = [&]() {
    if constexpr (kTC) {
      const size_t tb = (tc_tile_bytes(n, ell + nt) + 15) & ~size_t(15);
      if ((size_t)(sp - reg) < tb) sp = reg + tb;
    }
  };
  if constexpr (kSplit) {
    S.R = nullptr;
    reg = sp;
    S.C = carve<Real>(sp, kChunk * ld);
    sg = carve<Real>(sp, kChunk * lp);
    union_tiles();
  } else {
    S.R = carve<Real>(sp, (ell + nt) * ld);  // the sketch Y and test rows (or A itself when m <= ell)
    reg = sp;
    S.C = carve<Real>(sp, kChunk * ld);
    sg = carve<Real>(sp, kChunk * lp);
    union_tiles();
    S.v = carve<Real>(sp, 3 * (ell > kChunk ? ell : kChunk) + 3 * 32 * 32);
    S.vn1 = carve<double>(sp, n);
    S.vn2 = carve<double>(sp, n);
    S.perm = carve<int>(sp, n);
    S.scal = carve<double>(sp, 8);
    S.rs = carve<Real>(sp, 8);
    S.is = carve<int>(sp, 8);
  }
  S.act = carve_dofs<Real>(sp, n);
  S.row = carve_dofs<Real>(sp, kChunk);
  S.kind = carve<int>(sp, kChunk);
  const int wld = warp_ld(n);
  // (a row group's partial sketch: blockIdx.y of gridDim.y, stride 0 for one)
  Real* Yg = kSplit ? p.sketch_y + t.y_off + (int64_t)blockIdx.y * p.y_group_stride : nullptr;
  const int first = kSplit ? (int)blockIdx.y * kChunk : 0;   // this CTA's first chunk
  const int cstep = kSplit ? (int)gridDim.y * kChunk : kChunk;  // and its chunk stride

  const double ox = t.cx, oy = t.cy;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    load_dof<Real>(p.geo, p.sd, p.dofs[t.act_off + j], ox, oy, S.act, j);
  __syncthreads();
  long long clk0 = clock64(), clk_fill = 0, clk_fold = 0;
  int mr;
  if (!kSplit && p.y_parts > 0) {
    // the sketch (or the small matrix itself) is the sum of the row groups'
    // partial sketches, added in group order
    mr = m <= ell ? m : ell;
    const int rows = m <= ell ? m : ell + nt;
    const float* Y0 = p.sketch_y + t.y_off;
    const int total = rows * n, nth = blockDim.x;
    for (int e0 = threadIdx.x; e0 < total; e0 += 8 * nth) {
      // eight entries per thread, all their loads of a group in flight at once
      float acc[8];
      int src[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * nth;
        src[q] = e < total ? (e / n) * wld + e % n : -1;
        acc[q] = 0.f;
      }
      for (int g = 0; g < p.y_parts; ++g) {
        const float* Yp = Y0 + (int64_t)g * p.y_group_stride;
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = src[q] >= 0 ? Yp[src[q]] : 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] += v[q];
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * nth;
        if (e < total) S.R[(size_t)(e / n) * ld + e % n] = acc[q];
      }
    }
    __syncthreads();
    clk_fill = clock64() - clk0;
  } else if (kSplit && (m <= ell ? blockIdx.y > 0 : first >= m)) {
    // a row group with no rows: its partial sketch is zero (with m <= ell,
    // group 0 writes the whole matrix and the others zeros)
    mr = m <= ell ? m : ell;
    const int rows = m <= ell ? m : ell + nt;
    for (int e = threadIdx.x; e < rows * n; e += blockDim.x) Yg[(size_t)(e / n) * wld + e % n] = 0.f;
    return;
  } else if (m <= ell) {
    // small matrix: factor A itself
    mr = m;
    for (int c0 = 0; c0 < m; c0 += kChunk) {
      const int cnt = m - c0 < kChunk ? m - c0 : kChunk;
      fill_chunk<Real>(p, t, S, ld, c0, cnt, ox, oy);
      for (TileWalk w(n); w.j < cnt; w.next()) {
        const int i = w.j, j = w.i;
        if constexpr (kSplit) Yg[(size_t)(c0 + i) * wld + j] = S.C[(size_t)i * ld + j];
        else S.R[(size_t)(c0 + i) * ld + j] = S.C[(size_t)i * ld + j];
      }
      __syncthreads();
    }
    clk_fill = clock64() - clk0;
  } else if constexpr (kTC) {
    mr = ell;
    // Sketch on the tensor cores: per chunk, the CUDA cores write the
    // operand tiles, one thread issues 3 splits x 4 K steps of
    // tcgen05.mma per M tile and commits them to tc_bar; the tiles are
    // rewritten only after that barrier completes.  Every wait is bounded
    // and taken by thread 0 alone, which publishes the outcome in tc_ok, so
    // a give-up leaves the block uniformly (error flag, TMEM freed).
    __shared__ uint64_t tc_bar;
    __shared__ uint32_t tc_tmem;
    __shared__ int tc_ok;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = ell + nt;  // sketch rows, then the judge's test rows
    const int mtiles = tc_mtiles(rows);
    const int npad = tc_npad(n);
    unsigned char* om = reg;
    unsigned char* bt = reg + (size_t)mtiles * kTcOmegaTile;
    const uint32_t bbytes = (uint32_t)npad * kChunk * 2;
    const uint32_t ncols = tc_tmem_cols(mtiles * npad);
    if (warp == 0) {
      tc::tmem_alloc(&tc_tmem, ncols);
      tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
      tc::mbar_init(&tc_bar, 1);
      tc::fence_mbar_init();
      tc_ok = 1;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tc_tmem;
    const uint32_t idesc = tc::idesc_bf16_f32(128, npad);
    const uint32_t lbo_a = 128 * 16, lbo_b = (uint32_t)npad * 16;
    uint32_t phase = 0;
    for (int c0 = first; c0 < m; c0 += cstep) {
      const int cnt = m - c0 < kChunk ? m - c0 : kChunk;
      // the chunk's row points are staged while the previous chunk's MMAs
      // run (those read only the operand tiles); then the tiles are free
      // once the MMAs have completed.  The phase moves on only after a wait
      // that succeeded, so a give-up's last wait is on the MMAs in flight.
      stage_chunk_rows<Real>(p, t, S, c0, cnt, ox, oy);
      if (c0 > first && threadIdx.x == 0 && !tc::mbar_wait(&tc_bar, phase, kTcPolls)) tc_ok = 0;
      __syncthreads();
      if (!tc_ok) break;  // block-uniform
      if (c0 > first) phase ^= 1u;
      fill_chunk_tc(p, t, S, c0, cnt, npad, bt, bbytes, om, rows, mtiles);
      tc::fence_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) {
        tc::fence_after_sync();
        const uint32_t a0 = tc::smem_u32(om), b0 = tc::smem_u32(bt);
        for (int mt = 0; mt < mtiles; ++mt)
          for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int ks = 0; ks < kChunk / 16; ++ks) {
              const uint64_t ad =
                  tc::smem_desc(a0 + (uint32_t)mt * kTcOmegaTile + 2u * ks * lbo_a, lbo_a, 128);
              const uint64_t bd = tc::smem_desc(b0 + (uint32_t)x * bbytes + 2u * ks * lbo_b, lbo_b, 128);
              tc::mma_bf16(tmem + (uint32_t)(mt * npad), ad, bd, idesc,
                           (c0 > first || x > 0 || ks > 0) ? 1u : 0u);
            }
        tc::mma_commit(&tc_bar);
      }
    }
    if (tc_ok) {
      if (threadIdx.x == 0 && !tc::mbar_wait(&tc_bar, phase, kTcPolls)) tc_ok = 0;
      __syncthreads();
    }
    if (tc_ok) {
      // Y from tensor memory: warp w reads lanes 32 (w % 4) .. + 31 (sketch
      // rows), the column half w / 4, eight columns per load
      tc::fence_after_sync();
      const int qd = warp & 3, half = warp >> 2, hcols = npad >> 1;
      for (int mt = 0; mt < mtiles; ++mt) {
        const int sr = mt * 128 + 32 * qd + lane;
        for (int j0 = half * hcols; j0 < (half + 1) * hcols; j0 += 8) {
          float v[8];
          tc::tmem_ld8(tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(mt * npad + j0), v);
          if (sr < rows)
#pragma unroll
            for (int e = 0; e < 8; ++e)
              if (j0 + e < n) {
                if constexpr (kSplit) Yg[(size_t)sr * wld + j0 + e] = v[e];
                else S.R[(size_t)sr * ld + j0 + e] = v[e];
              }
        }
      }
    } else if (threadIdx.x == 0) {
      // gave up: one more bounded wait for the MMAs in flight, then report
      tc::mbar_wait(&tc_bar, phase, kTcPolls);
      if (p.status != nullptr) atomicExch(p.status, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
    if (!tc_ok) return;  // block-uniform
    clk_fill = clock64() - clk0;
    clk0 = clock64();
  } else {
    mr = ell;
    const int nrb = lp / 4, ncb = (n + 3) / 4, ntiles = nrb * ncb;
    constexpr int kMaxTiles = max_tiles<TS>();
    float acc[kMaxTiles][16];
#pragma unroll
    for (int q = 0; q < kMaxTiles; ++q)
#pragma unroll
      for (int e = 0; e < 16; ++e) acc[q][e] = 0.f;
    for (int c0 = first; c0 < m; c0 += cstep) {
      const int cnt = m - c0 < kChunk ? m - c0 : kChunk;
      fill_chunk<Real>(p, t, S, ld, c0, cnt, ox, oy);
      for (TileWalk w(lp); w.j < kChunk; w.next()) {
        const int ii = w.j, r = w.i;
        sg[w.e()] = ii < cnt ? sketch_or_test_sign(r, ell, nt, c0 + ii) : 0.f;
      }
      __syncthreads();
      const long long c1 = clock64();
#pragma unroll
      for (int q = 0; q < kMaxTiles; ++q) {
        const int tile = threadIdx.x + q * kThreads;
        if (tile >= ntiles) break;
        const int r0 = 4 * (tile / ncb), cc0 = 4 * (tile % ncb);
        float* a = acc[q];
#pragma unroll 4
        for (int ii = 0; ii < kChunk; ++ii) {
          const float4 cv = *reinterpret_cast<const float4*>(S.C + (size_t)ii * ld + cc0);
          const float4 sv = *reinterpret_cast<const float4*>(sg + (size_t)ii * lp + r0);
          a[0] += sv.x * cv.x;  a[1] += sv.x * cv.y;  a[2] += sv.x * cv.z;  a[3] += sv.x * cv.w;
          a[4] += sv.y * cv.x;  a[5] += sv.y * cv.y;  a[6] += sv.y * cv.z;  a[7] += sv.y * cv.w;
          a[8] += sv.z * cv.x;  a[9] += sv.z * cv.y;  a[10] += sv.z * cv.z; a[11] += sv.z * cv.w;
          a[12] += sv.w * cv.x; a[13] += sv.w * cv.y; a[14] += sv.w * cv.z; a[15] += sv.w * cv.w;
        }
      }
      __syncthreads();
      const long long c2 = clock64();
      clk_fill += c1 - clk0;
      clk_fold += c2 - c1;
      clk0 = c2;
    }
#pragma unroll
    for (int q = 0; q < kMaxTiles; ++q) {
      const int tile = threadIdx.x + q * kThreads;
      if (tile >= ntiles) break;
      const int r0 = 4 * (tile / ncb), cc0 = 4 * (tile % ncb);
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const int r = r0 + e / 4, c = cc0 + e % 4;
        if (r < ell + nt && c < n) {
          if constexpr (kSplit) Yg[(size_t)r * wld + c] = acc[q][e];
          else S.R[(size_t)r * ld + c] = acc[q][e];
        }
      }
    }
    __syncthreads();
  }
  if constexpr (kSplit) {
    (void)clk_fill;
    (void)clk_fold;
    return;
  }
  clk0 = clock64();
  // (trace: the steps' pivot and reflector time goes to the fold slot,
  // unused by the tensor-core sketch)
  const int k = mr > 0 ? cpqr_rank<Real, TS>(n, mr, p.tol, L, S,
                                             kTC && p.phase_clk != nullptr ? &clk_fold : nullptr)
                       : 0;
  const long long clk_cpqr = clock64() - clk0;
  const bool learned = p.redo != nullptr && !p.redo_pass;
  int flag = learned && sketch_too_small(k, n, m, ell, sketch_rows(n), nt > 0) ? 1 : 0;  // block-uniform
  const int r = n - k;
  if (flag == 0 && k > 0) {
    // Z = R11^{-1} R12 in place, one team per column of R12
    constexpr int ts = TS;
    const int tt = L.t;
    for (int c = L.c0; c < r; c += L.cstep) {
      const int col = k + c;
      for (int row = k - 1; row >= 0; --row) {
        Real zr = 0;
        if ((row % ts) == tt) {
          zr = S.R[(size_t)row * ld + col] * ((Real)1 / S.R[(size_t)row * ld + row]);
          S.R[(size_t)row * ld + col] = zr;
        }
        const int base = (threadIdx.x & 31) - tt;
        zr = __shfl_sync(team_mask(ts), zr, base + (row % ts));
        if (tt < row)
          axpy_sub(S.R + (size_t)tt * ld + col, ts * ld, S.R + (size_t)tt * ld + row, ts * ld, zr,
                   (row - tt + ts - 1) / ts);
        __syncwarp(team_mask(ts));
      }
    }
    __syncthreads();
    if (nt > 0) {
      // residual judge on the test rows (columns still in A's order: the
      // pivoted QR moved columns only within its mr rows)
      float w = judge_cols(S.R + (size_t)mr * ld, S.R, ld, S.perm, k, n, nt, threadIdx.x,
                           blockDim.x);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
      if ((threadIdx.x & 31) == 0) S.v[threadIdx.x >> 5] = w;
      __syncthreads();
      if (threadIdx.x == 0) {
        float mx = 0.f;
        for (int q = 0; q < kWarps; ++q) mx = fmaxf(mx, S.v[q]);
        S.is[2] = judge_flag(p, mx, nt, S.scal[2], ell, t.slot);
      }
      __syncthreads();
      flag = S.is[2];
    }
  }
  if (learned) {
    if (threadIdx.x == 0) p.redo[t.slot] = flag;
    if (flag) return;  // block-uniform
  }
  if (threadIdx.x == 0) p.ranks[t.slot] = k;
  for (int j = threadIdx.x; j < n; j += blockDim.x) p.perm[t.act_off + j] = S.perm[j];
  if (k > 0) {
    Real* T = reinterpret_cast<Real*>(p.fac) + t.fac_off + fac_T(k, r);
    for (int e = threadIdx.x; e < k * r; e += blockDim.x) {
      const int row = e % k, c = e / k;
      T[e] = S.R[(size_t)row * ld + k + c];
    }
  }
  if (p.phase_clk != nullptr && threadIdx.x == 0) {
    long long* o = p.phase_clk + 4 * (size_t)t.slot;
    o[0] = clk_fill;
    o[1] = clk_fold;
    o[2] = clk_cpqr;
    o[3] = clock64() - clk0 - clk_cpqr;
  }
}

// ---------------------------------------------------------------------------
// Second half of the split FP32 ID: one warp per box runs the column-pivoted
// QR of the box's sketch (rows mr = min(m, ell)) held in its own slice of
// shared memory, with no block-wide barrier: each lane owns the columns
// lane + 32 c (c < CPL) for the reflector updates and norm downdates, the
// pivot search and reflector norm are warp reductions.  Same rank rule,
// pivot order (first maximal partial norm) and norm downdating as
// cpqr_rank; then Z = R11^{-1} R12 by lane-local back substitution.
// ---------------------------------------------------------------------------
size_t id_cpqr_warp_bytes(int n) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  const int ell = sketch_rows(n);
  return al(sizeof(float) * (size_t)(ell + kIdTestRows) * warp_ld(n)) + al(sizeof(float) * ell) +
         2 * al(sizeof(float) * n) + al(sizeof(int) * n);
}

template <int CPL>
__global__ void __launch_bounds__(kThreads) id_cpqr_warp_kernel(IdParams p, int num_tasks,
                                                                 int wbytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ti = blockIdx.x * (blockDim.x >> 5) + warp;
  if (ti >= num_tasks) return;  // warp-uniform; nothing below synchronises the block
  const IdTask t = p.tasks[ti];
  if (p.redo_pass && p.redo[t.slot] == 0) return;  // warp-uniform
  const int n = t.n;
  const int ld = warp_ld(n);
  const int ell = task_ell(p, t);
  const int prow = p.pde == kStokes ? 2 * p.npp : p.npp;
  const int m = 2 * t.q + (t.use_proxy ? 2 * prow : 0);
  const int mr = m <= ell ? m : ell;
  const int nt = task_test_rows(p, t, ell, m);  // the judge's test rows follow the sketch
  unsigned char* sp = smem + (size_t)warp * wbytes;
  float* A = carve<float>(sp, (ell + nt) * ld);
  float* v = carve<float>(sp, ell);
  float* vn1 = carve<float>(sp, n);
  float* vn2 = carve<float>(sp, n);
  int* perm = carve<int>(sp, n);
  const float* Y = p.sketch_y + t.y_off;
  batched_copy(A, Y, (mr + nt) * ld, lane, 32);
  for (int j = lane; j < n; j += 32) perm[j] = j;
  __syncwarp();
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    const int j = lane + 32 * c;
    if (j < n) {
      float s = 0.f;
      for (int r = 0; r < mr; ++r) { const float a = A[(size_t)r * ld + j]; s += a * a; }
      vn1[j] = sqrtf(s);
      vn2[j] = vn1[j];
    }
  }
  __syncwarp();
  // Each column's norm below the current row is summed afresh while its
  // update is applied (one multiply-add per element, in its own lane), so the
  // reflector's norm |R_ii|, which sets the rank, is the pivot column's entry
  // of vn1: no reduction over the column.  A fresh FP32 sum of squares is
  // accurate to its own size (the norm LAPACK's sgeqp3 forms the same way).
  const int kmax = n < mr ? n : mr;
  int k = 0;
  double thr = 0.0;  // tol |R_00|
  float th = 0.f;
  for (int i = 0; i < kmax; ++i) {
    // pivot: first index of the largest norm (norms are >= 0, so their bit
    // patterns order as their values: two warp reductions)
    unsigned bb = 0u;
    int li = n;
    for (int j = i + lane; j < n; j += 32) {
      const unsigned val = __float_as_uint(vn1[j]);
      if (li == n || val > bb) { bb = val; li = j; }
    }
    const unsigned wb = __reduce_max_sync(0xffffffffu, bb);
    const int bi = (int)__reduce_min_sync(0xffffffffu, li < n && bb == wb ? (unsigned)li : (unsigned)n);
    const float nrm = vn1[bi];  // |R_ii| (read before the interchange moves vn1[i])
    __syncwarp();
    if (bi != i) {
      for (int r = lane; r < mr; r += 32) {
        const float a = A[(size_t)r * ld + bi];
        A[(size_t)r * ld + bi] = A[(size_t)r * ld + i];
        A[(size_t)r * ld + i] = a;
      }
      if (lane == 0) {
        const int tp = perm[bi];
        perm[bi] = perm[i];
        perm[i] = tp;
        vn1[bi] = vn1[i];
      }
      __syncwarp();
    }
    const float alpha = A[(size_t)i * ld + i];
    if (i == 0) {
      thr = fabs(p.tol * (double)nrm);
      th = (float)thr;
    } else if (nrm < th) {
      k = i;
      break;
    }
    const bool below = nrm > fabsf(alpha);  // some entry below the diagonal is non-zero
    float tau = 0.f, scale = 0.f, beta = 0.f;
    if (below) {
      beta = -copysignf(nrm, alpha);
      tau = (beta - alpha) / beta;
      scale = 1.f / (alpha - beta);
    }
    for (int r = i + 1 + lane; r < mr; r += 32) v[r] = A[(size_t)r * ld + i] * scale;
    __syncwarp();
    if (lane == 0 && below) A[(size_t)i * ld + i] = beta;
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int j = lane + 32 * c;
      if (j > i && j < n) {
        float aij = A[(size_t)i * ld + j];
        float s2 = 0.f;
        if (tau != 0.f) {
          float w0 = aij, w1 = 0.f, w2 = 0.f, w3 = 0.f;
          int r = i + 1;
          for (; r + 3 < mr; r += 4) {
            w0 += v[r] * A[(size_t)r * ld + j];
            w1 += v[r + 1] * A[(size_t)(r + 1) * ld + j];
            w2 += v[r + 2] * A[(size_t)(r + 2) * ld + j];
            w3 += v[r + 3] * A[(size_t)(r + 3) * ld + j];
          }
          for (; r < mr; ++r) w0 += v[r] * A[(size_t)r * ld + j];
          const float tw = tau * ((w0 + w1) + (w2 + w3));
          // y(q) -= tw v(q), four rows loaded ahead of their stores, with the
          // new entries' squares summed
          int q = i + 1;
          for (; q + 3 < mr; q += 4) {
            float y[4], x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              y[u] = A[(size_t)(q + u) * ld + j];
              x[u] = v[q + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float yn = y[u] - tw * x[u];
              A[(size_t)(q + u) * ld + j] = yn;
              s2 += yn * yn;
            }
          }
          for (; q < mr; ++q) {
            const float yn = A[(size_t)q * ld + j] - tw * v[q];
            A[(size_t)q * ld + j] = yn;
            s2 += yn * yn;
          }
          aij -= tw;
        } else {
          for (int q = i + 1; q < mr; ++q) { const float a = A[(size_t)q * ld + j]; s2 += a * a; }
        }
        vn1[j] = sqrtf(s2);
        A[(size_t)i * ld + j] = aij;
      }
    }
    __syncwarp();
  }
  const bool learned = p.redo != nullptr && !p.redo_pass;
  int flag = learned && sketch_too_small(k, n, m, ell, sketch_rows(n), nt > 0) ? 1 : 0;  // warp-uniform
  if (flag == 0 && k > 0) {
    // Z = R11^{-1} R12 in place, one lane per column of R12
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int col = lane + 32 * c;
      if (col >= k && col < n) {
        for (int row = k - 1; row >= 0; --row) {
          const float z = A[(size_t)row * ld + col] / A[(size_t)row * ld + row];
          A[(size_t)row * ld + col] = z;
          axpy_sub(A + col, ld, A + row, ld, z, row);
        }
      }
    }
    __syncwarp();
    if (nt > 0) {
      // residual judge on the test rows (columns in A's order: the pivoted
      // QR moved columns only within its mr rows)
      float w = judge_cols(A + (size_t)mr * ld, A, ld, perm, k, n, nt, lane, 32);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
      int f = 0;
      if (lane == 0) f = judge_flag(p, w, nt, thr, ell, t.slot);
      flag = __shfl_sync(0xffffffffu, f, 0);
    }
  }
  if (learned) {
    if (lane == 0) p.redo[t.slot] = flag;
    if (flag) return;  // warp-uniform
  }
  if (lane == 0) p.ranks[t.slot] = k;
  for (int j = lane; j < n; j += 32) p.perm[t.act_off + j] = perm[j];
  if (k > 0) {
    const int r = n - k;
    float* T = reinterpret_cast<float*>(p.fac) + t.fac_off + fac_T(k, r);
    for (int e = lane; e < k * r; e += 32) {
      const int row = e % k, c = e / k;
      T[e] = A[(size_t)row * ld + k + c];
    }
  }
}

template <class Real, int TS>
static void launch_id_t(const IdParams& p, int num_tasks, size_t smem, cudaStream_t st) {
  set_smem_once<id_kernel<Real, TS>>();
  id_kernel<Real, TS><<<num_tasks, kThreads, smem, st>>>(p);
}

template <int TS, bool kTC>
static void launch_sketch_tc(const IdParams& p, int num_tasks, size_t smem, cudaStream_t st) {
  set_smem_once<id_sketch_kernel<TS, false, kTC>>();
  id_sketch_kernel<TS, false, kTC><<<num_tasks, kThreads, smem, st>>>(p);
  if (p.redo != nullptr) {  // boxes whose predicted sketch was too small
    IdParams q = p;
    q.redo_pass = 1;
    id_sketch_kernel<TS, false, kTC><<<num_tasks, kThreads, smem, st>>>(q);
  }
}
template <int TS>
static void launch_sketch_t(const IdParams& p, int num_tasks, size_t smem, cudaStream_t st) {
  if (p.tc) launch_sketch_tc<TS, true>(p, num_tasks, smem, st);
  else launch_sketch_tc<TS, false>(p, num_tasks, smem, st);
}

// Split FP32 ID: the sketch (one CTA per box), then the warp-per-box QR.
template <int TS>
static void launch_split_pass(const IdParams& p, int num_tasks, int nmax, cudaStream_t st) {
  if (p.tc) {
    set_smem_once<id_sketch_kernel<TS, true, true>>();
    id_sketch_kernel<TS, true, true><<<num_tasks, kThreads, id_sketch_split_smem(nmax, true), st>>>(p);
  } else {
    set_smem_once<id_sketch_kernel<TS, true, false>>();
    id_sketch_kernel<TS, true, false>
        <<<num_tasks, kThreads, id_sketch_split_smem(nmax, false), st>>>(p);
  }
  const int wbytes = (int)id_cpqr_warp_bytes(nmax);
  int wpc = (int)((size_t)kSmemOptIn / wbytes);
  wpc = wpc < 1 ? 1 : wpc > kWarps ? kWarps : wpc;
  const int grid = (num_tasks + wpc - 1) / wpc;
  if (nmax <= 64) {
    set_smem_once<id_cpqr_warp_kernel<2>>();
    id_cpqr_warp_kernel<2><<<grid, 32 * wpc, (size_t)wbytes * wpc, st>>>(p, num_tasks, wbytes);
  } else {
    set_smem_once<id_cpqr_warp_kernel<4>>();
    id_cpqr_warp_kernel<4><<<grid, 32 * wpc, (size_t)wbytes * wpc, st>>>(p, num_tasks, wbytes);
  }
}

// A level of few boxes: the rows of each box over p.row_groups CTAs, each
// writing a partial sketch, then one CTA per box sums them and runs the
// pivoted QR, Z and the outputs.
template <int TS>
static void launch_grouped_t(const IdParams& p, int num_tasks, int nmax, cudaStream_t st) {
  const dim3 grid(num_tasks, p.row_groups);
  if (p.tc) {
    set_smem_once<id_sketch_kernel<TS, true, true>>();
    id_sketch_kernel<TS, true, true><<<grid, kThreads, id_sketch_split_smem(nmax, true), st>>>(p);
  } else {
    set_smem_once<id_sketch_kernel<TS, true, false>>();
    id_sketch_kernel<TS, true, false>
        <<<grid, kThreads, id_sketch_split_smem(nmax, false), st>>>(p);
  }
  IdParams q = p;
  q.y_parts = p.row_groups;
  launch_sketch_t<TS>(q, num_tasks, id_sketch_smem(nmax, p.tc != 0), st);
}

template <int TS>
static void launch_split_t(const IdParams& p, int num_tasks, int nmax, cudaStream_t st) {
  launch_split_pass<TS>(p, num_tasks, nmax, st);
  if (p.redo != nullptr) {  // boxes whose predicted sketch was too small
    IdParams q = p;
    q.redo_pass = 1;
    launch_split_pass<TS>(q, num_tasks, nmax, st);
  }
}

// ---------------------------------------------------------------------------
// FP32 wide ID: boxes of more than 128 columns (the top levels, whose ID
// matrices have thousands of rows).  One CTA per (task, block of kWideCols
// columns, range of rows) generates those rows of the ID matrix chunk by
// chunk and accumulates the partial sketch Omega(:, rows) A(rows, cols)
// (the same hashed signs as the other FP32 sketches); a second kernel sums
// the row ranges in a fixed order into the task's global tile; the direct
// pivoted QR (id_kernel, direct == 2) then runs on the ell x n sketch.
// ---------------------------------------------------------------------------
int id_sketch_rows(int n) { return sketch_rows(n); }
size_t id_wide_tile(int m, int n) { return id_direct_tile(m, n); }

constexpr int kWideMaxTiles = 5;  // 4x4 tiles per thread: <= 5 * 256 * 4 / kWideCols sketch rows
size_t id_wide_sketch_smem(int nmax) {
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  // the largest block any task of up to nmax columns uses (wide_sketch_block
  // is not monotonic: up to 640 rows whole, above that in blocks of <= 512)
  const int lp = std::min((sketch_rows(nmax) + 3) & ~3, 640);
  return al(sizeof(float) * kChunk * kWideCols) + al(sizeof(float) * (size_t)kChunk * lp) +
         dofs_bytes<float>(kWideCols) + dofs_bytes<float>(kChunk) + al(sizeof(int) * kChunk);
}

__global__ void __launch_bounds__(kThreads) id_wide_sketch_kernel(IdParams p,
                                                                  const WideItem* items,
                                                                  float* part) {
  const WideItem it = items[blockIdx.x];
  const IdTask t = p.tasks[it.task];
  const int n = t.n;
  const int nc = n - it.j0 < kWideCols ? n - it.j0 : kWideCols;
  const int sb = it.s1 - it.s0;  // this item's sketch rows, s0 + [0, sb)
  const int lp = (sb + 3) & ~3;
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* sp = smem;
  IdShared<float> S;
  S.C = carve<float>(sp, kChunk * kWideCols);
  float* sg = carve<float>(sp, kChunk * lp);
  S.act = carve_dofs<float>(sp, kWideCols);
  S.row = carve_dofs<float>(sp, kChunk);
  S.kind = carve<int>(sp, kChunk);
  const double ox = t.cx, oy = t.cy;
  for (int j = threadIdx.x; j < nc; j += blockDim.x)
    load_dof<float>(p.geo, p.sd, p.dofs[t.act_off + it.j0 + j], ox, oy, S.act, j);
  for (int e = threadIdx.x; e < kChunk * kWideCols; e += blockDim.x) S.C[e] = 0.f;
  __syncthreads();
  IdTask tc = t;  // the column block as a task of nc columns
  tc.n = nc;
  constexpr int ncb = kWideCols / 4;
  const int ntiles = (lp / 4) * ncb;
  float acc[kWideMaxTiles][16];
#pragma unroll
  for (int q = 0; q < kWideMaxTiles; ++q)
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[q][e] = 0.f;
  for (int c0 = it.r0; c0 < it.r1; c0 += kChunk) {
    const int cnt = it.r1 - c0 < kChunk ? it.r1 - c0 : kChunk;
    fill_chunk<float>(p, tc, S, kWideCols, c0, cnt, ox, oy);
    for (TileWalk w(lp); w.j < kChunk; w.next()) {
      const int ii = w.j, r = w.i;
      sg[w.e()] = (r < sb && ii < cnt) ? sketch_sign(it.s0 + r, c0 + ii) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kWideMaxTiles; ++q) {
      const int tile = threadIdx.x + q * kThreads;
      if (tile >= ntiles) break;
      const int r0 = 4 * (tile / ncb), cc0 = 4 * (tile % ncb);
      float* a = acc[q];
#pragma unroll 4
      for (int ii = 0; ii < kChunk; ++ii) {
        const float4 cv = *reinterpret_cast<const float4*>(S.C + (size_t)ii * kWideCols + cc0);
        const float4 sv = *reinterpret_cast<const float4*>(sg + (size_t)ii * lp + r0);
        a[0] += sv.x * cv.x;  a[1] += sv.x * cv.y;  a[2] += sv.x * cv.z;  a[3] += sv.x * cv.w;
        a[4] += sv.y * cv.x;  a[5] += sv.y * cv.y;  a[6] += sv.y * cv.z;  a[7] += sv.y * cv.w;
        a[8] += sv.z * cv.x;  a[9] += sv.z * cv.y;  a[10] += sv.z * cv.z; a[11] += sv.z * cv.w;
        a[12] += sv.w * cv.x; a[13] += sv.w * cv.y; a[14] += sv.w * cv.z; a[15] += sv.w * cv.w;
      }
    }
    __syncthreads();
  }
  float* out = part + it.part_off;
#pragma unroll
  for (int q = 0; q < kWideMaxTiles; ++q) {
    const int tile = threadIdx.x + q * kThreads;
    if (tile >= ntiles) break;
    const int r0 = 4 * (tile / ncb), cc0 = 4 * (tile % ncb);
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const int r = r0 + e / 4;
      if (r < sb) out[(size_t)(it.s0 + r) * kWideCols + cc0 + e % 4] = acc[q][e];
    }
  }
}

// Sum of a task's partial sketches over its row ranges, in order, into the
// row-major tile the direct pivoted QR reads (leading dimension as id_kernel
// lays it out for the task's n).
__global__ void __launch_bounds__(kThreads) id_wide_reduce_kernel(IdParams p, const float* part) {
  const IdTask t = p.tasks[blockIdx.x];
  if (t.m_dense <= 0) return;
  const int n = t.n, ell = t.m_dense, ns = t.wide_split;
  const int ld = layout_ld(n, team_size(n));
  float* A = reinterpret_cast<float*>(p.scratch) + t.scratch_off;
  const float* P = part + t.y_off;
  for (int e = threadIdx.x; e < ell * n; e += blockDim.x) {
    const int r = e / n, j = e % n, jb = j / kWideCols, jj = j % kWideCols;
    float s = 0.f;
    for (int q = 0; q < ns; ++q) s += P[((size_t)(jb * ns + q) * ell + r) * kWideCols + jj];
    A[(size_t)r * ld + j] = s;
  }
}

int launch_id_wide(const IdParams& p, int num_tasks, int nmax, const WideItem* items,
                   int num_items, float* part, cudaStream_t st) {
  if (num_tasks <= 0) return 0;
  int k = 0;
  if (num_items > 0) {
    set_smem_once<id_wide_sketch_kernel>();
    id_wide_sketch_kernel<<<num_items, kThreads, id_wide_sketch_smem(nmax), st>>>(p, items, part);
    id_wide_reduce_kernel<<<num_tasks, kThreads, 0, st>>>(p, part);
    k += 2;
  }
  IdParams q = p;
  q.direct = 2;
  launch_id_t<float, 1>(q, num_tasks, id_kernel_smem(nmax, true, false), st);
  return k + 1;
}

bool id_sketch_ok(int nmax) {
  return nmax <= 128 && id_sketch_smem(nmax, true) <= 227 * 1024 &&
         id_sketch_smem(nmax, false) <= 227 * 1024;
}


// All tasks of one launch use the team size of its largest box.  Returns
// the number of kernels launched.
int launch_id(const IdParams& p, int num_tasks, int nmax, size_t smem, bool fp32,
              cudaStream_t st) {
  if (num_tasks <= 0) return 0;
  const int passes = p.redo != nullptr ? 2 : 1;
  const int ts = team_size(nmax);
  // A level of few boxes: each box's rows over p.row_groups CTAs (partial
  // sketches), then the CTA-per-box QR on their sum.
  if (fp32 && p.dense == nullptr && id_sketch_ok(nmax) && p.sketch_y != nullptr &&
      p.row_groups > 1 && p.redo == nullptr) {
    if (ts == 4) launch_grouped_t<4>(p, num_tasks, nmax, st);
    else launch_grouped_t<2>(p, num_tasks, nmax, st);
    return 2;
  }
  // The warp-per-box QR pays off when a level has boxes enough to fill the
  // GPU; small levels keep the lower-latency CTA-per-box QR.
  if (fp32 && p.dense == nullptr && id_sketch_ok(nmax) && p.sketch_y != nullptr &&
      num_tasks >= (p.split_min_tasks > 0 ? p.split_min_tasks : 512)) {
    if (ts == 4) launch_split_t<4>(p, num_tasks, nmax, st);
    else launch_split_t<2>(p, num_tasks, nmax, st);
    return 2 * passes;
  }
  if (fp32 && p.dense == nullptr && id_sketch_ok(nmax)) {
    const size_t sm = id_sketch_smem(nmax, p.tc != 0);
    if (ts == 4) launch_sketch_t<4>(p, num_tasks, sm, st);
    else launch_sketch_t<2>(p, num_tasks, sm, st);
    return passes;
  }
  if (fp32) {
    if (ts == 4) launch_id_t<float, 4>(p, num_tasks, smem, st);
    else if (ts == 2) launch_id_t<float, 2>(p, num_tasks, smem, st);
    else launch_id_t<float, 1>(p, num_tasks, smem, st);
  } else {
    if (ts == 4) launch_id_t<double, 4>(p, num_tasks, smem, st);
    else if (ts == 2) launch_id_t<double, 2>(p, num_tasks, smem, st);
    else launch_id_t<double, 1>(p, num_tasks, smem, st);
  }
  return 1;
}

// Sets the dynamic shared-memory limit of the three FP64 ID kernel variants
// on the current device (the set-up step of rs_id_noalloc).
cudaError_t id_noalloc_prepare() {
  cudaError_t e = cudaFuncSetAttribute(id_kernel<double, 4>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemOptIn);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(id_kernel<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kSmemOptIn);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(id_kernel<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kSmemOptIn);
  return e;
}

}  // namespace rskel
