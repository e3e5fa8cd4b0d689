// Plan records shared by the host planner (solver.cpp) and the device kernels.
// All offsets index device pools owned by the solver handle.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define RS_HD
#else
#define RS_HD __host__ __device__
#endif

namespace rskel {

enum Pde : int { kLaplace = 0, kLaplaceNeumann = 1, kStokes = 2 };

// Boundary data in structure-of-arrays form, indexed by point.
template <class Real>
struct Geo {
  const Real* x;
  const Real* y;
  const Real* nx;
  const Real* ny;
  const Real* w;
  const Real* kap;
};

// One interpolative decomposition (kernel/kernel.cpp:293-423 + ie_mat.cpp:548-588).
struct IdTask {
  int n;            // active DOFs (columns)
  int act_off;      // active DOF indices at dofs[act_off .. act_off+n)
  int q;            // row-source DOFs ("inner" or "outside" lists)
  int rows_off;     // row-source DOF indices at dofs[rows_off .. rows_off+q)
  int use_proxy;    // levels >= 3: proxy-circle rows follow
  int slot;         // output slot: ranks[slot]
  double cx, cy;    // box centre (proxy circle centre)
  double pr;        // proxy radius
  int64_t fac_off;  // T (k x r) written at fac[fac_off]
  int64_t scratch_off;  // >= 0: global-memory tile for boxes too large for shared memory
  int64_t dense_off;    // >= 0: rows come from a given dense matrix (rs_id_batched)
  int m_dense;          // rows of that matrix
  int ell;              // FP32 split ID: sketch rows from the rank predictor (0: n + 16)
  int64_t y_off;        // FP32 split ID: the sketch (rows x warp leading dimension) at sketch_y[y_off]
                        // FP32 wide ID: first partial sketch of the task in the partial buffer
  int wide_split;       // FP32 wide ID: row ranges the partial sketches are split into
  int pad2;
};

// FP32 wide ID (boxes of more than 128 columns): one CTA per (task, block
// of kWideCols columns, row range), each writing a partial sketch
// (ell x kWideCols, row major) at part[part_off].
constexpr int kWideCols = 32;
struct WideItem {
  int task;     // index in the launch's task array
  int j0;       // first column
  int r0, r1;   // ID matrix rows [r0, r1)
  int s0, s1;   // sketch rows [s0, s1)
  int64_t part_off;
};
// Sketch rows one wide item forms: all of them up to 640 (the register
// tiles' limit), else blocks of at most 512.
inline int wide_sketch_block(int ell) {
  if (ell <= 640) return ell;
  const int nb = (ell + 511) / 512;
  return (((ell + nb - 1) / nb) + 3) & ~3;
}

// One elimination (skel_factorization.cpp:77-128) or, for boxes that are not
// compressed, the assembly of the box's Schur-complemented block.
// Where entry (a, b) of a box's matrix comes from.  The box's active DOFs
// are its children's surviving DOFs, child by child (child c's run starts at
// active position cstart[c]; a leaf is one run with no block).  When DOFs a
// and b fall in the same run and that child has a Schur-complemented block
// (ce[c] >= 0), the entry is E[ce[c] + i_a + cld[c] i_b] with i the
// positions within the run; otherwise it comes from the kernel.
struct DecoupleTask {
  int n;            // active DOFs
  int act_off;      // active DOFs at dofs[act_off..)
  int slot;         // ranks[slot] (k; 0 means "assemble only")
  int perm_off;     // permutation at perm[perm_off..) (n entries)
  int64_t fac_off;  // T, L, U, X_rr LU at fac[fac_off..)
  int64_t piv_off;  // X_rr pivots at piv[piv_off..)
  int64_t e_off;    // output block E (k x k, or n x n when not compressed)
  int64_t scratch_off;  // >= 0: global-memory tile for large boxes
  int cstart[4];    // first active position of each child's run (runs in child order)
  int cld[4];       // leading dimension of each child's block
  int64_t ce[4];    // offset of each child's block in the E pool, -1 = kernel
};

// One node of a solve sweep (skel_factorization.cpp:388-426, 507-592).
struct SweepTask {
  int k, r;
  int skel_off;     // skeleton DOFs at dofs[skel_off..)
  int red_off;      // redundant DOFs at dofs[red_off..)
  int64_t fac_off;  // T, L, U, X_rr LU at fac[fac_off..)
  int64_t piv_off;
};

// Factor block layout at fac_off for a node with k skeleton and r redundant DOFs.
RS_HD inline int64_t fac_T(int, int) { return 0; }
RS_HD inline int64_t fac_L(int k, int r) { return (int64_t)k * r; }
RS_HD inline int64_t fac_U(int k, int r) { return 2 * (int64_t)k * r; }
RS_HD inline int64_t fac_X(int k, int r) { return 3 * (int64_t)k * r; }
// Doubles reserved per node with n active DOFs (any split k + r = n).
// max over k of 3k(n-k) + (n-k)^2 is 9n^2/8 (at k = n/4).
RS_HD inline int64_t fac_reserve(int n) { return (5 * (int64_t)n * n) / 4 + 8; }

}  // namespace rskel
