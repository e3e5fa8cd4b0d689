// Fast multipole evaluation of the Laplace double-layer operator in FP64,
// used for the residual of the FP32 factorization's iterative refinement.
//
// In complex notation (z = x + iy, nu = n_x + i n_y) the double-layer kernel
// of ie_solver/kernel/kernel.cpp:123-165 is
//     K_ij = -(w_j / 2pi) Re( nu_j / (z_i - z_j) )   (i != j),
// so (K mu)_i = diag_i mu_i + Re sum_{j != i} c_j / (z_i - z_j) with complex
// charges c_j = -(w_j / 2pi) nu_j mu_j: a Cauchy sum, evaluated by the
// classical 2D fast multipole method (Greengard & Rokhlin 1987) with the
// adaptive U/V/W/X lists of Carrier, Greengard & Rokhlin (1988) built on the
// solver's own quadtree.  Expansions are scaled by box size (multipole
// coefficients by s^-k, local coefficients by s^l) so that no power
// overflows for small boxes.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "devbuf.hpp"
#include "plan.hpp"
#include "tree.hpp"

namespace rskel {

struct FmmPlan {
  int p = 0;          // expansion order
  int nbox = 0;
  int npts = 0;
  int nlevels = 0;
  bool built = false;
  // per box (tree node id order)
  DevBuf<double> cx, cy, side;
  DevBuf<int> pstart, pcount;  // leaf point ranges in slot order (count 0: not a leaf)
  DevBuf<int> parent;
  DevBuf<int> children;        // 4 per box, -1 for leaves
  int max_leaf_pts = 0;
  // slot order of points (leaf by leaf)
  DevBuf<int> slot_pt;         // slot -> point
  DevBuf<double> zx, zy;       // slot coordinates
  // interaction lists (CSR over boxes)
  DevBuf<int> v_off, v_idx, w_off, w_idx, x_off, x_idx, u_off, u_idx;
  // boxes grouped by level for the tree passes (deepest first in host order)
  std::vector<std::vector<int>> level_boxes;
  std::vector<int> level_off;
  DevBuf<int> lvl_boxes;       // concatenated level lists
  std::vector<int> leaves_h;
  DevBuf<int> leaves;
  std::vector<int> m2l_boxes_h;
  DevBuf<int> m2l_boxes;       // boxes with non-empty V or X lists
  DevBuf<double> binom;        // (2p) x (2p), binom[a * 2p + b] = C(a, b)
  // work buffers
  DevBuf<double> charge;       // complex charges, slot-major: 2 * (slot + npts * rhs)
  DevBuf<double> mpole, local; // complex: 2 * (k + p * (rhs + nrhs * box))
  int cap_rhs = 0;
};

// Builds the lists on the host from the tree (points interleaved, sd = 1).
// Expansion orders 2..64 are supported.
bool fmm_build(FmmPlan& f, const QuadTree& tree, const double* points, int npts, int p,
               cudaStream_t st);

// y[:, q] = K mu[:, q] for the Laplace double layer (device pointers, column
// major npts x nrhs); geo holds the per-point boundary data.
cudaError_t fmm_laplace_apply(FmmPlan& f, const Geo<double>& geo, const double* mu, int nrhs,
                              double* y, cudaStream_t st);

}  // namespace rskel
