// Fast multipole evaluation of the boundary operators (Laplace double layer,
// Laplace-Neumann, Stokes double layer), used for the residual of the FP32
// factorization's iterative refinement.  The Laplace formulation follows;
// the Neumann and Stokes forms (further Cauchy sums) are in fmm.cu.
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
// overflows for small boxes.  Boxes holding no points are left out of every
// list: their expansions are zero and they have no targets.
//
// Three arithmetic variants share one plan: FP64; float-float ("double
// single": an unevaluated pair of floats carrying ~48 bits, run on the FP32
// pipes, which GB300 has ~58x more of than FP64) for the full FP64-accurate
// residual; and FP32 (order p32) for products with refinement corrections,
// whose size is already ~1e-6 of the solution's.  Every point is stored
// relative to the centre of its leaf (as FP64, and as a hi + lo float
// pair), and box-centre offsets are formed in FP64, so differences of nearby
// points keep their relative accuracy in every variant.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "devbuf.hpp"
#include "plan.hpp"
#include "tree.hpp"

namespace rskel {

enum FmmArith : int { kFmmF64 = 0, kFmmF32 = 1, kFmmDF = 2 };

struct FmmPlan {
  int p = 0;          // expansion order, FP64 and float-float variants
  int p32 = 0;        // expansion order, FP32 variant (fmm_set_order32)
  int p32_tab = 0;    // order binom32 was built for: the largest p32
  int nbox = 0;
  int npts = 0;
  int nlevels = 0;
  bool built = false;
  // per box (tree node id order)
  DevBuf<double> cx, cy, side;
  DevBuf<int> pstart, pcount;  // leaf point ranges in slot order (count 0: not a leaf)
  DevBuf<int> parent;
  DevBuf<int> children;        // 4 per box, -1 for leaves or empty children
  // slot order of points (leaf by leaf)
  DevBuf<int> slot_pt;         // slot -> point
  DevBuf<double> rx, ry;       // slot coordinates relative to the leaf centre
  DevBuf<float> rxh, rxl, ryh, ryl;  // the same as hi + lo float pairs
  // interaction lists (CSR over boxes)
  DevBuf<int> v_off, v_idx, w_off, w_idx, x_off, x_idx, u_off, u_idx;
  // non-empty boxes grouped by level (tree passes)
  std::vector<int> level_off;
  DevBuf<int> lvl_boxes;       // concatenated level lists
  std::vector<int> leaves_h;   // non-empty leaves
  DevBuf<int> leaves;
  std::vector<int> m2l_boxes_h;
  DevBuf<int> m2l_boxes;       // boxes with non-empty V or X lists
  DevBuf<double> binom;        // (2p) x (2p), binom[a * 2p + b] = C(a, b)
  DevBuf<float> binom_df;      // the same table as hi + lo pairs
  DevBuf<float> binom32;       // (2 p32) x (2 p32)
  size_t v_pairs = 0, u_pairs = 0, w_pairs = 0, x_pairs = 0;
  // work buffers (complex pairs of the variant's number type; sized for FP64)
  DevBuf<double> charge;       // 2 * (slot + npts * rhs)
  DevBuf<double> src;          // near-field source data, per slot (Laplace, Neumann)
  DevBuf<double> mpole, local; // 2 * (k + p * (rhs + nrhs * box))
  DevBuf<double> r1;           // per right-hand side: the rank-one sums (Neumann, Stokes)
  DevBuf<double> nearsum;      // the near field's sums per (slot, rhs), Laplace and Neumann
  HostBuf<unsigned char> stage;  // pinned staging of the plan's uploads
  // The near field (P2P) of a Laplace or Neumann product, and its M2P over
  // the W lists once the upward pass is done, run on a side stream of the
  // lowest priority, beside the tree passes (P2M, M2M, M2L, L2L) on the
  // caller's stream: those are chains of small launches whose latency leaves
  // most SMs idle.  Created on first use.
  struct SideStream {
    cudaStream_t st = nullptr;
    cudaEvent_t charges = nullptr, near = nullptr, mpole = nullptr;
    SideStream() = default;
    SideStream(const SideStream&) = delete;
    SideStream& operator=(const SideStream&) = delete;
    ~SideStream() {
      if (st) cudaStreamDestroy(st);
      if (charges) cudaEventDestroy(charges);
      if (near) cudaEventDestroy(near);
      if (mpole) cudaEventDestroy(mpole);
    }
  } nearq;
};

// The plan's host side: lists, slot order and leaf-relative coordinates,
// built from the tree without touching the GPU (so that it can run on a
// host thread while the factorization runs), then uploaded.
struct FmmHostPlan {
  bool ok = false;
  int p = 0, p32 = 0, nbox = 0, npts = 0, nlevels = 0;
  std::vector<double> cx, cy, side, rx, ry;
  std::vector<float> rxh, rxl, ryh, ryl, binom32;
  std::vector<int> pstart, pcount, parent, children, slot_pt, vo, vi, wo, wi, xo, xi, uo, ui,
      lvl_flat, level_off, leaves_h, m2l_boxes_h;
  size_t v_pairs = 0, u_pairs = 0, w_pairs = 0, x_pairs = 0;
};
bool fmm_plan_host(FmmHostPlan& h, const QuadTree& tree, const double* points, int npts, int p,
                   int p32);
bool fmm_plan_upload(FmmPlan& f, FmmHostPlan& h, cudaStream_t st);

// Builds the lists on the host from the tree (points interleaved, sd = 1).
// Orders 2..64 are supported for both variants.
bool fmm_build(FmmPlan& f, const QuadTree& tree, const double* points, int npts, int p, int p32,
               cudaStream_t st);

// y[:, q] = ya * y[:, q] + yb * (K mu)[:, q] for the operator of `pde`
// (Pde: Laplace double layer, Laplace-Neumann, Stokes double layer with its
// rank-one completion) as kernel_entry defines it; device pointers, column
// major D x nrhs (D = npts, or 2 npts interleaved for Stokes); y is not read
// when ya == 0.  Arithmetic `arith` (FmmArith); geo holds the per-point
// boundary data.
cudaError_t fmm_apply(FmmPlan& f, int pde, const Geo<double>& geo, const double* mu, int nrhs,
                      double* y, double ya, double yb, int arith, cudaStream_t st);
// Sets the order of the FP64 and float-float variants (2..64; the plan's
// lists do not depend on it).  Synchronous: call between products.
bool fmm_set_order(FmmPlan& f, int p, cudaStream_t st);
// Sets the order of the FP32 variant, 2 .. the order the plan was built
// with (its binomial table serves every lower order).  Takes effect with the
// next fmm_apply; nothing is synchronised.
bool fmm_set_order32(FmmPlan& f, int p);
// Kernels one fmm_apply launches.
int fmm_launches(const FmmPlan& f, int pde, int nrhs);

}  // namespace rskel
