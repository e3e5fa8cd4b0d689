// Host construction of the FMM interaction lists on the solver's quadtree.
//
// Lists (Carrier, Greengard & Rokhlin 1988), with adjacency meaning the
// closed squares touch:
//   colleagues(B): same-level boxes adjacent to B (B included), the children
//                  of the colleagues of B's parent that touch B;
//   V(B): the other children of those colleagues (same level, separated);
//   for a leaf B, descending into each non-leaf colleague: a child that
//   touches B is descended into (or, if a leaf, joins U(B), and B joins its
//   U list); a child that does not touch B joins W(B) and B joins its X list.
//   Leaf colleagues (and B itself) join U(B).
// Boxes with no points are skipped throughout.
// The quadtree's own neighbour lists follow the reference's construction,
// including its `y < top && y < bottom` condition (quadtree.cpp:209), so the
// FMM recomputes adjacency from the box geometry instead.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fmm.hpp"

namespace rskel {

namespace {

struct Box {
  double x0, y0, s;
};

bool touch(const Box& a, const Box& b, double eps) {
  return a.x0 <= b.x0 + b.s + eps && b.x0 <= a.x0 + a.s + eps && a.y0 <= b.y0 + b.s + eps &&
         b.y0 <= a.y0 + a.s + eps;
}

template <class T>
cudaError_t upload(DevBuf<T>& d, const std::vector<T>& h) {
  cudaError_t e = d.ensure(std::max<size_t>(h.size(), 1));
  if (e != cudaSuccess) return e;
  if (h.empty()) return cudaSuccess;
  return cudaMemcpy(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void csr(const std::vector<std::vector<int>>& lists, std::vector<int>* off, std::vector<int>* idx) {
  off->assign(lists.size() + 1, 0);
  idx->clear();
  for (size_t i = 0; i < lists.size(); ++i) {
    idx->insert(idx->end(), lists[i].begin(), lists[i].end());
    (*off)[i + 1] = (int)idx->size();
  }
}

// Pascal triangle, P2 x P2: t[a * P2 + b] = C(a, b)
void pascal(int P2, std::vector<double>* t) {
  t->assign((size_t)P2 * P2, 0.0);
  for (int a = 0; a < P2; ++a) {
    (*t)[(size_t)a * P2] = 1.0;
    for (int b = 1; b <= a; ++b)
      (*t)[(size_t)a * P2 + b] =
          (*t)[(size_t)(a - 1) * P2 + b - 1] + (b < a ? (*t)[(size_t)(a - 1) * P2 + b] : 0.0);
  }
}

}  // namespace

bool fmm_set_order(FmmPlan& f, int p) {
  if (p < 2 || p > 64) return false;
  std::vector<double> binom;
  pascal(2 * p, &binom);
  std::vector<float> binom_df(2 * binom.size());
  for (size_t i = 0; i < binom.size(); ++i) {
    binom_df[2 * i] = (float)binom[i];
    binom_df[2 * i + 1] = (float)(binom[i] - (double)binom_df[2 * i]);
  }
  if (upload(f.binom, binom) != cudaSuccess || upload(f.binom_df, binom_df) != cudaSuccess)
    return false;
  f.p = p;
  return true;
}

bool fmm_build(FmmPlan& f, const QuadTree& tree, const double* points, int npts, int p, int p32,
               cudaStream_t st) {
  (void)st;
  if (p < 2 || p > 64 || p32 < 2 || p32 > 64 || npts <= 0) return false;
  const int nb = (int)tree.nodes.size();
  f.p32 = p32;
  f.nbox = nb;
  f.npts = npts;
  std::vector<Box> box(nb);
  for (int i = 0; i < nb; ++i)
    box[i] = Box{tree.nodes[i].corners[0], tree.nodes[i].corners[1], tree.nodes[i].side};
  // points per subtree; empty boxes take part in nothing
  std::vector<int> cnt(nb, 0);
  for (int lv = (int)tree.levels.size() - 1; lv >= 0; --lv)
    for (int b : tree.levels[lv]) {
      const TreeNode& nd = tree.nodes[b];
      if (nd.is_leaf) cnt[b] = (int)nd.original.size() / tree.sd;
      else
        for (int q = 0; q < 4; ++q) cnt[b] += cnt[nd.children[q]];
    }
  auto live = [&](int b) { return cnt[b] > 0; };
  // (a forest has one root per tree; lists never cross trees)
  double root_side = 0;
  for (int r : tree.roots) root_side = std::max(root_side, tree.nodes[r].side);
  const double eps = 1e-9 * root_side;
  std::vector<std::vector<int>> coll(nb), V(nb), W(nb), X(nb), U(nb);
  for (int r : tree.roots)
    if (live(r)) coll[r].push_back(r);
  for (size_t lv = 1; lv < tree.levels.size(); ++lv) {
    for (int b : tree.levels[lv]) {
      if (!live(b)) continue;
      const int par = tree.nodes[b].parent;
      for (int c : coll[par]) {
        if (tree.nodes[c].is_leaf) continue;
        for (int q = 0; q < 4; ++q) {
          const int d = tree.nodes[c].children[q];
          if (!live(d)) continue;
          if (touch(box[d], box[b], eps)) coll[b].push_back(d);
          else V[b].push_back(d);
        }
      }
    }
  }
  // U, W, X for leaves
  std::vector<int> stack;
  for (int b = 0; b < nb; ++b) {
    if (!tree.nodes[b].is_leaf || !live(b)) continue;
    for (int c : coll[b]) {
      if (tree.nodes[c].is_leaf) {
        U[b].push_back(c);
        continue;
      }
      stack.assign(1, c);
      while (!stack.empty()) {
        const int node = stack.back();
        stack.pop_back();
        for (int q = 0; q < 4; ++q) {
          const int d = tree.nodes[node].children[q];
          if (!live(d)) continue;
          if (touch(box[d], box[b], eps)) {
            if (tree.nodes[d].is_leaf) {
              U[b].push_back(d);
              U[d].push_back(b);
            } else {
              stack.push_back(d);
            }
          } else {
            W[b].push_back(d);
            X[d].push_back(b);
          }
        }
      }
    }
  }
  // slot order: leaves in level order, each leaf's points in its DOF order
  std::vector<int> pstart(nb, 0), pcount(nb, 0), slot_pt;
  slot_pt.reserve(npts);
  f.leaves_h.clear();
  for (int id : tree.level_order) {
    if (!tree.nodes[id].is_leaf) continue;
    pstart[id] = (int)slot_pt.size();
    for (size_t q = 0; q < tree.nodes[id].original.size(); q += tree.sd)
      slot_pt.push_back(tree.nodes[id].original[q] / tree.sd);
    pcount[id] = (int)slot_pt.size() - pstart[id];
    if (pcount[id] > 0) f.leaves_h.push_back(id);
  }
  if ((int)slot_pt.size() != npts) return false;
  auto split = [](double v, float* hi, float* lo) {
    *hi = (float)v;
    *lo = (float)(v - (double)*hi);
  };
  std::vector<double> cx(nb), cy(nb), side(nb);
  std::vector<int> parent(nb), children(4 * (size_t)nb, -1);
  for (int i = 0; i < nb; ++i) {
    if (!tree.nodes[i].is_leaf)
      for (int q = 0; q < 4; ++q) {
        const int c = tree.nodes[i].children[q];
        children[4 * (size_t)i + q] = live(c) ? c : -1;
      }
    cx[i] = box[i].x0 + box[i].s / 2.0;
    cy[i] = box[i].y0 + box[i].s / 2.0;
    side[i] = box[i].s;
    parent[i] = tree.nodes[i].parent;
  }
  // coordinates relative to the leaf centre
  std::vector<double> rx(npts), ry(npts);
  std::vector<float> rxh(npts), rxl(npts), ryh(npts), ryl(npts);
  for (int leaf : f.leaves_h)
    for (int s2 = pstart[leaf]; s2 < pstart[leaf] + pcount[leaf]; ++s2) {
      rx[s2] = points[2 * slot_pt[s2]] - cx[leaf];
      ry[s2] = points[2 * slot_pt[s2] + 1] - cy[leaf];
      split(rx[s2], &rxh[s2], &rxl[s2]);
      split(ry[s2], &ryh[s2], &ryl[s2]);
    }
  // non-empty boxes by level
  f.nlevels = (int)tree.levels.size();
  std::vector<int> lvl_flat;
  f.level_off.assign(f.nlevels + 1, 0);
  for (int lv = 0; lv < f.nlevels; ++lv) {
    for (int b : tree.levels[lv])
      if (live(b)) lvl_flat.push_back(b);
    f.level_off[lv + 1] = (int)lvl_flat.size();
  }
  f.m2l_boxes_h.clear();
  for (int b = 0; b < nb; ++b)
    if (!V[b].empty() || !X[b].empty()) f.m2l_boxes_h.push_back(b);
  std::vector<int> vo, vi, wo, wi, xo, xi, uo, ui;
  csr(V, &vo, &vi);
  csr(W, &wo, &wi);
  csr(X, &xo, &xi);
  csr(U, &uo, &ui);
  f.v_pairs = vi.size();
  f.w_pairs = wi.size();
  f.x_pairs = xi.size();
  f.u_pairs = ui.size();
  std::vector<double> b32d;
  pascal(2 * p32, &b32d);
  std::vector<float> binom32(b32d.begin(), b32d.end());
  bool ok = fmm_set_order(f, p) && upload(f.cx, cx) == cudaSuccess && upload(f.cy, cy) == cudaSuccess &&
            upload(f.side, side) == cudaSuccess && upload(f.pstart, pstart) == cudaSuccess &&
            upload(f.pcount, pcount) == cudaSuccess && upload(f.parent, parent) == cudaSuccess &&
            upload(f.children, children) == cudaSuccess &&
            upload(f.slot_pt, slot_pt) == cudaSuccess && upload(f.rx, rx) == cudaSuccess &&
            upload(f.ry, ry) == cudaSuccess && upload(f.rxh, rxh) == cudaSuccess &&
            upload(f.rxl, rxl) == cudaSuccess && upload(f.ryh, ryh) == cudaSuccess &&
            upload(f.ryl, ryl) == cudaSuccess && upload(f.v_off, vo) == cudaSuccess &&
            upload(f.v_idx, vi) == cudaSuccess && upload(f.w_off, wo) == cudaSuccess &&
            upload(f.w_idx, wi) == cudaSuccess && upload(f.x_off, xo) == cudaSuccess &&
            upload(f.x_idx, xi) == cudaSuccess && upload(f.u_off, uo) == cudaSuccess &&
            upload(f.u_idx, ui) == cudaSuccess && upload(f.lvl_boxes, lvl_flat) == cudaSuccess &&
            upload(f.leaves, f.leaves_h) == cudaSuccess &&
            upload(f.m2l_boxes, f.m2l_boxes_h) == cudaSuccess &&
            upload(f.binom32, binom32) == cudaSuccess;
  f.built = ok;
  return ok;
}

}  // namespace rskel
