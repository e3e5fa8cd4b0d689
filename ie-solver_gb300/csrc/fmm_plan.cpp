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
#include <cstring>
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

// Plan arrays go to the device through the plan's pinned staging buffer
// (asynchronous copies on the plan's stream; the build synchronises once
// at its end, before the buffer can be written again).
struct Uploader {
  FmmPlan& f;
  cudaStream_t st;
  size_t used = 0;
  cudaError_t err = cudaSuccess;
  template <class T>
  bool operator()(DevBuf<T>& d, const std::vector<T>& h) {
    if (err != cudaSuccess) return false;
    if ((err = d.ensure(std::max<size_t>(h.size(), 1))) != cudaSuccess) return false;
    if (h.empty()) return true;
    const size_t bytes = h.size() * sizeof(T), off = (used + 255) & ~size_t(255);
    if (off + bytes > f.stage.cap) {  // full: wait for the copies in flight, start over
      if ((err = cudaStreamSynchronize(st)) != cudaSuccess) return false;
      if ((err = f.stage.ensure(std::max<size_t>(2 * f.stage.cap, bytes + 4096))) != cudaSuccess)
        return false;
      used = 0;
      return (*this)(d, h);
    }
    std::memcpy(f.stage.p + off, h.data(), bytes);
    used = off + bytes;
    err = cudaMemcpyAsync(d.p, f.stage.p + off, bytes, cudaMemcpyHostToDevice, st);
    return err == cudaSuccess;
  }
};

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

bool fmm_set_order32(FmmPlan& f, int p) {
  if (p < 2 || p > f.p32_tab) return false;
  f.p32 = p;
  return true;
}

bool fmm_set_order(FmmPlan& f, int p, cudaStream_t st) {
  if (p < 2 || p > 64) return false;
  std::vector<double> binom;
  pascal(2 * p, &binom);
  std::vector<float> binom_df(2 * binom.size());
  for (size_t i = 0; i < binom.size(); ++i) {
    binom_df[2 * i] = (float)binom[i];
    binom_df[2 * i + 1] = (float)(binom[i] - (double)binom_df[2 * i]);
  }
  Uploader up{f, st};
  if (!up(f.binom, binom) || !up(f.binom_df, binom_df)) return false;
  if (cudaStreamSynchronize(st) != cudaSuccess) return false;
  f.p = p;
  return true;
}

bool fmm_plan_host(FmmHostPlan& f, const QuadTree& tree, const double* points, int npts, int p,
                   int p32) {
  f.ok = false;
  if (p < 2 || p > 64 || p32 < 2 || p32 > 64 || npts <= 0) return false;
  const int nb = (int)tree.nodes.size();
  f.p = p;
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
  f.binom32.assign(b32d.begin(), b32d.end());
  f.cx.swap(cx);
  f.cy.swap(cy);
  f.side.swap(side);
  f.pstart.swap(pstart);
  f.pcount.swap(pcount);
  f.parent.swap(parent);
  f.children.swap(children);
  f.slot_pt.swap(slot_pt);
  f.rx.swap(rx);
  f.ry.swap(ry);
  f.rxh.swap(rxh);
  f.rxl.swap(rxl);
  f.ryh.swap(ryh);
  f.ryl.swap(ryl);
  f.vo.swap(vo);
  f.vi.swap(vi);
  f.wo.swap(wo);
  f.wi.swap(wi);
  f.xo.swap(xo);
  f.xi.swap(xi);
  f.uo.swap(uo);
  f.ui.swap(ui);
  f.lvl_flat.swap(lvl_flat);
  f.ok = true;
  return true;
}

bool fmm_plan_upload(FmmPlan& f, FmmHostPlan& h, cudaStream_t st) {
  f.built = false;
  if (!h.ok) return false;
  f.p32 = h.p32;
  f.p32_tab = h.p32;
  f.nbox = h.nbox;
  f.npts = h.npts;
  f.nlevels = h.nlevels;
  f.level_off = h.level_off;
  f.leaves_h = h.leaves_h;
  f.m2l_boxes_h = h.m2l_boxes_h;
  f.v_pairs = h.v_pairs;
  f.w_pairs = h.w_pairs;
  f.x_pairs = h.x_pairs;
  f.u_pairs = h.u_pairs;
  Uploader up{f, st};
  bool ok = up(f.cx, h.cx) && up(f.cy, h.cy) && up(f.side, h.side) && up(f.pstart, h.pstart) &&
            up(f.pcount, h.pcount) && up(f.parent, h.parent) && up(f.children, h.children) &&
            up(f.slot_pt, h.slot_pt) && up(f.rx, h.rx) && up(f.ry, h.ry) && up(f.rxh, h.rxh) &&
            up(f.rxl, h.rxl) && up(f.ryh, h.ryh) && up(f.ryl, h.ryl) && up(f.v_off, h.vo) &&
            up(f.v_idx, h.vi) && up(f.w_off, h.wo) && up(f.w_idx, h.wi) && up(f.x_off, h.xo) &&
            up(f.x_idx, h.xi) && up(f.u_off, h.uo) && up(f.u_idx, h.ui) &&
            up(f.lvl_boxes, h.lvl_flat) && up(f.leaves, h.leaves_h) &&
            up(f.m2l_boxes, h.m2l_boxes_h) && up(f.binom32, h.binom32) &&
            cudaStreamSynchronize(st) == cudaSuccess && fmm_set_order(f, h.p, st);
  f.built = ok;
  return ok;
}

bool fmm_build(FmmPlan& f, const QuadTree& tree, const double* points, int npts, int p, int p32,
               cudaStream_t st) {
  FmmHostPlan h;
  return fmm_plan_host(h, tree, points, npts, p, p32) && fmm_plan_upload(f, h, st);
}

}  // namespace rskel
