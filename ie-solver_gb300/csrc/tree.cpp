// Host quadtree construction; see tree.hpp for the rules it reproduces.
#include "tree.hpp"

#include <omp.h>

#include <algorithm>
#include <cmath>

namespace rskel {

int QuadTree::new_node() {
  nodes.emplace_back();
  return static_cast<int>(nodes.size()) - 1;
}

void QuadTree::push_level(int level, int id) {
  if (static_cast<int>(levels.size()) <= level) levels.resize(level + 1);
  levels[level].push_back(id);
}

// A box's own DOF list (the reference's original_box, which it appends to
// every box on a point's path, quadtree.cpp:230-269) is the ordered union of
// its leaves' lists, since every list is in point order: only leaves keep one.
std::vector<int> QuadTree::box_dofs(int id) const {
  if (nodes[id].is_leaf) return nodes[id].original;
  std::vector<int> out, stack(1, id);
  while (!stack.empty()) {
    const int b = stack.back();
    stack.pop_back();
    if (nodes[b].is_leaf) {
      out.insert(out.end(), nodes[b].original.begin(), nodes[b].original.end());
    } else {
      for (int c = 0; c < 4; ++c)
        if (nodes[b].children[c] >= 0) stack.push_back(nodes[b].children[c]);
    }
  }
  std::sort(out.begin(), out.end());
  return out;
}

// quadtree.cpp:275-432
void QuadTree::subdivide(int id) {
  nodes[id].is_leaf = 0;
  double c[8];
  for (int i = 0; i < 8; ++i) c[i] = nodes[id].corners[i];
  const double midx = ((c[6] - c[0]) / 2.0) + c[0];
  const double midy = ((c[3] - c[1]) / 2.0) + c[1];
  const int bl = new_node(), tl = new_node(), tr = new_node(), br = new_node();
  const double cb[8] = {c[0], c[1], c[2], midy, midx, midy, midx, c[7]};
  const double ct[8] = {c[0], midy, c[2], c[3], midx, c[5], midx, midy};
  const double cr[8] = {midx, midy, midx, c[3], c[4], c[5], c[6], midy};
  const double cq[8] = {midx, c[1], midx, midy, c[4], midy, c[6], c[7]};
  for (int i = 0; i < 8; ++i) {
    nodes[bl].corners[i] = cb[i];
    nodes[tl].corners[i] = ct[i];
    nodes[tr].corners[i] = cr[i];
    nodes[br].corners[i] = cq[i];
  }
  const int kids[4] = {bl, tl, tr, br};
  for (int k : kids) {
    nodes[k].level = nodes[id].level + 1;
    nodes[k].side = nodes[id].side / 2.0;
    nodes[k].parent = id;
  }
  const int lv = nodes[id].level + 1;
  push_level(lv, bl);
  push_level(lv, br);
  push_level(lv, tr);
  push_level(lv, tl);
  TreeNode& nd = nodes[id];
  nd.bl = bl; nd.tl = tl; nd.tr = tr; nd.br = br;
  nd.children[0] = bl; nd.children[1] = tl; nd.children[2] = tr; nd.children[3] = br;
  std::vector<int> parent_dofs;
  parent_dofs.swap(nd.original);  // a box above the leaves keeps no list (box_dofs)
  for (size_t idx = 0; idx < parent_dofs.size(); idx += sd) {
    const int mi = parent_dofs[idx];
    const int pv = (mi / sd) * 2;
    const double x = pts_[pv], y = pts_[pv + 1];
    int dst;
    if (x < midx && y < midy) dst = bl;
    else if (x < midx && y >= midy) dst = tl;
    else if (x >= midx && y < midy) dst = br;
    else dst = tr;
    for (int q = 0; q < sd; ++q) nodes[dst].original.push_back(mi + q);
  }
  if (static_cast<int>(nodes[bl].original.size()) > leaf_) subdivide(bl);
  if (static_cast<int>(nodes[tl].original.size()) > leaf_) subdivide(tl);
  if (static_cast<int>(nodes[tr].original.size()) > leaf_) subdivide(tr);
  if (static_cast<int>(nodes[br].original.size()) > leaf_) subdivide(br);
}

// quadtree.cpp:185-227: the boxes below `small` whose corners touch the
// leaf `big`, in the reference's walk order, appended to *out.  The
// reference walks the whole subtree of `small`; a subtree whose box can hold
// no corner that passes either test (a corner on big's top or bottom line
// inside its x range, or, by the reference's condition, on its left or
// right line below its bottom) is skipped, with a margin of 1e-12 around the
// 1e-14 tests: the walk order and the hits are unchanged.
void QuadTree::descendant_neighbors(int big, int small, std::vector<int>* out) const {
  const double top = nodes[big].corners[3];
  const double bottom = nodes[big].corners[1];
  const double left = nodes[big].corners[0];
  const double right = nodes[big].corners[4];
  {
    const double* sc = nodes[small].corners;
    const double sx0 = sc[0], sx1 = sc[4], sy0 = sc[1], sy1 = sc[3], m = 1e-12;
    const bool near_row = (sy0 - m < top && top < sy1 + m) || (sy0 - m < bottom && bottom < sy1 + m);
    const bool can_a = sx1 > left - m && sx0 < right + m && near_row;
    const bool near_col = (sx0 - m < left && left < sx1 + m) || (sx0 - m < right && right < sx1 + m);
    const bool can_b = sy0 < bottom + m && near_col;
    if (!can_a && !can_b) return;
  }
  for (int i = 0; i < 8; i += 2) {
    const double x = nodes[small].corners[i];
    const double y = nodes[small].corners[i + 1];
    bool hit = false;
    if (x > left && x < right) {
      if (std::fabs(y - top) < 1e-14 || std::fabs(y - bottom) < 1e-14) hit = true;
    }
    // The reference tests `y < top && y < bottom` here (not y > bottom).
    if (!hit && y < top && y < bottom) {
      if (std::fabs(x - left) < 1e-14 || std::fabs(x - right) < 1e-14) hit = true;
    }
    if (hit) {
      out->push_back(small);
      break;
    }
  }
  for (int c = 0; c < 4; ++c) {
    const int ch = nodes[small].children[c];
    if (ch >= 0) descendant_neighbors(big, ch, out);
  }
}

namespace {
// A box of the partition before it is numbered.
struct PBox {
  double corners[8];
  double side;
  int level;
  int parent;   // PBox index
  int kids[4];  // PBox indices {bl, tl, tr, br}; -1 for a leaf
  int a, b;     // its points: ord[a, b), ascending point index
  int t;        // the point whose arrival splits it (boxes that split)
};
constexpr int kMaxTreeDepth = 256;  // boxes 2^-256 of the root: coincident points
}  // namespace

// The tree that inserting points 0..n-1 one at a time (add, subdivide)
// makes, formed by recursive partition of the point indices with the same
// midpoint comparisons.  A box splits iff more than cap = max_leaf_dofs / sd
// of the points fall in it, and it splits when the (cap + 1)-th of them in
// index order arrives.  The splits one point causes form a chain, from a box
// down through the one child that holds all cap + 1 of its points, so ordering
// the splits by (that point, depth) gives the order in which insertion creates
// boxes; node ids and level lists follow it.  Leaf lists are in point order,
// as insertion leaves them.  Returns false when points coincide so that
// boxes split past kMaxTreeDepth levels (insertion would not end).
bool QuadTree::partition_build(int n) {
  const int cap = leaf_ / sd;
  std::vector<int> ord(n), tmp(n);
  std::vector<unsigned char> quad(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::vector<PBox> box(1);
  {
    PBox& r = box[0];
    for (int i = 0; i < 8; ++i) r.corners[i] = nodes[root].corners[i];
    r.side = nodes[root].side;
    r.level = 0;
    r.parent = -1;
    r.kids[0] = r.kids[1] = r.kids[2] = r.kids[3] = -1;
    r.a = 0;
    r.b = n;
    r.t = -1;
  }
  const double* pts = pts_;
  int* const ordp = ord.data();
  int* const tmpp = tmp.data();
  unsigned char* const quadp = quad.data();
  // quadrant of ord[j] (0 bl, 1 tl, 2 tr, 3 br: x < midx goes left, y < midy
  // goes down, as in subdivide) into quad[j], counted into c[4]
  auto classify = [pts, ordp, quadp](int j0, int j1, double midx, double midy, int* c) {
    const int* __restrict o = ordp;
    unsigned char* __restrict qd = quadp;
    int c0 = 0, c1 = 0, c2 = 0;
    for (int j = j0; j < j1; ++j) {
      const size_t v = static_cast<size_t>(o[j]);
      const double x = pts[2 * v], y = pts[2 * v + 1];
      const int left = x < midx, low = y < midy;
      const int q = left ? (low ? 0 : 1) : (low ? 3 : 2);
      qd[j] = static_cast<unsigned char>(q);
      c0 += q == 0;
      c1 += q == 1;
      c2 += q == 2;
    }
    c[0] = c0;
    c[1] = c1;
    c[2] = c2;
    c[3] = (j1 - j0) - c0 - c1 - c2;
  };
  // stable scatter of ord[j0, j1) to tmp from the four write positions (in
  // registers: an indexed position array would chain every store to the last)
  auto scatter = [ordp, tmpp, quadp](int j0, int j1, const int* pos) {
    const int* __restrict o = ordp;
    const unsigned char* __restrict qd = quadp;
    int* __restrict t = tmpp;
    int p0 = pos[0], p1 = pos[1], p2 = pos[2], p3 = pos[3];
    for (int j = j0; j < j1; ++j) {
      const int v = o[j];
      switch (qd[j]) {
        case 0: t[p0++] = v; break;
        case 1: t[p1++] = v; break;
        case 2: t[p2++] = v; break;
        default: t[p3++] = v; break;
      }
    }
  };
  const int nthreads = std::max(1, omp_get_max_threads());
  constexpr int kChunked = 16384;  // boxes at least this large split over threads
  std::vector<int> level_boxes(1, 0), split, splits, big_cnt;
  std::vector<double> mid;
  std::vector<int> cnt;
  while (!level_boxes.empty()) {
    split.clear();
    for (int k : level_boxes)
      if (box[k].b - box[k].a > cap) {
        if (box[k].level >= kMaxTreeDepth) return false;
        split.push_back(k);
      }
    if (split.empty()) break;
    const int ns = static_cast<int>(split.size());
    mid.resize(2 * (size_t)ns);
    cnt.assign(4 * (size_t)ns, 0);
    size_t work = 0;
    for (int i = 0; i < ns; ++i) {
      PBox& bx = box[split[i]];
      const double* c = bx.corners;
      mid[2 * i] = ((c[6] - c[0]) / 2.0) + c[0];
      mid[2 * i + 1] = ((c[3] - c[1]) / 2.0) + c[1];
      bx.t = ord[bx.a + cap];  // ord is ascending within a box
      work += bx.b - bx.a;
    }
    // large boxes: chunks over the threads, offsets by prefix over chunks
    for (int i = 0; i < ns; ++i) {
      const PBox& bx = box[split[i]];
      if (nthreads == 1 || bx.b - bx.a < kChunked) continue;
      const int a = bx.a, b = bx.b, len = b - a;
      big_cnt.assign(4 * (size_t)nthreads, 0);
#pragma omp parallel num_threads(nthreads)
      {
        const int nt = omp_get_num_threads(), t = omp_get_thread_num();
        const int chunk = (len + nt - 1) / nt;
        const int j0 = std::min(b, a + t * chunk), j1 = std::min(b, j0 + chunk);
        classify(j0, j1, mid[2 * i], mid[2 * i + 1], &big_cnt[4 * (size_t)t]);
#pragma omp barrier
        int pos[4];
        for (int q = 0, base = a; q < 4; ++q) {
          int before = 0, total = 0;
          for (int u = 0; u < nt; ++u) {
            if (u < t) before += big_cnt[4 * (size_t)u + q];
            total += big_cnt[4 * (size_t)u + q];
          }
          pos[q] = base + before;
          base += total;
          if (t == 0) cnt[4 * (size_t)i + q] = total;
        }
        scatter(j0, j1, pos);
#pragma omp barrier
        std::copy(tmp.begin() + j0, tmp.begin() + j1, ord.begin() + j0);
      }
    }
    // the other boxes: one thread each
#pragma omp parallel for schedule(dynamic, 2) if (nthreads > 1 && work > 4096)
    for (int i = 0; i < ns; ++i) {
      const PBox& bx = box[split[i]];
      if (nthreads > 1 && bx.b - bx.a >= kChunked) continue;
      int* c = &cnt[4 * (size_t)i];
      classify(bx.a, bx.b, mid[2 * i], mid[2 * i + 1], c);
      const int pos[4] = {bx.a, bx.a + c[0], bx.a + c[0] + c[1], bx.a + c[0] + c[1] + c[2]};
      scatter(bx.a, bx.b, pos);
      std::copy(tmp.begin() + bx.a, tmp.begin() + bx.b, ord.begin() + bx.a);
    }
    // children, corners as in subdivide: box i's four at base + 4 i + q
    const int base = static_cast<int>(box.size());
    box.resize(box.size() + 4 * (size_t)ns);
    level_boxes.resize(4 * (size_t)ns);
#pragma omp parallel for schedule(static) if (nthreads > 1 && ns >= 256)
    for (int i = 0; i < ns; ++i) {
      const int k = split[i];
      double c[8];
      for (int u = 0; u < 8; ++u) c[u] = box[k].corners[u];
      const double midx = mid[2 * i], midy = mid[2 * i + 1];
      const double cq[4][8] = {{c[0], c[1], c[2], midy, midx, midy, midx, c[7]},
                               {c[0], midy, c[2], c[3], midx, c[5], midx, midy},
                               {midx, midy, midx, c[3], c[4], c[5], c[6], midy},
                               {midx, c[1], midx, midy, c[4], midy, c[6], c[7]}};
      const double side = box[k].side / 2.0;
      const int level = box[k].level + 1;
      int start = box[k].a;
      for (int q = 0; q < 4; ++q) {
        const int idx = base + 4 * i + q;
        PBox& ch = box[idx];
        for (int u = 0; u < 8; ++u) ch.corners[u] = cq[q][u];
        ch.side = side;
        ch.level = level;
        ch.parent = k;
        ch.kids[0] = ch.kids[1] = ch.kids[2] = ch.kids[3] = -1;
        ch.a = start;
        ch.b = start + cnt[4 * (size_t)i + q];
        ch.t = -1;
        start = ch.b;
        box[k].kids[q] = idx;
        level_boxes[4 * (size_t)i + q] = idx;
      }
    }
    splits.insert(splits.end(), split.begin(), split.end());
  }
  std::stable_sort(splits.begin(), splits.end(), [&box](int u, int v) {
    return box[u].t != box[v].t ? box[u].t < box[v].t : box[u].level < box[v].level;
  });
  std::vector<int> id(box.size(), -1);
  id[0] = root;
  int next = root + 1;
  levels.assign(1, std::vector<int>(1, root));
  for (int k : splits) {
    for (int q = 0; q < 4; ++q) id[box[k].kids[q]] = next++;
    const int lv = box[k].level + 1;
    if (static_cast<int>(levels.size()) <= lv) levels.resize(lv + 1);
    // level lists take the children as bl, br, tr, tl
    for (int q : {0, 3, 2, 1}) levels[lv].push_back(id[box[k].kids[q]]);
  }
  nodes.resize(box.size());
  const int nbox = static_cast<int>(box.size());
#pragma omp parallel for schedule(dynamic, 64) if (nbox >= 1024)
  for (int k = 0; k < nbox; ++k) {
    const PBox& p = box[k];
    TreeNode& nd = nodes[id[k]];
    nd.level = p.level;
    nd.parent = p.parent >= 0 ? id[p.parent] : -1;
    nd.is_leaf = p.kids[0] < 0 ? 1 : 0;
    for (int q = 0; q < 4; ++q) nd.children[q] = p.kids[q] >= 0 ? id[p.kids[q]] : -1;
    nd.bl = nd.children[0];
    nd.tl = nd.children[1];
    nd.tr = nd.children[2];
    nd.br = nd.children[3];
    for (int i = 0; i < 8; ++i) nd.corners[i] = p.corners[i];
    nd.side = p.side;
    nd.tree_id = 0;
    nd.original.clear();
    if (nd.is_leaf) {
      nd.original.reserve(static_cast<size_t>(p.b - p.a) * sd);
      for (int j = p.a; j < p.b; ++j)
        for (int c = 0; c < sd; ++c) nd.original.push_back(sd * ord[j] + c);
    }
  }
  return true;
}

bool QuadTree::build(const double* points, int n, int sd_, int max_leaf_dofs) {
  levels.clear();
  if (n <= 0 || points == nullptr) {
    nodes.clear();
    return false;
  }
  pts_ = points;
  sd = sd_;
  leaf_ = max_leaf_dofs;
  // the previous tree's nodes are overwritten in place (partition_build),
  // so their lists' storage is reused
  if (nodes.empty()) nodes.emplace_back();
  double mn = points[0], mx = points[0];  // min and max are exact in any order
#pragma omp parallel for reduction(min : mn) reduction(max : mx) if (n >= 16384)
  for (int i = 0; i < 2 * n; ++i) {
    if (points[i] < mn) mn = points[i];
    if (points[i] > mx) mx = points[i];
  }
  min = mn;
  max = mx;
  const double lo = mn - 0.01, hi = mx + 0.01;
  root = 0;
  TreeNode& r = nodes[root];
  const double rc[8] = {lo, lo, lo, hi, hi, hi, hi, lo};
  for (int i = 0; i < 8; ++i) r.corners[i] = rc[i];
  r.side = hi - lo;
  if (!partition_build(n)) {
    nodes.clear();
    levels.clear();
    pts_ = nullptr;
    return false;
  }
  compute_neighbors();
  number_levels();
  roots.assign(1, root);
  pts_ = nullptr;
  return true;
}

void QuadTree::merge(const std::vector<QuadTree>& parts, const std::vector<int>& dof_offset) {
  nodes.clear();
  levels.clear();
  roots.clear();
  sd = parts.empty() ? 1 : parts[0].sd;
  min = 0;
  max = 0;
  for (size_t t = 0; t < parts.size(); ++t) {
    const QuadTree& q = parts[t];
    const int o = static_cast<int>(nodes.size());
    auto sh = [o](int id) { return id >= 0 ? id + o : -1; };
    for (TreeNode nd : q.nodes) {
      nd.parent = sh(nd.parent);
      for (int c = 0; c < 4; ++c) nd.children[c] = sh(nd.children[c]);
      nd.bl = sh(nd.bl);
      nd.tl = sh(nd.tl);
      nd.tr = sh(nd.tr);
      nd.br = sh(nd.br);
      for (int& nb : nd.neighbors) nb = sh(nb);
      for (int& d : nd.original) d += dof_offset[t];
      nd.tree_id = static_cast<int>(t);
      nodes.push_back(std::move(nd));
    }
    if (levels.size() < q.levels.size()) levels.resize(q.levels.size());
    for (size_t lv = 0; lv < q.levels.size(); ++lv)
      for (int id : q.levels[lv]) levels[lv].push_back(id + o);
    roots.push_back(q.root + o);
    if (t == 0 || q.min < min) min = q.min;
    if (t == 0 || q.max > max) max = q.max;
  }
  root = roots.empty() ? -1 : roots[0];
  number_levels();
}

// quadtree.cpp:131-175, level by level.  Within a level each box's own
// list takes its siblings and cousins (reading only the coarser level's
// finished lists), and each leaf finds the finer boxes touching it; the
// boxes of a level are independent there and run in parallel.  The
// leaf <-> finer-box links then go in sequentially, in level order, so
// every list is in the reference's order.  (A leaf's walk reads only its own
// same-level neighbours, and the links it adds are to finer boxes, whose
// own sibling/cousin entries come after them, as in the reference.)
void QuadTree::compute_neighbors() {
  for (TreeNode& nd : nodes) nd.neighbors.clear();
  const double sqrt2 = std::sqrt(2.0);
  std::vector<std::vector<int>> hits;
  std::vector<int> extra(nodes.size(), 0), slot(nodes.size(), 0), touched, group, group_off,
      group_fill;
  for (size_t lv = 0; lv < levels.size(); ++lv) {
    const std::vector<int>& L = levels[lv];
    const int m = static_cast<int>(L.size());
    if (static_cast<int>(hits.size()) < m) hits.resize(m);
#pragma omp parallel for schedule(dynamic, 16) if (m >= 256)
    for (int k = 0; k < m; ++k) {
      const int a = L[k];
      TreeNode& na = nodes[a];
      const int par = na.parent;
      if (par >= 0) {
        const std::vector<int>& pn = nodes[par].neighbors;
        na.neighbors.reserve(na.neighbors.size() + 3 + 4 * pn.size());
        for (int c = 0; c < 4; ++c) {
          const int sib = nodes[par].children[c];
          if (sib != a) na.neighbors.push_back(sib);
        }
        for (size_t q = 0; q < pn.size(); ++q) {
          for (int c = 0; c < 4; ++c) {
            const int cousin = nodes[pn[q]].children[c];
            if (cousin < 0 || nodes[cousin].level != na.level) continue;
            const double dx = na.corners[0] - nodes[cousin].corners[0];
            const double dy = na.corners[1] - nodes[cousin].corners[1];
            const double dist = std::sqrt(dx * dx + dy * dy);
            if (dist < na.side * sqrt2 + 1e-5) na.neighbors.push_back(cousin);
          }
        }
      }
      hits[k].clear();
      if (na.is_leaf) {
        for (size_t q = 0; q < na.neighbors.size(); ++q) {
          const int nb = na.neighbors[q];
          if (nodes[nb].level != na.level) continue;
          for (int c = 0; c < 4; ++c) {
            const int ch = nodes[nb].children[c];
            if (ch >= 0) descendant_neighbors(a, ch, &hits[k]);
          }
        }
      }
    }
    // The links, in the reference's order, with the list appends in
    // parallel: each leaf of the level appends its own hits, and each finer
    // box appends the leaves that found it in level order (grouped by a
    // counting pass over the hits, which keeps that order).
    touched.clear();
    for (int k = 0; k < m; ++k)
      for (int sm : hits[k])
        if (extra[sm]++ == 0) touched.push_back(sm);
    const int nt = static_cast<int>(touched.size());
    group_off.resize(nt + 1);
    group_off[0] = 0;
    for (int u = 0; u < nt; ++u) {
      slot[touched[u]] = u;
      group_off[u + 1] = group_off[u] + extra[touched[u]];
    }
    group.resize(group_off[nt]);
    group_fill.assign(group_off.begin(), group_off.end() - 1);
    for (int k = 0; k < m; ++k)
      for (int sm : hits[k]) group[group_fill[slot[sm]]++] = L[k];
#pragma omp parallel for schedule(dynamic, 32) if (nt + m >= 512)
    for (int u = 0; u < nt + m; ++u) {
      if (u < nt) {
        std::vector<int>& nb = nodes[touched[u]].neighbors;
        nb.reserve(nb.size() + (group_off[u + 1] - group_off[u]) + 12);  // + siblings, cousins
        nb.insert(nb.end(), group.begin() + group_off[u], group.begin() + group_off[u + 1]);
        extra[touched[u]] = 0;
      } else {
        const int k = u - nt;
        std::vector<int>& nb = nodes[L[k]].neighbors;
        nb.insert(nb.end(), hits[k].begin(), hits[k].end());
      }
    }
  }
}

void QuadTree::number_levels() {
  level_order.clear();
  level_rank.assign(nodes.size(), -1);
  for (const auto& lvl : levels)
    for (int id : lvl) {
      level_rank[id] = static_cast<int>(level_order.size());
      level_order.push_back(id);
    }
}

// The leaf holding (x, y), by the midpoint rule of recursive_add.
int QuadTree::find_leaf(double x, double y) const {
  int cur = root;
  while (!nodes[cur].is_leaf) {
    const TreeNode& nd = nodes[cur];
    const double midx = ((nd.corners[6] - nd.corners[0]) / 2.0) + nd.corners[0];
    const double midy = ((nd.corners[3] - nd.corners[1]) / 2.0) + nd.corners[1];
    if (x < midx && y < midy) cur = nd.bl;
    else if (x < midx && y >= midy) cur = nd.tl;
    else if (x >= midx && y < midy) cur = nd.br;
    else cur = nd.tr;
  }
  return cur;
}

// quadtree.cpp:435-461
void QuadTree::mark(int id, std::vector<char>* marked) const {
  for (int cur = id; cur >= 0; cur = nodes[cur].parent) {
    (*marked)[cur] = 1;
    for (int nb : nodes[cur].neighbors) (*marked)[nb] = 1;
  }
}

// quadtree.cpp:464-513: the subtree's leaf DOFs move into `id`, which
// becomes a leaf; its descendants leave the tree.
void QuadTree::consolidate(int id, std::vector<char>* dead) {
  std::vector<int> queue(1, id), dofs;
  for (size_t i = 0; i < queue.size(); ++i) {
    const TreeNode& cur = nodes[queue[i]];
    if (cur.is_leaf) dofs.insert(dofs.end(), cur.original.begin(), cur.original.end());
    else
      for (int c = 0; c < 4; ++c)
        if (cur.children[c] >= 0) queue.push_back(cur.children[c]);
    if (queue[i] != id) (*dead)[queue[i]] = 1;
  }
  TreeNode& nd = nodes[id];
  nd.original = dofs;
  nd.bl = nd.tl = nd.tr = nd.br = -1;
  for (int c = 0; c < 4; ++c) nd.children[c] = -1;
  nd.is_leaf = 1;
}

void QuadTree::perturb(const double* old_points, const double* new_points, int n_new,
                       const std::vector<int>& old_to_new, std::vector<int>* id_map,
                       std::vector<char>* marked) {
  const int n_old = static_cast<int>(old_to_new.size());
  std::vector<char> found(n_new, 0);
  for (int p = 0; p < n_old; ++p)
    if (old_to_new[p] >= 0) found[old_to_new[p]] = 1;
  marked->assign(nodes.size(), 0);
  // renumber the leaves' DOFs (quadtree.cpp:583-598)
  for (TreeNode& nd : nodes) {
    if (!nd.is_leaf) continue;
    std::vector<int> ob;
    for (int d : nd.original) {
      const int q = old_to_new[d / sd];
      if (q >= 0) ob.push_back(sd * q + d % sd);
    }
    nd.original.swap(ob);
  }
  // additions (quadtree.cpp:639-668)
  std::vector<int> bursting;
  for (int i = 0; i < n_new; ++i) {
    if (found[i]) continue;
    const int leaf = find_leaf(new_points[2 * i], new_points[2 * i + 1]);
    for (int c = 0; c < sd; ++c) nodes[leaf].original.push_back(sd * i + c);
    bursting.push_back(leaf);
    mark(leaf, marked);
  }
  // DOFs below each box (quadtree.cpp:670-684)
  std::vector<int> below(nodes.size(), 0);
  for (int lv = static_cast<int>(levels.size()) - 1; lv >= 0; --lv)
    for (int id : levels[lv]) {
      if (nodes[id].is_leaf) below[id] = static_cast<int>(nodes[id].original.size());
      const int par = nodes[id].parent;
      if (par >= 0) below[par] += below[id];
    }
  // deletions (quadtree.cpp:686-715): the first box on the way down holding
  // fewer than MAX_LEAF_DOFS DOFs is consolidated
  std::vector<char> sparse(nodes.size(), 0);
  for (int p = 0; p < n_old; ++p) {
    if (old_to_new[p] >= 0) continue;
    const double x = old_points[2 * p], y = old_points[2 * p + 1];
    int cur = root;
    bool path_marked = false;
    while (!nodes[cur].is_leaf) {
      if (below[cur] < leaf_ && !path_marked) {
        path_marked = true;
        sparse[cur] = 1;
      }
      const TreeNode& nd = nodes[cur];
      const double midx = ((nd.corners[6] - nd.corners[0]) / 2.0) + nd.corners[0];
      const double midy = ((nd.corners[3] - nd.corners[1]) / 2.0) + nd.corners[1];
      if (x < midx && y < midy) cur = nd.bl;
      else if (x < midx && y >= midy) cur = nd.tl;
      else if (x >= midx && y < midy) cur = nd.br;
      else cur = nd.tr;
    }
    mark(cur, marked);
  }
  // split bursting leaves (quadtree.cpp:727-733), new boxes start unmarked-
  // less: they have no factorization
  pts_ = new_points;
  const size_t before = nodes.size();
  for (int id : bursting)
    if (nodes[id].is_leaf && static_cast<int>(nodes[id].original.size()) > leaf_) subdivide(id);
  pts_ = nullptr;
  marked->resize(nodes.size(), 1);
  for (size_t i = before; i < nodes.size(); ++i) (*marked)[i] = 1;
  // consolidate sparse boxes (quadtree.cpp:737-739)
  std::vector<char> dead(nodes.size(), 0);
  for (size_t id = 0; id < sparse.size(); ++id)
    if (sparse[id] && !dead[id]) consolidate(static_cast<int>(id), &dead);
  // renumber without the removed boxes; levels keep their order
  id_map->assign(nodes.size(), -1);
  std::vector<TreeNode> kept;
  std::vector<char> kmark;
  for (size_t id = 0; id < nodes.size(); ++id) {
    if (dead[id]) continue;
    (*id_map)[id] = static_cast<int>(kept.size());
    kept.push_back(nodes[id]);
    kmark.push_back((*marked)[id]);
  }
  auto remap = [&](int v) { return v >= 0 ? (*id_map)[v] : -1; };
  for (TreeNode& nd : kept) {
    nd.parent = remap(nd.parent);
    for (int c = 0; c < 4; ++c) nd.children[c] = remap(nd.children[c]);
    nd.bl = remap(nd.bl);
    nd.tl = remap(nd.tl);
    nd.tr = remap(nd.tr);
    nd.br = remap(nd.br);
  }
  for (auto& lvl : levels) {
    std::vector<int> l2;
    for (int id : lvl)
      if (!dead[id]) l2.push_back((*id_map)[id]);
    lvl.swap(l2);
  }
  while (!levels.empty() && levels.back().empty()) levels.pop_back();
  root = remap(root);
  roots.assign(1, root);
  nodes.swap(kept);
  marked->swap(kmark);
  compute_neighbors();  // quadtree.cpp:759-797, the same rules as the build
  number_levels();
}

}  // namespace rskel
