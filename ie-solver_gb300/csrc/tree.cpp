// Host quadtree construction; see tree.hpp for the rules it reproduces.
#include "tree.hpp"

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

// quadtree.cpp:230-269.  The reference appends the point's DOFs to every
// box on its path; here they go to the leaf only (a box's own list is the
// ordered union of its leaves' lists, since every list is in point order,
// and box_dofs forms it when asked): the tree, its creation order and every
// leaf list come out the same.  The walk starts from the previous point's
// box when the point lies in it: a box's edges are the very midpoints the
// walk compares with (x < mid goes left), so the box test [x0, x1) x [y0, y1)
// takes the same decisions as the walk from the root.
void QuadTree::add(int id, double x, double y, int point) {
  int cur = id;
  if (hint_ >= 0) {
    const TreeNode& h = nodes[hint_];
    if (x >= h.corners[0] && x < h.corners[4] && y >= h.corners[1] && y < h.corners[3]) cur = hint_;
  }
  while (!nodes[cur].is_leaf) {
    const TreeNode& nd = nodes[cur];
    const double midx = ((nd.corners[6] - nd.corners[0]) / 2.0) + nd.corners[0];
    const double midy = ((nd.corners[3] - nd.corners[1]) / 2.0) + nd.corners[1];
    if (x < midx && y < midy) cur = nd.bl;
    else if (x < midx && y >= midy) cur = nd.tl;
    else if (x >= midx && y < midy) cur = nd.br;
    else cur = nd.tr;
  }
  for (int c = 0; c < sd; ++c) nodes[cur].original.push_back(sd * point + c);
  hint_ = cur;
  if (static_cast<int>(nodes[cur].original.size()) > leaf_) subdivide(cur);
}

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

// quadtree.cpp:185-227.  The reference walks the whole subtree of `small`;
// a subtree whose box can hold no corner that passes either test (a corner
// on big's top or bottom line inside its x range, or, by the reference's
// condition, on its left or right line below its bottom) is skipped, with
// a margin of 1e-12 around the 1e-14 tests: the walk order and the hits are
// unchanged.
void QuadTree::descendant_neighbors(int big, int small) {
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
      nodes[big].neighbors.push_back(small);
      nodes[small].neighbors.push_back(big);
      break;
    }
  }
  for (int c = 0; c < 4; ++c) {
    const int ch = nodes[small].children[c];
    if (ch >= 0) descendant_neighbors(big, ch);
  }
}

bool QuadTree::build(const double* points, int n, int sd_, int max_leaf_dofs) {
  nodes.clear();
  levels.clear();
  if (n <= 0 || points == nullptr) return false;
  pts_ = points;
  sd = sd_;
  leaf_ = max_leaf_dofs;
  nodes.reserve(static_cast<size_t>(8 * (n * sd_ / (max_leaf_dofs > 0 ? max_leaf_dofs : 1) + 1)));
  double mn = points[0], mx = points[0];
  for (int i = 0; i < 2 * n; ++i) {
    if (points[i] < mn) mn = points[i];
    if (points[i] > mx) mx = points[i];
  }
  min = mn;
  max = mx;
  const double lo = mn - 0.01, hi = mx + 0.01;
  root = new_node();
  TreeNode& r = nodes[root];
  const double rc[8] = {lo, lo, lo, hi, hi, hi, hi, lo};
  for (int i = 0; i < 8; ++i) r.corners[i] = rc[i];
  r.side = hi - lo;
  push_level(0, root);
  hint_ = -1;
  for (int i = 0; i < n; ++i) add(root, points[2 * i], points[2 * i + 1], i);

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

// quadtree.cpp:131-175
void QuadTree::compute_neighbors() {
  for (TreeNode& nd : nodes) nd.neighbors.clear();
  const double sqrt2 = std::sqrt(2.0);
  for (size_t lv = 0; lv < levels.size(); ++lv) {
    for (size_t k = 0; k < levels[lv].size(); ++k) {
      const int a = levels[lv][k];
      const int par = nodes[a].parent;
      if (par >= 0) {
        for (int c = 0; c < 4; ++c) {
          const int sib = nodes[par].children[c];
          if (sib != a) nodes[a].neighbors.push_back(sib);
        }
        const std::vector<int>& pn = nodes[par].neighbors;
        for (size_t q = 0; q < pn.size(); ++q) {
          for (int c = 0; c < 4; ++c) {
            const int cousin = nodes[pn[q]].children[c];
            if (cousin < 0 || nodes[cousin].level != nodes[a].level) continue;
            const double dx = nodes[a].corners[0] - nodes[cousin].corners[0];
            const double dy = nodes[a].corners[1] - nodes[cousin].corners[1];
            const double dist = std::sqrt(dx * dx + dy * dy);
            if (dist < nodes[a].side * sqrt2 + 1e-5) nodes[a].neighbors.push_back(cousin);
          }
        }
      }
      if (nodes[a].is_leaf) {
        for (size_t q = 0; q < nodes[a].neighbors.size(); ++q) {
          const int nb = nodes[a].neighbors[q];
          if (nodes[nb].level != nodes[a].level) continue;
          for (int c = 0; c < 4; ++c) {
            const int ch = nodes[nb].children[c];
            if (ch >= 0) descendant_neighbors(a, ch);
          }
        }
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
