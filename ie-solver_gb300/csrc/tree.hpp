// Host quadtree over the boundary nodes, bit-exact with the reference's
// QuadTree::initialize_tree (ie_solver/quadtree/quadtree.cpp:39-432):
//  * bounding square [min - 0.01, max + 0.01] with min/max pooled over x and y;
//  * points inserted in index order, DOFs sd*i + c pushed along the path;
//  * a leaf splits when its DOF count exceeds max_leaf_dofs; children are
//    appended to their level as bl, br, tr, tl, while children[] is
//    {bl, tl, tr, br}; the parent's DOFs are redistributed in parent order;
//  * neighbour lists: siblings, parents' neighbours' children within
//    s*sqrt(2) + 1e-5 (bottom-left corners), plus leaf <-> finer-box links
//    including the reference's `y < top && y < bottom` condition.
// Compiled with floating-point contraction off so x86-64 and aarch64 hosts
// produce the same tree.
#pragma once

#include <vector>

namespace rskel {

struct TreeNode {
  int level = 0;
  int is_leaf = 1;
  int parent = -1;
  int children[4] = {-1, -1, -1, -1};  // bl, tl, tr, br
  int bl = -1, tl = -1, tr = -1, br = -1;
  double corners[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // {BL, TL, TR, BR} x,y pairs
  double side = 0;
  std::vector<int> neighbors;
  std::vector<int> original;  // DOF indices (leaves only; QuadTree::box_dofs for any box)
  int tree_id = 0;            // which tree of a forest (batch of boundaries) the box is in
};

struct QuadTree {
  std::vector<TreeNode> nodes;           // creation order
  std::vector<std::vector<int>> levels;  // node ids per level, reference order
  double min = 0, max = 0;
  int root = -1;
  std::vector<int> roots;  // every tree's root (a forest holds one tree per boundary)
  int sd = 1;

  // points: interleaved (2n). Returns false on empty input.
  bool build(const double* points, int n, int sd, int max_leaf_dofs);
  // A forest of independent trees, one per boundary of a batch: the parts'
  // nodes appended in order with their ids shifted, their DOF indices
  // shifted by dof_offset[t], levels merged by depth (level l holds every
  // tree's level-l boxes, tree by tree), neighbour lists within each tree.
  void merge(const std::vector<QuadTree>& parts, const std::vector<int>& dof_offset);
  // A box's DOFs in point order: the leaf's list, or the ordered union of
  // the leaves below it (original_box of the reference).
  std::vector<int> box_dofs(int id) const;

  // QuadTree::perturb (quadtree.cpp:435-801) for a boundary whose points
  // moved: old_to_new[p] is the new index of old point p (-1 if it is gone),
  // points of the new boundary not in the old one are added.  Leaf DOF
  // lists are renumbered, added points go to their leaves, emptied subtrees
  // below MAX_LEAF_DOFS are consolidated, bursting leaves split, and the
  // neighbour lists are rebuilt.  Nodes are then renumbered without the
  // removed ones: id_map[old id] = new id or -1.  marked[new id] = 1 for the
  // boxes whose factorization is dropped (mark_neighbors_and_parents: the
  // leaves that gained or lost points, their neighbours, their ancestors and
  // the ancestors' neighbours), and for new boxes.
  void perturb(const double* old_points, const double* new_points, int n_new,
               const std::vector<int>& old_to_new, std::vector<int>* id_map,
               std::vector<char>* marked);
  // level-order numbering (level 0 first) <-> creation ids
  std::vector<int> level_order;   // level-order index -> node id
  std::vector<int> level_rank;    // node id -> level-order index

 private:
  const double* pts_ = nullptr;
  int leaf_ = 32;
  int new_node();
  void push_level(int level, int id);
  void subdivide(int id);
  bool partition_build(int n);
  void descendant_neighbors(int big, int small, std::vector<int>* out) const;
  void compute_neighbors();
  void number_levels();
  int find_leaf(double x, double y) const;
  void mark(int id, std::vector<char>* marked) const;
  void consolidate(int id, std::vector<char>* dead);
};

}  // namespace rskel
