// Driver that runs the reference solver (compiled from its own sources by
// oracle/Makefile into oracle/_ref/) on one problem file and writes what it
// computed: the quadtree (level order, corners, DOF lists, neighbor lists),
// per-box skeleton/redundant lists, the solution, and factor/solve timings.
//
// Test infrastructure only: it produces golden vectors and pins the oracle
// restatement.  It is never linked into the product library.
//
// Problem file ("RSPROB01"), little endian:
//   int32 pde, sd, num_points, num_holes, nrhs, max_leaf_dofs, num_proxy_points,
//         num_threads, repeats, dense_check
//   double id_tol
//   double points[2N], normals[2N], weights[N], curvatures[N]
//   double hole_centers[2H], hole_radii[H]
//   double rhs[N*sd*nrhs]   (column major)
// Result file ("RSRES001"): a sequence of named int32/float64 arrays.
#include <omp.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <unordered_map>

#include "ie_solver/ie_mat.h"
#include "ie_solver/quadtree/quadtree.h"
#include "ie_solver/kernel/kernel.h"
#include "ie_solver/skel_factorization/skel_factorization.h"
#include "ie_solver/linear_solve.h"
#include "ie_solver/boundaries/boundary.h"

using namespace ie_solver;

namespace {

class DataBoundary : public Boundary {
 public:
  void initialize(int, BoundaryCondition) override {}
  bool is_in_domain(const Vec2&) override { return true; }
};

struct Problem {
  int pde, sd, n, h, nrhs, leaf, npp, threads, repeats, dense_check;
  double tol;
  std::vector<double> pts, nrm, w, curv, hc, hr, rhs;
};

bool read_exact(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

bool read_problem(const char* path, Problem* pr) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  char magic[8];
  int32_t hdr[10];
  bool ok = read_exact(f, magic, 8) && memcmp(magic, "RSPROB01", 8) == 0 &&
            read_exact(f, hdr, sizeof(hdr)) && read_exact(f, &pr->tol, 8);
  if (ok) {
    pr->pde = hdr[0]; pr->sd = hdr[1]; pr->n = hdr[2]; pr->h = hdr[3]; pr->nrhs = hdr[4];
    pr->leaf = hdr[5]; pr->npp = hdr[6]; pr->threads = hdr[7]; pr->repeats = hdr[8];
    pr->dense_check = hdr[9];
    auto rd = [&](std::vector<double>& v, size_t cnt) {
      v.resize(cnt);
      return cnt == 0 || read_exact(f, v.data(), cnt * 8);
    };
    ok = rd(pr->pts, 2 * (size_t)pr->n) && rd(pr->nrm, 2 * (size_t)pr->n) &&
         rd(pr->w, pr->n) && rd(pr->curv, pr->n) && rd(pr->hc, 2 * (size_t)pr->h) &&
         rd(pr->hr, pr->h) && rd(pr->rhs, (size_t)pr->n * pr->sd * pr->nrhs);
  }
  fclose(f);
  return ok;
}

struct Writer {
  FILE* f;
  explicit Writer(const char* path) { f = fopen(path, "wb"); if (f) fwrite("RSRES001", 1, 8, f); }
  ~Writer() { if (f) fclose(f); }
  void head(const std::string& name, int32_t dtype, int64_t cnt) {
    int32_t len = (int32_t)name.size();
    fwrite(&len, 4, 1, f); fwrite(name.data(), 1, len, f);
    fwrite(&dtype, 4, 1, f); fwrite(&cnt, 8, 1, f);
  }
  void i32(const std::string& name, const std::vector<int32_t>& v) {
    head(name, 1, (int64_t)v.size()); if (!v.empty()) fwrite(v.data(), 4, v.size(), f);
  }
  void f64(const std::string& name, const std::vector<double>& v) {
    head(name, 2, (int64_t)v.size()); if (!v.empty()) fwrite(v.data(), 8, v.size(), f);
  }
};

void csr_append(std::vector<int32_t>* off, std::vector<int32_t>* val, const std::vector<int>& v) {
  if (off->empty()) off->push_back(0);
  for (int x : v) val->push_back(x);
  off->push_back((int32_t)val->size());
}

ie_solver_config::Pde pde_of(int p) {
  return p == 0 ? ie_solver_config::LAPLACE
                : (p == 1 ? ie_solver_config::LAPLACE_NEUMANN : ie_solver_config::STOKES);
}

// The bordered operator [K U; Psi -I] applied to [mu; alpha] minus [f; 0],
// evaluated in row blocks so that large cases never hold the dense matrix.
void dense_residual(const Kernel& kernel, int ndofs, const ie_Mat& mu, const ie_Mat& f,
                    const ie_Mat& U, const ie_Mat& Psi, const ie_Mat* alpha,
                    std::vector<double>* res) {
  std::vector<int> all(ndofs);
  for (int i = 0; i < ndofs; ++i) all[i] = i;
  int nrhs = mu.width();
  res->assign((size_t)ndofs * nrhs, 0.0);
  const int blk = 256;
  for (int r0 = 0; r0 < ndofs; r0 += blk) {
    int r1 = std::min(ndofs, r0 + blk);
    std::vector<int> rows(all.begin() + r0, all.begin() + r1);
    ie_Mat kb = kernel(rows, all);
    ie_Mat prod = kb * mu;
    for (int c = 0; c < nrhs; ++c)
      for (int i = r0; i < r1; ++i) {
        double v = prod.get(i - r0, c) - f.get(i, c);
        if (alpha) for (int j = 0; j < U.width(); ++j) v += U.get(i, j) * alpha->get(j, c);
        (*res)[(size_t)c * ndofs + i] = v;
      }
  }
  if (alpha) {
    for (int i = 0; i < Psi.height(); ++i) {
      double v = -alpha->get(i, 0);
      for (int j = 0; j < ndofs; ++j) v += Psi.get(i, j) * mu.get(j, 0);
      res->push_back(v);
    }
  }
}

// The tree in level order: node fields, DOF lists and neighbour lists.
void write_tree(Writer& w, QuadTree& tree) {
  std::unordered_map<const QuadTreeNode*, int> gid;
  std::vector<const QuadTreeNode*> order;
  std::vector<int32_t> level_sizes;
  for (QuadTreeLevel* lvl : tree.levels) {
    level_sizes.push_back((int32_t)lvl->nodes.size());
    for (QuadTreeNode* nd : lvl->nodes) { gid[nd] = (int)order.size(); order.push_back(nd); }
  }
  std::vector<int32_t> lev, leaf, parent, children, compressed, nbr_off, nbr, orig_off, orig,
      act_off, act, skel_off, skel, red_off, red, near_off, near;
  std::vector<double> corners, side;
  for (const QuadTreeNode* nd : order) {
    lev.push_back(nd->level);
    leaf.push_back(nd->is_leaf ? 1 : 0);
    parent.push_back(nd->parent ? gid[nd->parent] : -1);
    for (int c = 0; c < 4; ++c) children.push_back(nd->children[c] ? gid[nd->children[c]] : -1);
    compressed.push_back(nd->compressed ? 1 : 0);
    for (int c = 0; c < 8; ++c) corners.push_back(nd->corners[c]);
    side.push_back(nd->side_length);
    std::vector<int> nb;
    for (QuadTreeNode* x : nd->neighbors) nb.push_back(gid[x]);
    csr_append(&nbr_off, &nbr, nb);
    csr_append(&orig_off, &orig, nd->src_dof_lists.original_box);
    csr_append(&act_off, &act, nd->src_dof_lists.active_box);
    csr_append(&skel_off, &skel, nd->src_dof_lists.skel);
    csr_append(&red_off, &red, nd->src_dof_lists.redundant);
    csr_append(&near_off, &near, nd->src_dof_lists.near);
  }
  w.i32("level_sizes", level_sizes);
  w.i32("node_level", lev); w.i32("node_leaf", leaf); w.i32("node_parent", parent);
  w.i32("node_children", children); w.i32("node_compressed", compressed);
  w.f64("node_corners", corners); w.f64("node_side", side);
  w.i32("nbr_off", nbr_off); w.i32("nbr", nbr);
  w.i32("orig_off", orig_off); w.i32("orig", orig);
  w.i32("active_off", act_off); w.i32("active", act);
  w.i32("skel_off", skel_off); w.i32("skel", skel);
  w.i32("red_off", red_off); w.i32("red", red);
  w.i32("near_off", near_off); w.i32("near", near);
}

int run_id_mode(const char* in, const char* out) {
  // "ID mode": read matrices (int32 count; per matrix int32 m, n; double tol;
  // double a[m*n] column major), run ie_Mat::id on each, write rank/perm/Z.
  FILE* f = fopen(in, "rb");
  if (!f) return 2;
  int32_t cnt = 0;
  if (!read_exact(f, &cnt, 4)) return 2;
  Writer w(out);
  std::vector<int32_t> ranks, perm_off, perm, dims;
  std::vector<double> zall;
  std::vector<int32_t> z_off{0};
  for (int t = 0; t < cnt; ++t) {
    int32_t mn[2]; double tol;
    if (!read_exact(f, mn, 8) || !read_exact(f, &tol, 8)) return 2;
    ie_Mat a(mn[0], mn[1]);
    if (!read_exact(f, a.mat, (size_t)mn[0] * mn[1] * 8)) return 2;
    std::vector<int> p;
    ie_Mat z;
    int k = a.id(&p, &z, tol);
    ranks.push_back(k);
    dims.push_back(mn[0]); dims.push_back(mn[1]);
    std::vector<int> pp(p.begin(), p.end());
    csr_append(&perm_off, &perm, pp);
    if (k > 0) for (int j = 0; j < z.width(); ++j) for (int i = 0; i < z.height(); ++i) zall.push_back(z.get(i, j));
    z_off.push_back((int32_t)zall.size());
  }
  fclose(f);
  w.i32("ranks", ranks); w.i32("dims", dims); w.i32("perm_off", perm_off); w.i32("perm", perm);
  w.f64("z", zall); w.i32("z_off", z_off);
  return 0;
}

DataBoundary boundary_of(const Problem& pr) {
  DataBoundary bnd;
  bnd.boundary_shape = Boundary::BoundaryShape::CIRCLE;
  bnd.points = pr.pts; bnd.normals = pr.nrm; bnd.weights = pr.w; bnd.curvatures = pr.curv;
  for (int i = 0; i < pr.h; ++i) {
    Hole hole;
    hole.center = Vec2(pr.hc[2 * i], pr.hc[2 * i + 1]);
    hole.radius = pr.hr[i];
    hole.num_nodes = 0;
    bnd.holes.push_back(hole);
  }
  return bnd;
}

int run_perturb_mode(int count, char** in, const char* out) {
  // "perturb mode": QuadTree::initialize_tree on the first problem's
  // boundary, then QuadTree::perturb (quadtree.cpp:520-801) with each later
  // problem's boundary in turn; writes the final tree.  No factorization:
  // the tree update does not depend on which boxes are compressed.
  std::vector<Problem> prs(count);
  for (int i = 0; i < count; ++i)
    if (!read_problem(in[i], &prs[i])) { fprintf(stderr, "bad problem file\n"); return 2; }
  if (prs[0].leaf != MAX_LEAF_DOFS) {
    fprintf(stderr, "this binary is built for leaf %d\n", MAX_LEAF_DOFS);
    return 3;
  }
  DataBoundary first = boundary_of(prs[0]);
  QuadTree tree;
  tree.initialize_tree(&first, std::vector<double>(), prs[0].sd, 2);
  for (int i = 1; i < count; ++i) {
    DataBoundary next = boundary_of(prs[i]);
    tree.perturb(next);
  }
  Writer w(out);
  if (!w.f) return 4;
  write_tree(w, tree);
  w.f64("tree_minmax", std::vector<double>{tree.min, tree.max});
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 4 && std::string(argv[1]) == "--id") return run_id_mode(argv[2], argv[3]);
  if (argc >= 5 && std::string(argv[1]) == "--perturb")
    return run_perturb_mode(argc - 3, argv + 2, argv[argc - 1]);
  // optional third argument --strong: SkelFactorization with strong admissibility
  const bool strong = argc == 4 && std::string(argv[3]) == "--strong";
  if (argc != 3 && !strong) {
    fprintf(stderr, "usage: %s problem.rsp result.rsr [--strong] | --id in out\n", argv[0]);
    return 2;
  }
  Problem pr;
  if (!read_problem(argv[1], &pr)) { fprintf(stderr, "bad problem file\n"); return 2; }
  if (pr.leaf != MAX_LEAF_DOFS || pr.npp != NUM_PROXY_POINTS) {
    fprintf(stderr, "this binary is built for leaf %d / proxy %d, problem wants %d / %d\n",
            MAX_LEAF_DOFS, NUM_PROXY_POINTS, pr.leaf, pr.npp);
    return 3;
  }
  scipy_openblas_set_num_threads(1);
  int ndofs = pr.n * pr.sd;
  DataBoundary bnd;
  bnd.boundary_shape = Boundary::BoundaryShape::CIRCLE;
  bnd.points = pr.pts; bnd.normals = pr.nrm; bnd.weights = pr.w; bnd.curvatures = pr.curv;
  for (int i = 0; i < pr.h; ++i) {
    Hole hole;
    hole.center = Vec2(pr.hc[2 * i], pr.hc[2 * i + 1]);
    hole.radius = pr.hr[i];
    hole.num_nodes = 0;
    bnd.holes.push_back(hole);
  }
  ie_Mat f(ndofs, pr.nrhs);
  memcpy(f.mat, pr.rhs.data(), pr.rhs.size() * 8);
  bnd.boundary_values = f;
  ie_solver_config::Pde pde = pde_of(pr.pde);
  Kernel::IMPROVE_CONDITION = 0;
  Kernel kernel(pr.sd, 2, pde, &bnd, std::vector<double>());
  bool holes = pr.h > 0 && pde != ie_solver_config::LAPLACE_NEUMANN;
  ie_Mat U, Psi;
  if (holes) {
    U = initialize_U_mat(pde, bnd.holes, bnd.points);
    Psi = initialize_Psi_mat(pde, bnd.holes, &bnd);
  }

  std::vector<double> t_factor, t_solve;
  QuadTree* keep = nullptr;
  ie_Mat mu, alpha;
  SkelFactorization sf(pr.tol, strong, pr.threads);
  int reps = std::max(1, pr.repeats);
  for (int rep = 0; rep < reps; ++rep) {
    QuadTree* tree = new QuadTree();
    tree->initialize_tree(&bnd, std::vector<double>(), pr.sd, 2);
    if (holes) { tree->U = U; tree->Psi = Psi; }
    double t0 = omp_get_wtime();
    sf.skeletonize(kernel, tree);
    double t1 = omp_get_wtime();
    if (holes) linear_solve(sf, *tree, f, &mu, &alpha);
    else linear_solve(sf, *tree, f, &mu);
    double t2 = omp_get_wtime();
    t_factor.push_back(t1 - t0);
    t_solve.push_back(t2 - t1);
    if (rep == reps - 1) keep = tree; else delete tree;
  }

  Writer w(argv[2]);
  if (!w.f) return 4;
  QuadTree& tree = *keep;
  write_tree(w, tree);
  std::vector<int32_t> allskel(tree.root->src_dof_lists.active_box.begin(),
                               tree.root->src_dof_lists.active_box.end());
  w.i32("allskel", allskel);
  w.f64("mu", std::vector<double>(mu.mat, mu.mat + (size_t)mu.height() * mu.width()));
  if (holes) w.f64("alpha", std::vector<double>(alpha.mat, alpha.mat + alpha.height()));
  w.f64("t_factor", t_factor); w.f64("t_solve", t_solve);
  w.i32("threads", std::vector<int32_t>{pr.threads});
  w.f64("tree_minmax", std::vector<double>{tree.min, tree.max});
  if (pr.dense_check) {
    std::vector<double> res;
    dense_residual(kernel, ndofs, mu, f, U, Psi, holes ? &alpha : nullptr, &res);
    w.f64("dense_residual", res);
  }
  delete keep;
  return 0;
}
