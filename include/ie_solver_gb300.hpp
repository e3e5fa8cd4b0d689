// C++ facade with the reference's interface for the factor + solve path of
// jpryan1/ie-solver, over the GB300 solver's C ABI (rskel.h).  Header-only;
// link with -lrskel.
//
// Names, argument meaning and call order follow the reference:
//   ie_solver_config      io/io.h:18-38
//   ie_Mat                ie_mat.h:19-111 (column-major owned storage)
//   Hole, Boundary        boundaries/boundary.h:11-15, 39-60 (data members)
//   Kernel                kernel/kernel.h:28-88 (construction, operator())
//   QuadTree, nodes       quadtree/quadtree.h:16-139
//   SkelFactorization     skel_factorization/skel_factorization.h:19-95
//   linear_solve, initialize_U_mat, initialize_Psi_mat, get_domain_points,
//   boundary_integral_solve                               linear_solve.h:20-35
// so a caller written against the reference compiles against this header.
// The factorization itself runs on the GPU: QuadTree owns the solver handle
// (rs_solver) that holds the tree and, after skeletonize, the factors; the
// per-node matrices of the reference (T, L, U, X_rr) stay on the device and
// are not mirrored.  Errors throw ie_solver::rs_error (the reference asserts
// or exits; it exits on a bordered system with nothing compressed,
// skel_factorization.cpp:209-212, which here is RS_ERR_NO_COMPRESSION).
// Beyond the reference: ie_solver_config carries the leaf size, proxy-point
// count and arithmetic (plain FP64, or FP32 factorization + FP64 refinement);
// the reference's compile-time defaults are the defaults here.
#ifndef IE_SOLVER_GB300_HPP_
#define IE_SOLVER_GB300_HPP_

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rskel.h"

namespace ie_solver {

struct rs_error : std::runtime_error {
  rs_status code;
  rs_error(rs_status c, const std::string& what) : std::runtime_error(what), code(c) {}
};

namespace detail {
inline void check(rs_status rc, const rs_solver* s, const char* where) {
  if (rc == RS_OK) return;
  std::string msg = std::string(where) + " failed (status " + std::to_string((int)rc) + ")";
  const char* e = rs_last_error(s);
  if (e && *e) msg += ": " + std::string(e);
  throw rs_error(rc, msg);
}
}  // namespace detail

// io/io.h:18-38, plus the reference's compile-time constants as fields.
struct ie_solver_config {
  enum Pde { LAPLACE, LAPLACE_NEUMANN, STOKES };
  int num_boundary_points = 512;
  int domain_size = 20;
  int domain_dimension = 2;
  int solution_dimension = 1;
  double id_tol = 1e-6;
  Pde pde = LAPLACE;
  bool is_strong_admissibility = false;
  int num_threads = 4;            // accepted, unused: the GPU schedules the boxes
  int max_leaf_dofs = 32;         // MAX_LEAF_DOFS (quadtree/quadtree.h:10)
  int num_proxy_points = 128;     // NUM_PROXY_POINTS (kernel/kernel.h:11)
  rs_precision precision = RS_FP64;
};

// ---------------------------------------------------------------------------
// ie_Mat: owned column-major double matrix (ie_mat.h:19-111).
// ---------------------------------------------------------------------------
struct ie_Mat {
  double* mat = nullptr;
  int lda_ = 0, height_ = 0, width_ = 0;

  ie_Mat() {}
  ie_Mat(int h, int w) : lda_(h), height_(h), width_(w) {
    if (h > 0 && w > 0) mat = new double[(size_t)h * w]();
  }
  ~ie_Mat() { delete[] mat; }
  ie_Mat(const ie_Mat& o) : ie_Mat(o.height_, o.width_) {
    for (int j = 0; j < width_; ++j)
      for (int i = 0; i < height_; ++i) set(i, j, o.get(i, j));
  }
  ie_Mat& operator=(const ie_Mat& o) {
    if (this != &o) {
      ie_Mat t(o);
      swap(t);
    }
    return *this;
  }
  ie_Mat(ie_Mat&& o) noexcept { swap(o); }
  ie_Mat& operator=(ie_Mat&& o) noexcept {
    swap(o);
    return *this;
  }
  void swap(ie_Mat& o) noexcept {
    std::swap(mat, o.mat);
    std::swap(lda_, o.lda_);
    std::swap(height_, o.height_);
    std::swap(width_, o.width_);
  }

  int height() const { return height_; }
  int width() const { return width_; }
  double get(int i, int j) const { return mat[i + (size_t)lda_ * j]; }
  void set(int i, int j, double a) { mat[i + (size_t)lda_ * j] = a; }
  void addset(int i, int j, double a) { mat[i + (size_t)lda_ * j] += a; }

  void eye(int n) {
    *this = ie_Mat(n, n);
    for (int i = 0; i < n; ++i) set(i, i, 1.0);
  }
  void transpose_into(ie_Mat* t) const {
    *t = ie_Mat(width_, height_);
    for (int j = 0; j < width_; ++j)
      for (int i = 0; i < height_; ++i) t->set(j, i, get(i, j));
  }
  ie_Mat transpose() const {
    ie_Mat t;
    transpose_into(&t);
    return t;
  }

  // A(I, J) and the range forms [s, e)
  ie_Mat operator()(const std::vector<int>& I, const std::vector<int>& J) const {
    ie_Mat out((int)I.size(), (int)J.size());
    for (size_t j = 0; j < J.size(); ++j)
      for (size_t i = 0; i < I.size(); ++i) out.set((int)i, (int)j, get(I[i], J[j]));
    return out;
  }
  ie_Mat operator()(const std::vector<int>& I, int col_s, int col_e) const {
    return (*this)(I, range(col_s, col_e));
  }
  ie_Mat operator()(int row_s, int row_e, const std::vector<int>& J) const {
    return (*this)(range(row_s, row_e), J);
  }
  ie_Mat operator()(int row_s, int row_e, int col_s, int col_e) const {
    return (*this)(range(row_s, row_e), range(col_s, col_e));
  }
  void set_submatrix(const std::vector<int>& I, const std::vector<int>& J, const ie_Mat& A,
                     bool transpose_A = false) {
    for (size_t j = 0; j < J.size(); ++j)
      for (size_t i = 0; i < I.size(); ++i)
        set(I[i], J[j], transpose_A ? A.get((int)j, (int)i) : A.get((int)i, (int)j));
  }
  void set_submatrix(int row_s, int row_e, int col_s, int col_e, const ie_Mat& A,
                     bool transpose_A = false, bool = false) {
    set_submatrix(range(row_s, row_e), range(col_s, col_e), A, transpose_A);
  }
  void set_submatrix(const std::vector<int>& I, int col_s, int col_e, const ie_Mat& A,
                     bool transpose_A = false) {
    set_submatrix(I, range(col_s, col_e), A, transpose_A);
  }
  void set_submatrix(int row_s, int row_e, const std::vector<int>& J, const ie_Mat& A,
                     bool transpose_A = false) {
    set_submatrix(range(row_s, row_e), J, A, transpose_A);
  }

  ie_Mat& operator+=(const ie_Mat& o) { return axpy(1.0, o); }
  ie_Mat& operator-=(const ie_Mat& o) { return axpy(-1.0, o); }
  ie_Mat& operator*=(double a) {
    for (int j = 0; j < width_; ++j)
      for (int i = 0; i < height_; ++i) set(i, j, a * get(i, j));
    return *this;
  }
  ie_Mat& operator/=(double a) { return *this *= 1.0 / a; }
  ie_Mat operator-() const { return *this * -1.0; }
  ie_Mat operator+(const ie_Mat& o) const { return ie_Mat(*this) += o; }
  ie_Mat operator-(const ie_Mat& o) const { return ie_Mat(*this) -= o; }
  ie_Mat operator*(double a) const { return ie_Mat(*this) *= a; }
  ie_Mat operator/(double a) const { return ie_Mat(*this) /= a; }
  ie_Mat operator*(const ie_Mat& o) const {
    if (width_ != o.height_) throw rs_error(RS_ERR_ARG, "ie_Mat product: inner sizes differ");
    ie_Mat out(height_, o.width_);
    for (int j = 0; j < o.width_; ++j)
      for (int l = 0; l < width_; ++l) {
        const double b = o.get(l, j);
        for (int i = 0; i < height_; ++i) out.addset(i, j, get(i, l) * b);
      }
    return out;
  }

  double one_norm() const {
    double best = 0;
    for (int j = 0; j < width_; ++j) {
      double s = 0;
      for (int i = 0; i < height_; ++i) s += std::fabs(get(i, j));
      best = s > best ? s : best;
    }
    return best;
  }
  double frob_norm() const {
    double s = 0;
    for (int j = 0; j < width_; ++j)
      for (int i = 0; i < height_; ++i) s += get(i, j) * get(i, j);
    return std::sqrt(s);
  }
  double vec_two_norm() const { return frob_norm(); }
  double max_entry_magnitude() const {
    double m = 0;
    for (int j = 0; j < width_; ++j)
      for (int i = 0; i < height_; ++i) m = std::fabs(get(i, j)) > m ? std::fabs(get(i, j)) : m;
    return m;
  }

 private:
  static std::vector<int> range(int s, int e) {
    std::vector<int> r;
    for (int i = s; i < e; ++i) r.push_back(i);
    return r;
  }
  ie_Mat& axpy(double a, const ie_Mat& o) {
    if (o.height_ != height_ || o.width_ != width_)
      throw rs_error(RS_ERR_ARG, "ie_Mat sum: sizes differ");
    for (int j = 0; j < width_; ++j)
      for (int i = 0; i < height_; ++i) addset(i, j, a * o.get(i, j));
    return *this;
  }
};

// ---------------------------------------------------------------------------
// Boundary data (boundaries/boundary.h).  Shapes and boundary conditions are
// the caller's: a subclass (or this class directly) fills the vectors.
// ---------------------------------------------------------------------------
struct Vec2 {
  double a[2] = {0, 0};
  Vec2() {}
  Vec2(double x, double y) { a[0] = x; a[1] = y; }
};
struct Hole {
  Vec2 center;
  double radius = 0;
  int num_nodes = 0;
};
class Boundary {
 public:
  std::vector<double> points, normals, curvatures, weights;
  std::vector<Hole> holes;
  ie_Mat boundary_values;
  virtual ~Boundary() {}
  // Which domain points boundary_integral_solve evaluates (the reference's
  // shapes override it; every point by default).
  virtual bool is_in_domain(const Vec2&) const { return true; }
};

namespace detail {
inline rs_pde to_pde(ie_solver_config::Pde p) {
  return p == ie_solver_config::STOKES ? RS_STOKES
         : p == ie_solver_config::LAPLACE_NEUMANN ? RS_LAPLACE_NEUMANN
                                                  : RS_LAPLACE;
}
// A handle for `b` with the given settings; the caller owns it.
inline rs_solver* make_handle(const Boundary& b, rs_pde pde, double id_tol, int leaf, int npp,
                              rs_precision prec) {
  rs_config c;
  rs_config_default(&c);
  c.pde = pde;
  c.solution_dimension = pde == RS_STOKES ? 2 : 1;
  c.id_tol = id_tol;
  c.max_leaf_dofs = leaf;
  c.num_proxy_points = npp;
  c.precision = prec;
  rs_solver* s = nullptr;
  check(rs_create(&c, &s), nullptr, "rs_create");
  std::vector<double> hc, hr;
  for (const Hole& h : b.holes) {
    hc.push_back(h.center.a[0]);
    hc.push_back(h.center.a[1]);
    hr.push_back(h.radius);
  }
  rs_status rc = rs_set_geometry(s, (int)b.weights.size(), b.points.data(), b.normals.data(),
                                 b.weights.data(), b.curvatures.data(), (int)b.holes.size(),
                                 hc.data(), hr.data());
  if (rc != RS_OK) {
    std::string e = rs_last_error(s);
    rs_destroy(s);
    throw rs_error(rc, "rs_set_geometry failed: " + e);
  }
  return s;
}
}  // namespace detail

// ---------------------------------------------------------------------------
// Kernel (kernel/kernel.h:28-88): dense blocks of the boundary operator.
// ---------------------------------------------------------------------------
struct Kernel {
  int solution_dimension, domain_dimension;
  ie_solver_config::Pde pde;
  Boundary* boundary;
  std::vector<double> domain_points;

  Kernel(int solution_dimension_, int domain_dimension_, ie_solver_config::Pde pde_,
         Boundary* boundary_, std::vector<double> domain_points_)
      : solution_dimension(solution_dimension_),
        domain_dimension(domain_dimension_),
        pde(pde_),
        boundary(boundary_),
        domain_points(std::move(domain_points_)) {}
  Kernel(const Kernel& o)
      : Kernel(o.solution_dimension, o.domain_dimension, o.pde, o.boundary, o.domain_points) {}
  Kernel& operator=(const Kernel&) = delete;
  ~Kernel() {
    if (h_) rs_destroy(h_);
  }

  // K(I, J) over DOF indices (kernel.cpp:105-120), evaluated on the GPU.
  ie_Mat operator()(const std::vector<int>& I, const std::vector<int>& J,
                    double* timing = nullptr) const {
    (void)timing;
    ie_Mat out((int)I.size(), (int)J.size());
    if (I.empty() || J.empty()) return out;
    rs_solver* s = handle();
    detail::check(rs_kernel_block(s, I.data(), (int)I.size(), J.data(), (int)J.size(), out.mat),
                  s, "rs_kernel_block");
    return out;
  }

 private:
  mutable rs_solver* h_ = nullptr;
  rs_solver* handle() const {
    if (!h_) h_ = detail::make_handle(*boundary, detail::to_pde(pde), 1e-6, 32, 128, RS_FP64);
    return h_;
  }
};

// ---------------------------------------------------------------------------
// QuadTree (quadtree/quadtree.h).  Nodes are host mirrors of the device
// tree: geometry, DOF lists and the skeleton bookkeeping.
// ---------------------------------------------------------------------------
struct InteractionLists {
  std::vector<int> original_box, active_box, redundant, skel, near, skelnear, permutation;
};

struct QuadTreeNode {
  int id = 0, level = 0;
  bool is_leaf = true, compressed = false;
  double side_length = 0;
  QuadTreeNode *tl = nullptr, *tr = nullptr, *bl = nullptr, *br = nullptr;
  QuadTreeNode* parent = nullptr;
  QuadTreeNode* children[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<QuadTreeNode*> neighbors;
  InteractionLists src_dof_lists, tgt_dof_lists;
  double corners[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // {BL, TL, TR, BR}
};

struct QuadTreeLevel {
  std::vector<QuadTreeNode*> nodes;
  ~QuadTreeLevel() {
    for (QuadTreeNode* n : nodes) delete n;
  }
};

class SkelFactorization;

class QuadTree {
 public:
  int solution_dimension = 1, domain_dimension = 2;
  double min = 0, max = 0;
  Boundary* boundary = nullptr;
  std::vector<double> domain_points;
  QuadTreeNode* root = nullptr;
  // The bordered system's blocks (quadtree.h:104): callers may set them as
  // the reference's tests do; the factorization builds its own on the device
  // from the boundary's holes.
  ie_Mat U, Psi;
  std::vector<QuadTreeLevel*> levels;

  QuadTree() {}
  QuadTree(const QuadTree&) = delete;
  QuadTree& operator=(const QuadTree&) = delete;
  ~QuadTree() { clear(); }

  // quadtree.cpp:39-180; the boundary is copied, as the reference does.
  void initialize_tree(Boundary* boundary_, const std::vector<double>& domain_points_,
                       int solution_dimension_, int domain_dimension_) {
    clear();
    own_ = *boundary_;
    boundary = &own_;
    domain_points = domain_points_;
    solution_dimension = solution_dimension_;
    domain_dimension = domain_dimension_;
    h_ = detail::make_handle(own_, solution_dimension == 2 ? RS_STOKES : RS_LAPLACE, 1e-6,
                             leaf_, npp_, RS_FP64);
    detail::check(rs_build_tree(h_), h_, "rs_build_tree");
    mirror();
  }
  void reset() {
    if (boundary) {
      Boundary b = own_;
      std::vector<double> d = domain_points;
      initialize_tree(&b, d, solution_dimension, domain_dimension);
    }
  }
  void reset(Boundary* boundary_) {
    initialize_tree(boundary_, domain_points, solution_dimension, domain_dimension);
  }

  // quadtree.cpp:435-801: the boundary changed locally; the tree is updated
  // and the next skeletonize refactors only the boxes near the change.
  void perturb(const Boundary& perturbed_boundary) {
    own_ = perturbed_boundary;
    std::vector<double> hc, hr;
    for (const Hole& h : own_.holes) {
      hc.push_back(h.center.a[0]);
      hc.push_back(h.center.a[1]);
      hr.push_back(h.radius);
    }
    detail::check(rs_perturb(h_, (int)own_.weights.size(), own_.points.data(),
                             own_.normals.data(), own_.weights.data(), own_.curvatures.data(),
                             (int)own_.holes.size(), hc.data(), hr.data()),
                  h_, "rs_perturb");
    mirror();
    perturbed_ = true;
  }

  rs_solver* handle() const { return h_; }
  // Leaf size and proxy-point count of the tree and its factorization.
  void set_gb300_options(int max_leaf_dofs, int num_proxy_points) {
    leaf_ = max_leaf_dofs;
    npp_ = num_proxy_points;
  }

 private:
  friend class SkelFactorization;
  Boundary own_;
  rs_solver* h_ = nullptr;
  int leaf_ = 32, npp_ = 128;
  bool perturbed_ = false;   // the handle holds a factorization to update

  void clear() {
    for (QuadTreeLevel* l : levels) delete l;
    levels.clear();
    root = nullptr;
    if (h_) rs_destroy(h_);
    h_ = nullptr;
  }
  std::vector<int> list(int node, int which) const {
    int len = 0;
    detail::check(rs_node_list(h_, node, which, nullptr, 0, &len), h_, "rs_node_list");
    std::vector<int> v(len);
    if (len) detail::check(rs_node_list(h_, node, which, v.data(), len, &len), h_, "rs_node_list");
    return v;
  }
  // Rebuilds the host mirror from the handle (level order numbering).
  void mirror() {
    for (QuadTreeLevel* l : levels) delete l;
    levels.clear();
    rs_stats st;
    detail::check(rs_get_stats(h_, &st), h_, "rs_get_stats");
    detail::check(rs_tree_bounds(h_, &min, &max), h_, "rs_tree_bounds");
    std::vector<QuadTreeNode*> all(st.num_nodes);
    std::vector<int> info((size_t)st.num_nodes * 10);
    for (int i = 0; i < st.num_nodes; ++i) {
      QuadTreeNode* nd = new QuadTreeNode();
      int* f = &info[(size_t)i * 10];
      detail::check(rs_node_info(h_, i, f, nd->corners, &nd->side_length), h_, "rs_node_info");
      nd->id = i;
      nd->level = f[0];
      nd->is_leaf = f[1] != 0;
      nd->compressed = f[7] != 0;
      InteractionLists& L = nd->src_dof_lists;
      L.original_box = list(i, 0);
      L.active_box = list(i, 1);
      L.skel = list(i, 2);
      L.redundant = list(i, 3);
      L.near = list(i, 4);
      L.permutation = list(i, 6);
      L.skelnear = L.skel;
      nd->tgt_dof_lists = L;
      while ((int)levels.size() <= nd->level) levels.push_back(new QuadTreeLevel());
      levels[nd->level]->nodes.push_back(nd);
      all[i] = nd;
    }
    for (int i = 0; i < st.num_nodes; ++i) {
      const int* f = &info[(size_t)i * 10];
      QuadTreeNode* nd = all[i];
      nd->parent = f[2] >= 0 ? all[f[2]] : nullptr;
      for (int c = 0; c < 4; ++c) nd->children[c] = f[3 + c] >= 0 ? all[f[3 + c]] : nullptr;
      nd->bl = nd->children[0];
      nd->tl = nd->children[1];
      nd->tr = nd->children[2];
      nd->br = nd->children[3];
      for (int nb : list(i, 5)) nd->neighbors.push_back(all[nb]);
    }
    root = all.empty() ? nullptr : all[0];
  }
};

// ---------------------------------------------------------------------------
// SkelFactorization (skel_factorization/skel_factorization.h:19-95)
// ---------------------------------------------------------------------------
class SkelFactorization {
 public:
  double id_tol = 1e-6, make_mat_time = 0, id_time = 0, schur_time = 0;
  int num_threads = 1;
  bool strong_admissibility = false;
  rs_precision precision = RS_FP64;

  SkelFactorization() {}
  SkelFactorization(double id_tol_, bool strong_admissibility_, int nt)
      : id_tol(id_tol_), num_threads(nt), strong_admissibility(strong_admissibility_) {}

  // skel_factorization.cpp:140-310: the factors live in tree's handle.
  void skeletonize(const Kernel& K, QuadTree* tree) {
    if (strong_admissibility)
      throw rs_error(RS_ERR_ARG, "strong admissibility is not supported");
    if (tree->perturbed_ && tree->h_) {
      // after QuadTree::perturb: keep the compressed boxes (skel_factorization.cpp:157)
      detail::check(rs_factor(tree->h_), tree->h_, "rs_factor");
      tree->perturbed_ = false;
      tree->mirror();
      return;
    }
    rs_solver* s = detail::make_handle(*tree->boundary, detail::to_pde(K.pde), id_tol,
                                       tree->leaf_, tree->npp_, precision);
    rs_status rc = rs_factor(s);
    if (rc != RS_OK) {
      std::string e = rs_last_error(s);
      rs_destroy(s);
      throw rs_error(rc, "rs_factor failed: " + e);
    }
    if (tree->h_) rs_destroy(tree->h_);
    tree->h_ = s;
    tree->mirror();
    rs_stats st;
    detail::check(rs_get_stats(s, &st), s, "rs_get_stats");
    id_time = st.id_ms * 1e-3;
    schur_time = st.decouple_ms * 1e-3;
  }

  // skel_factorization.cpp:507-592
  void solve(const QuadTree& quadtree, ie_Mat* x, const ie_Mat& b) const {
    detail::check(rs_solve(quadtree.handle(), b.mat, b.width(), x->mat, nullptr),
                  quadtree.handle(), "rs_solve");
  }
  // skel_factorization.cpp:596-777 (bordered system for holes)
  void multiply_connected_solve(const QuadTree& quadtree, ie_Mat* x, ie_Mat* alpha,
                                const ie_Mat& b) const {
    detail::check(rs_solve(quadtree.handle(), b.mat, b.width(), x->mat, alpha->mat),
                  quadtree.handle(), "rs_solve");
  }
};

// linear_solve.cpp:115-129
inline void linear_solve(const SkelFactorization& skel_factorization, const QuadTree& quadtree,
                         const ie_Mat& f, ie_Mat* mu, ie_Mat* alpha = nullptr) {
  *mu = ie_Mat((int)quadtree.boundary->weights.size() * quadtree.solution_dimension,
               f.width());
  if (alpha == nullptr) {
    skel_factorization.solve(quadtree, mu, f);
  } else {
    skel_factorization.multiply_connected_solve(quadtree, mu, alpha, f);
  }
}

// linear_solve.cpp:269-279: a size x size grid over [x_min, x_max] x
// [y_min, y_max], x outer.
inline void get_domain_points(int domain_size, std::vector<double>* points, double x_min,
                              double x_max, double y_min, double y_max) {
  for (int i = 0; i < domain_size; ++i) {
    const double x = x_min + (double)i / (domain_size - 1) * (x_max - x_min);
    for (int j = 0; j < domain_size; ++j) {
      points->push_back(x);
      points->push_back(y_min + (double)j / (domain_size - 1) * (y_max - y_min));
    }
  }
}

// linear_solve.cpp:188-266: factor, solve for the boundary's own data and
// evaluate the solution (K_domain mu + U_forward alpha) at domain_points,
// zero where boundary->is_in_domain is false.
inline ie_Mat boundary_integral_solve(const ie_solver_config& config, QuadTree* quadtree,
                                      const std::vector<double>& domain_points) {
  Boundary* boundary = quadtree->boundary;
  SkelFactorization sf(config.id_tol, config.is_strong_admissibility, config.num_threads);
  sf.precision = config.precision;
  Kernel kernel(config.solution_dimension, config.domain_dimension, config.pde, boundary,
                domain_points);
  sf.skeletonize(kernel, quadtree);
  const int nb = boundary->holes.empty() || config.pde == ie_solver_config::LAPLACE_NEUMANN
                     ? 0
                     : (config.pde == ie_solver_config::STOKES ? 3 : 1) *
                           (int)boundary->holes.size();
  ie_Mat mu, alpha(nb, 1);
  linear_solve(sf, *quadtree, boundary->boundary_values, &mu, nb ? &alpha : nullptr);
  const int nt = (int)domain_points.size() / 2;
  std::vector<unsigned char> inside(nt);
  for (int i = 0; i < nt; ++i)
    inside[i] = boundary->is_in_domain(Vec2(domain_points[2 * i], domain_points[2 * i + 1]));
  ie_Mat out(nt * config.solution_dimension, 1);
  detail::check(rs_domain_eval(quadtree->handle(), nt, domain_points.data(), inside.data(),
                               mu.mat, nb ? alpha.mat : nullptr, 1, out.mat),
                quadtree->handle(), "rs_domain_eval");
  return out;
}

// linear_solve.cpp:20-64: U, the hole columns of the bordered operator.
// Laplace: U(i, h) = log|x_i - c_h|.  Stokes: per hole a Stokeslet pair and
// a rotlet, 1/(4 pi) (log(1/r) I + r r^T / r^2) and (r_y, -r_x) / (4 pi r^2).
inline ie_Mat initialize_U_mat(const ie_solver_config::Pde pde, const std::vector<Hole>& holes,
                               const std::vector<double>& tgt_points) {
  const int n = (int)tgt_points.size() / 2, H = (int)holes.size();
  const double pi = 3.14159265358979323846;
  if (pde != ie_solver_config::STOKES) {
    ie_Mat U(n, H);
    for (int h = 0; h < H; ++h)
      for (int i = 0; i < n; ++i) {
        const double dx = tgt_points[2 * i] - holes[h].center.a[0];
        const double dy = tgt_points[2 * i + 1] - holes[h].center.a[1];
        U.set(i, h, std::log(std::sqrt(dx * dx + dy * dy)));
      }
    return U;
  }
  ie_Mat U(2 * n, 3 * H);
  for (int h = 0; h < H; ++h)
    for (int i = 0; i < n; ++i) {
      const double rx = tgt_points[2 * i] - holes[h].center.a[0];
      const double ry = tgt_points[2 * i + 1] - holes[h].center.a[1];
      const double r2 = rx * rx + ry * ry, lg = std::log(1.0 / std::sqrt(r2));
      const double s = 1.0 / (4.0 * pi);
      U.set(2 * i, 3 * h, s * (lg + rx * rx / r2));
      U.set(2 * i + 1, 3 * h, s * (rx * ry / r2));
      U.set(2 * i, 3 * h + 1, s * (rx * ry / r2));
      U.set(2 * i + 1, 3 * h + 1, s * (lg + ry * ry / r2));
      U.set(2 * i, 3 * h + 2, ry * (s / r2));
      U.set(2 * i + 1, 3 * h + 2, -rx * (s / r2));
    }
  return U;
}

// linear_solve.cpp:67-112: Psi, the hole rows: per hole the quadrature
// weights of its own boundary points (Laplace), plus for Stokes the row
// w (y, -x) in absolute coordinates.  A point belongs to the first hole
// whose centre lies within that hole's radius (plus 1e-8) of it.
inline ie_Mat initialize_Psi_mat(const ie_solver_config::Pde pde, const std::vector<Hole>& holes,
                                 Boundary* boundary) {
  const int n = (int)boundary->weights.size(), H = (int)holes.size();
  auto on_hole = [&](int i, int h) {
    const double dx = boundary->points[2 * i] - holes[h].center.a[0];
    const double dy = boundary->points[2 * i + 1] - holes[h].center.a[1];
    return std::sqrt(dx * dx + dy * dy) < holes[h].radius + 1e-8;
  };
  if (pde != ie_solver_config::STOKES) {
    ie_Mat Psi(H, n);
    for (int i = 0; i < n; ++i)
      for (int h = 0; h < H; ++h)
        if (on_hole(i, h)) {
          Psi.set(h, i, boundary->weights[i]);
          break;
        }
    return Psi;
  }
  ie_Mat Psi(3 * H, 2 * n);
  for (int i = 0; i < n; ++i)
    for (int h = 0; h < H; ++h)
      if (on_hole(i, h)) {
        const double w = boundary->weights[i];
        Psi.set(3 * h, 2 * i, w);
        Psi.set(3 * h + 1, 2 * i + 1, w);
        Psi.set(3 * h + 2, 2 * i, w * boundary->points[2 * i + 1]);
        Psi.set(3 * h + 2, 2 * i + 1, -w * boundary->points[2 * i]);
        break;
      }
  return Psi;
}

}  // namespace ie_solver

#endif  // IE_SOLVER_GB300_HPP_
