/* CPU restatement of the reference recursive-skeletonization solver
 * (jpryan1/ie-solver), used ONLY as a checker: by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  It is never
 * linked into or called by the product library.
 *
 * Pinned against the reference itself: tests/test_oracle_pin.py compares its
 * quadtrees (bit-exact), per-box ranks and solutions with the reference built
 * from its own sources (oracle/_ref, via oracle/ref_dump.cpp) and with the
 * committed golden fixtures in tests/golden/.
 *
 * Every routine cites the reference file:line it restates.  All arithmetic is
 * IEEE double with floating-point contraction disabled (-ffp-contract=off),
 * so results are identical on x86-64 and aarch64 hosts.
 */
#ifndef RS_ORACLE_H
#define RS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

#define ORC_LAPLACE 0
#define ORC_LAPLACE_NEUMANN 1
#define ORC_STOKES 2

typedef struct orc_solver orc_solver;

/* Copies the boundary data.  points/normals interleaved (2n), weights and
 * curvatures (n), hole centres interleaved (2h) and radii (h). */
orc_solver* orc_create(int pde, int sd, int n, const double* points, const double* normals,
                       const double* weights, const double* curvatures, int num_holes,
                       const double* hole_centers, const double* hole_radii, double id_tol,
                       int max_leaf_dofs, int num_proxy_points, int num_threads);
void orc_destroy(orc_solver* s);

/* quadtree.cpp:39-180 (no domain points). */
int orc_build_tree(orc_solver* s);
/* skel_factorization.cpp:140-310 (weak admissibility).  Returns 0 on success. */
int orc_factor(orc_solver* s);
/* skel_factorization.cpp:507-592 (no holes, nrhs columns) or :596-777
 * (holes, single RHS).  f and mu are (n*sd) x nrhs column major; alpha gets
 * 3h (Stokes) or h (Laplace) values when holes exist. */
int orc_solve(orc_solver* s, const double* f, int nrhs, double* mu, double* alpha);

/* Introspection (valid after orc_build_tree / orc_factor). */
int orc_num_levels(const orc_solver* s);
int orc_num_nodes(const orc_solver* s);
/* Nodes are numbered in level order (level 0 first, then each level's node
 * list in order), the same numbering oracle/ref_dump.cpp writes.  info gets
 * {level, is_leaf, parent, child0..3, compressed, num_skel, num_redundant}. */
void orc_node_info(const orc_solver* s, int node, int* info, double* corners8, double* side);
/* which: 0 original_box, 1 active_box, 2 skel, 3 redundant, 4 near,
 *        5 neighbors (node numbers), 6 permutation.
 * Returns the list length; copies up to cap entries into out. */
int orc_node_list(const orc_solver* s, int node, int which, int* out, int cap);
int orc_allskel(const orc_solver* s, int* out, int cap);
double orc_tree_min(const orc_solver* s);
double orc_tree_max(const orc_solver* s);
/* Factor blocks of a compressed node: T (k x r), L (k x r), U (r x k),
 * X_rr (r x r, before LU), schur update (k x k), all column major. */
int orc_node_factors(const orc_solver* s, int node, double* T, double* L, double* U,
                     double* Xrr, double* schur);

/* Stand-alone pieces. */
/* kernel.cpp:105-290: dense block K(I, J), column major |I| x |J|. */
void orc_kernel_block(const orc_solver* s, const int* I, int nI, const int* J, int nJ,
                      double* out);
/* kernel.cpp:293-423: the ID matrix of a node as the reference builds it at
 * compression time; returns rows m (copies up to cap entries). */
int orc_id_matrix(const orc_solver* s, int node, double* out, long cap, int* n_out);
/* ie_mat.cpp:548-588 (dgeqp3 + rank scan + dtrtrs): A is m x n column major
 * (not modified).  Returns the rank k (0 = no compression); perm gets n
 * 0-based column indices, Z gets k x (n-k) column major, rdiag gets the n
 * diagonal entries of R. */
int orc_id(const double* A, int m, int n, double tol, int* perm, double* Z, double* rdiag);
/* y = K x over all DOFs (dense, OpenMP), x and y are (n*sd) x nrhs. */
void orc_matvec(const orc_solver* s, const double* x, int nrhs, double* y);
/* U (n*sd x 3h or h) and Psi (3h or h x n*sd), linear_solve.cpp:20-112. */
int orc_border_dims(const orc_solver* s);
void orc_border_mats(const orc_solver* s, double* U, double* Psi);

/* Wall-clock seconds of the last orc_factor / orc_solve. */
double orc_last_factor_seconds(const orc_solver* s);
double orc_last_solve_seconds(const orc_solver* s);

#ifdef __cplusplus
}
#endif
#endif
