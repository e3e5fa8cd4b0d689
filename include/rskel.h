/* rskel: GB300-native recursive-skeletonization direct solver for 2D Laplace
 * and Stokes double-layer boundary integral equations.  C ABI.
 *
 * This is the drop-in boundary for the factor + solve path of jpryan1/ie-solver.
 * Each entry point replaces the reference interface cited beside it (paths
 * within that project).  All entry points return an rs_status (0 = success);
 * no call exits the process or asserts.  Pointers are plain host pointers
 * unless an argument is documented as a device pointer.  A handle owns one
 * CUDA stream; a handle is not thread-safe, distinct handles are independent.
 */
#ifndef RSKEL_H
#define RSKEL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  RS_OK = 0,
  RS_ERR_ARG = 1,          /* invalid argument (null pointer, bad size, bad enum) */
  RS_ERR_STATE = 2,        /* call out of order (e.g. solve before factor) */
  RS_ERR_CUDA = 3,         /* a CUDA runtime call failed; see rs_last_error */
  RS_ERR_NO_DEVICE = 4,    /* no usable GPU; there is no CPU fallback */
  RS_ERR_CAPACITY = 5,     /* a box exceeded the supported block size */
  RS_ERR_NUMERIC = 6,      /* non-finite value or exactly singular pivot */
  RS_ERR_NO_COMPRESSION = 7 /* bordered system with no redundant DOFs
                               (skel_factorization.cpp:209-212 exits there) */
} rs_status;

/* ie_solver_config::Pde (io/io.h:20-24). */
typedef enum { RS_LAPLACE = 0, RS_LAPLACE_NEUMANN = 1, RS_STOKES = 2 } rs_pde;

/* Arithmetic of the factorization. */
typedef enum {
  RS_FP64 = 0,        /* plain FP64, the reference's arithmetic */
  RS_FP32_REFINE = 1  /* FP32 factorization + FP64 iterative refinement */
} rs_precision;

/* ie_solver_config (io/io.h:18-38) plus the compile-time constants of the
 * reference made runtime fields: MAX_LEAF_DOFS (quadtree/quadtree.h:10),
 * NUM_PROXY_POINTS and RADIUS_RATIO (kernel/kernel.h:11-12),
 * MIN_DOFS_TO_COMPRESS (skel_factorization/skel_factorization.h:11). */
typedef struct {
  int pde;                   /* rs_pde */
  int solution_dimension;    /* 1 (Laplace) or 2 (Stokes) */
  int domain_dimension;      /* must be 2 */
  double id_tol;             /* ID tolerance, > 0 */
  int max_leaf_dofs;         /* reference default 32 */
  int num_proxy_points;      /* reference default 128 */
  double radius_ratio;       /* reference default 1.5 */
  int min_dofs_to_compress;  /* reference default 16 */
  int is_strong_admissibility; /* must be 0 (weak admissibility only) */
  int precision;             /* rs_precision */
  double refine_tol;         /* RS_FP32_REFINE: target relative residual */
  int refine_max_iters;      /* RS_FP32_REFINE: maximum refinement steps */
  double fp32_id_tol;        /* RS_FP32_REFINE: ID tolerance of the FP32 factor
                                (at least id_tol; FP32 cannot resolve below ~1e-6) */
  int device;                /* CUDA device ordinal */
  int fmm_order;             /* RS_FP32_REFINE, Laplace: multipole order of the
                                FP64 residual, 2..64 (0 = matched to refine_tol:
                                28 at 1e-11, 31 at 1e-12) */
  double rank_headroom;      /* rank model (rs_set_rank_model): sketch rows
                                ell = ceil(rank_headroom * k_pred) + rank_extra_rows,
                                default 1.25 and 12 */
  int rank_extra_rows;
  int refine_verify;         /* RS_FP32_REFINE: convergence of the residual recurrence
                                (FP32 products of corrections) is confirmed by a fresh
                                float-float residual, refinement going on while that is
                                above refine_tol: 1 (default) = when the recurrence's error
                                bound (the FP32 products' error times the residuals they
                                multiplied, summed) could take it above refine_tol;
                                2 = always; 0 = never */
  int refine_solver;         /* RS_FP32_REFINE correction equation: 0 (default) = one
                                application of the FP32 factorization per step, switching to
                                GMRES-IR when a step cuts the residual by less than 10x;
                                1 = always the former; 2 = always GMRES-IR (flexible GMRES
                                preconditioned by the FP32 factorization, FP32 multipole
                                products, up to 31 steps per refinement step) */
  int use_graphs;            /* 1 (default): the factorization's inverse (no holes) runs as
                                one CUDA graph launch, captured on first use after each
                                rs_factor; 0: plain launches */
  int root_inverse;          /* RS_FP32_REFINE, root blocks of at most 128 DOFs: 1 (default)
                                = inverted once per factorization (Gauss-Jordan with partial
                                pivoting), one product per application; 0 = LU with partial
                                pivoting and triangular solves (dgetrf/dgetrs, as FP64 and
                                larger roots always do) */
  double rank_judge;         /* rank model: residual judge of the truncated sketches.  A box
                                sketched with the predicted ell rows also forms 8 test rows
                                with independent signs; its ID is redone with the full sketch
                                when the residual they estimate, for any redundant column,
                                exceeds rank_judge * id_tol * (the largest column norm).
                                Default 4; 0 = off (only the rank-settling rule judges) */
  int tensor_cores;          /* RS_FP32_REFINE: 1 (default) = the FP32 randomized ID's sketch
                                Y = Omega A runs on the tensor cores (tcgen05.mma, BF16
                                operands with A split in three BF16 parts, FP32 accumulation
                                in tensor memory); 0 = on the CUDA cores (FP32 FMA) */
  int id_row_groups;         /* RS_FP32_REFINE, levels with fewer ID boxes than SMs: each
                                box's ID matrix rows (its 64-row chunks, round robin) are
                                sketched by this many CTAs, whose partial sketches the pivoted
                                QR sums in a fixed order.  -1 (default) = about two CTAs per
                                SM over the level, at most one per chunk and 16 per box;
                                0 or 1 = one CTA per box; 2..16 = that many */
  int fmm_order32;           /* RS_FP32_REFINE: multipole order of the FP32 products of
                                refinement corrections.  0 (default) = chosen per correction
                                from the accuracy it needs: the product's error, about
                                10^(-0.36 p) relative to the correction, times the residual the
                                correction came from, is kept below a quarter of what the
                                residual recurrence's error bound has left of refine_tol / 2
                                (and never asked below what order 16 gives), so the later,
                                smaller corrections take orders down to 4; GMRES-IR's products
                                stay at 16.  2..16 = that order for every FP32 product */
} rs_config;

typedef struct rs_solver rs_solver;

/* Fills cfg with the reference defaults (io/io.h:11-14, 18-38). */
void rs_config_default(rs_config* cfg);

/* SkelFactorization(double id_tol, bool strong, int nt)
 * (skel_factorization/skel_factorization.cpp:26-32) + Kernel(...)
 * (kernel/kernel.h:28-35). */
rs_status rs_create(const rs_config* cfg, rs_solver** out);
rs_status rs_destroy(rs_solver* s);

/* Boundary data vectors (boundaries/boundary.h:39-41): points and normals
 * interleaved (2*num_points), weights and curvatures (num_points).  Holes
 * (boundaries/boundary.h:11-15) are optional: centres interleaved (2*h) and
 * radii (h).  The data are copied. */
rs_status rs_set_geometry(rs_solver* s, int num_points, const double* points,
                          const double* normals, const double* weights,
                          const double* curvatures, int num_holes,
                          const double* hole_centers, const double* hole_radii);

/* A batch of independent boundaries without holes in one handle (no
 * reference counterpart; the reference solves one boundary per
 * SkelFactorization).  Boundary t has num_points[t] points; the arrays are
 * the boundaries' data vectors concatenated in order, and right-hand sides
 * and solutions are concatenated the same way (column of length
 * sum(num_points) * sd).  rs_build_tree builds one quadtree per boundary
 * and merges them into a forest: every tree level of every boundary is
 * factored in the same launches, and each boundary keeps its own root
 * block.  Refinement residuals are judged per boundary and column.
 * Not available for a batch: holes, rs_perturb, rs_matvec (dense),
 * rs_domain_eval, and RS_FP32_REFINE with other kernels than RS_LAPLACE. */
rs_status rs_set_geometry_batch(rs_solver* s, int count, const int* num_points,
                                const double* points, const double* normals,
                                const double* weights, const double* curvatures);

/* QuadTree::initialize_tree(boundary, {}, sd, 2) (quadtree/quadtree.cpp:39-180).
 * Host-side; needs no GPU. */
rs_status rs_build_tree(rs_solver* s);

/* QuadTree::perturb (quadtree/quadtree.cpp:435-801): the boundary changed
 * (points matched to the old ones by exact coordinates).  The tree is
 * updated in place, and the next rs_factor refactors only the boxes whose
 * neighbourhood changed, keeping the others' factors, as skeletonize does
 * after perturb (skel_factorization.cpp:157).  Arguments as rs_set_geometry;
 * before rs_build_tree it is rs_set_geometry.  Host-side; needs no GPU. */
rs_status rs_perturb(rs_solver* s, int num_points, const double* points,
                     const double* normals, const double* weights,
                     const double* curvatures, int num_holes,
                     const double* hole_centers, const double* hole_radii);

/* SkelFactorization::skeletonize (skel_factorization.cpp:140-310), including
 * the bordered system for holes (initialize_U_mat / initialize_Psi_mat,
 * linear_solve.cpp:20-112).  Builds the tree first when needed. */
rs_status rs_factor(rs_solver* s);

/* linear_solve (linear_solve.cpp:115-129) -> SkelFactorization::solve
 * (skel_factorization.cpp:507-592) or multiply_connected_solve (:596-777).
 * f and mu: (num_points*sd) x nrhs, column major, host memory.  alpha:
 * (3h Stokes, h Laplace) x nrhs when holes exist, else may be NULL. */
rs_status rs_solve(rs_solver* s, const double* f, int nrhs, double* mu, double* alpha);

/* Same as rs_solve with device pointers (no host copies); work is ordered on
 * the handle's stream and the call returns without synchronising. */
rs_status rs_solve_device(rs_solver* s, const double* d_f, int nrhs, double* d_mu,
                          double* d_alpha);

/* Kernel::operator()(I, J) (kernel/kernel.cpp:105-120): dense block
 * K(I, J), column major |I| x |J|, evaluated on the GPU. */
rs_status rs_kernel_block(rs_solver* s, const int* I, int nI, const int* J, int nJ,
                          double* out);

/* y = K x over all DOFs (dense, FP64 accurate, on the GPU), the operator whose
 * inverse the factorization represents.  x, y: (num_points*sd) x nrhs. */
rs_status rs_matvec(rs_solver* s, const double* x, int nrhs, double* y);

/* y = K x through the fast multipole method used by the refinement (Laplace,
 * Laplace-Neumann and Stokes operators as rs_kernel_block defines them).
 * arith = 0: FP64; 2: float-float
 * (pairs of floats, ~48-bit significands, on the FP32 pipes), the variant of
 * the refinement's full residual; both at order rs_config.fmm_order.
 * arith = 1: the FP32 variant used for products with refinement corrections
 * (~1e-7 relative at order 16; at rs_config.fmm_order32 when that is set).  No reference counterpart: the reference applies K only
 * densely in its tests (ie_solver_test.cpp:87-95). */
rs_status rs_matvec_fast(rs_solver* s, const double* x, int nrhs, double* y, int arith);

/* The solution at points off the boundary, as boundary_integral_solve
 * assembles it (linear_solve.cpp:188-266, schur_solve 140-154):
 * u = K_domain mu + U_forward alpha, with K_domain from
 * Initialization::InitializeDomainKernel (initialization.cpp:11-135) and
 * U_forward = initialize_U_mat at the targets (linear_solve.cpp:20-64).
 * targets: interleaved (2*num_targets); in_domain: per-target flags
 * (Boundary::is_in_domain in the reference; targets flagged 0 get 0), or
 * NULL for all inside; mu: (num_points*sd) x nrhs; alpha: the hole unknowns
 * from rs_solve (NULL without holes); out: (num_targets*sd) x nrhs.  Host
 * memory, column major.  Evaluated directly in FP64 on the GPU. */
rs_status rs_domain_eval(rs_solver* s, int num_targets, const double* targets,
                         const unsigned char* in_domain, const double* mu, const double* alpha,
                         int nrhs, double* out);

/* ie_Mat::id (ie_mat.cpp:548-588) for a batch of matrices on the GPU.
 * mats: concatenated column-major m_i x n_i blocks (offsets a_off, in
 * doubles); ranks[i] gets k (0 = no compression); perm gets n_i 0-based
 * column indices at p_off[i]; Z gets k x (n_i - k) at z_off[i] (caller
 * reserves n_i*n_i doubles). */
rs_status rs_id_batched(rs_solver* s, int count, const double* mats, const int64_t* a_off,
                        const int* m, const int* n, double tol, int* ranks, int* perm,
                        const int64_t* p_off, double* Z, const int64_t* z_off);

/* One FP64 ID of a device-resident column-major m x n matrix A (lda = m) on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) of the current
 * device, with no device allocation.  No counterpart in the reference: it is
 * rs_id_batched's kernel with its global scratch tile taken from a fixed
 * 4 MiB file-scope device array instead of cudaMalloc.  It is meant for
 * callers that cannot allocate device memory: a process whose device memory
 * is owned by another caching allocator (PyTorch's, for instance), or a
 * stream pipeline that cannot take cudaMalloc/cudaFree's implicit device
 * synchronisation.  The array stays resident on every device that loads the
 * library until the process exits.
 * Outputs (device pointers): *rank = k (0 = no compression), perm = n
 * 0-based column indices, Z = k x (n - k) column major (reserve n*n/4 + 1
 * doubles).  Asynchronous: results are ready when `stream` is.
 * Limits: the padded tile, ceil(m/64)*64 * (n + 32) + ceil(m/64)*64 + 64
 * doubles, must fit in 524288 doubles (for example m = 2048 with n <= 222,
 * or m = 1024 with n <= 478), and the kernel's shared memory must fit in
 * 227 KB; larger sizes return RS_ERR_CAPACITY without touching the device.
 * The first call on a device sets up the device (symbol addresses and the
 * kernel's shared-memory attribute): make it before any stream capture.
 * The set-up is kept for the life of the process: after a cudaDeviceReset
 * of a device, do not call this entry point on that device again.
 * All calls on a device share the scratch array: calls that overlap in time
 * race and must be serialised by the caller.  Nothing needs to start at
 * zero.  A CUDA error already pending in the calling thread is returned as
 * RS_ERR_CUDA (and left pending) without launching anything. */
rs_status rs_id_noalloc(int m, int n, const double* A, double tol, int* rank, int* perm,
                        double* Z, void* stream);

/* Self-test of the bounded grid barrier that the cooperative kernels (the
 * bordered system's S inverse) synchronise with.  No counterpart in the
 * reference, which has no GPU code.  Runs `rounds` (1..64) grid barriers on
 * `device` over one CTA per SM, each wait limited to `spins` polls (at most
 * the production limit of 2^22).  CTA `skip_block` (-1: none) leaves
 * without arriving, so the other CTAs' waits run out: they raise the error
 * flag and return, the way a barrier timeout surfaces in rs_factor as
 * RS_ERR_CUDA "grid barrier timed out", with the context still usable.
 * Outputs: *err = the flag (0 or 1), the fewest and most barriers passed by
 * the CTAs that ran them, and the kernel's device time in ms.  Allocates a
 * few bytes of device memory per call. */
rs_status rs_barrier_selftest(int device, int skip_block, unsigned spins, int rounds, int* err,
                              int* passed_min, int* passed_max, float* ms);

/* --- learned skeleton ranks (the RS_FP32_REFINE factorization's ID) ---
 * No counterpart in the reference.  A 16 -> 64 -> 64 -> 1 multilayer
 * perceptron (ReLU, ReLU, sigmoid) predicts each box's rank fraction k/n
 * from RS_RANK_FEATURES features the host computes per box (ID matrix
 * sizes, tree level and box size, tolerance, kernel, curvature and spread
 * of the box's boundary piece).  The FP32 randomized ID of a box of at most
 * 128 DOFs then sketches with ell = min(n + 16, ceil(h ceil(n y)) + e) rows (h = rank_headroom, e =
 * rank_extra_rows of rs_config)
 * instead of n + 16.  A box whose truncated sketch does not settle its rank
 * with 8 rows to spare is redone on the device with the full sketch, so a
 * poor prediction costs time, not accuracy.
 * Weights: W1 (64 x 16, row major), b1 (64), W2 (64 x 64), b2 (64), w3 (64),
 * b3 (1), RS_RANK_WEIGHTS floats in all. */
#define RS_RANK_FEATURES 16
#define RS_RANK_WEIGHTS 5313
/* Deterministic initial weights (He-scaled uniform, host only). */
void rs_rank_model_init(uint64_t seed, float* weights);
/* Uses `weights` (host, copied) for this handle's RS_FP32_REFINE
 * factorizations from the next rs_factor on; NULL switches it off. */
rs_status rs_set_rank_model(rs_solver* s, const float* weights);
/* Training samples of the last rs_factor: per box that was tried for
 * compression, its features (row major, RS_RANK_FEATURES per box) and the
 * rank fraction it got (k/n; 1 when not compressed).  Writes up to cap
 * samples; *count gets the number available. */
rs_status rs_rank_samples(const rs_solver* s, float* features, float* targets, int cap,
                          int* count);
/* `epochs` full-batch Adam steps (lr; betas 0.9, 0.999) on the mean squared
 * error of the predicted fractions, on the handle's device.  weights: host,
 * in and out; *loss gets the mean loss at the last step's weights before
 * its update. */
rs_status rs_rank_train(rs_solver* s, const float* features, const float* targets, int count,
                        int epochs, float lr, float* weights, float* loss);
/* The inference kernel's fractions, and the gradient kernel's d(loss)/dW
 * with the mean loss (host arrays). */
rs_status rs_rank_predict(rs_solver* s, const float* weights, const float* features, int count,
                          float* out);
rs_status rs_rank_gradient(rs_solver* s, const float* weights, const float* features,
                           const float* targets, int count, float* grad, float* loss);

/* Autotuner (no reference counterpart): times factorizations of the
 * handle's current geometry (RS_FP32_REFINE: each with one refined solve of
 * eight columns of point-source potentials from outside the geometry, since
 * the launch shapes change the factorization's rounding and so the solve's
 * refinement steps) over the launch shapes that
 * depend on the problem and keeps the fastest for this handle's later
 * factorizations:
 * the level size from which the FP32 sketched ID's pivoted QR runs one
 * warp per box instead of one CTA per box (128, 256, 512 (default), 1024,
 * never), then the wide ID's CTAs per SM (1, 2 (default), 4), then the
 * threads per box of the Schur eliminations (0 (default): per level, 128
 * when one wave of 256-thread CTAs does not hold the level's boxes, else
 * 256; or 256 or 128 for every level).  Each candidate is the median
 * of `reps` factorizations.  The choices are returned (pointers may be
 * NULL).  The handle must be factored again before solving. */
rs_status rs_autotune(rs_solver* s, int reps, int* split_min_tasks, int* wide_ctas_per_sm,
                      int* elim_threads);

/* --- introspection (tree and factorization), for tests and tooling --- */
typedef struct {
  int num_levels, num_nodes, num_compressed, num_skel_root;
  int max_active, max_rank, max_rows;
  double t_tree_ms, t_factor_ms, t_solve_ms;   /* host wall clock of last calls */
  double dev_factor_ms, dev_solve_ms;          /* CUDA-event time of last calls */
  double id_flops, decouple_flops, solve_bytes; /* algorithmic work of last calls */
  double id_ms, decouple_ms;                   /* CUDA-event time in those kernels */
  int refine_iters;                            /* iterations of last solve */
  double refine_residual;                      /* final relative residual */
  int kernel_launches;                         /* kernels launched by last factor+solve */
  double host_plan_ms, host_wait_ms, host_post_ms; /* last factor: host list building and
                                                      launches, waiting for ranks, and
                                                      bookkeeping after them */
  int boxes_factored;                          /* boxes compressed by the last rs_factor */
  double residual64_ms, residual32_ms;         /* last RS_FP32_REFINE solve: CUDA-event time of
                                                  the FP64 residual products and of the FP32
                                                  correction products */
  int rank_predicted, rank_redo;               /* last rs_factor with a rank model: boxes whose
                                                  sketch size was predicted, and those of them
                                                  redone with the full sketch */
  double sketch_rows;                          /* last RS_FP32_REFINE rs_factor: rows of the
                                                  randomized-ID sketches of boxes of <= 512 DOFs,
                                                  summed (a redone box counts both sketches) */
  int krylov_steps;                            /* last solve: GMRES steps of GMRES-IR */
  int rank_redo_judge;                         /* of rank_redo: boxes whose sketch settled the
                                                  rank but failed the residual judge */
  double level_gap_ms;                         /* last rs_factor: device time between one
                                                  level's last kernel and the next level's
                                                  first, summed (the device waiting for the
                                                  host's planning of the next level) */
} rs_stats;
rs_status rs_get_stats(const rs_solver* s, rs_stats* out);

/* Node numbering is level order (QuadTree::levels, quadtree.h:107): level 0,
 * then each level's node list in order.  info gets {level, is_leaf, parent,
 * child0..child3 (bl, tl, tr, br), compressed, num_skel, num_redundant}. */
rs_status rs_node_info(const rs_solver* s, int node, int* info, double* corners8,
                       double* side);
/* which: 0 original_box, 1 active_box, 2 skel, 3 redundant, 4 near,
 * 5 neighbors (node numbers), 6 permutation (InteractionLists, quadtree.h:16-49).
 * Writes up to cap entries; *len gets the full length. */
rs_status rs_node_list(const rs_solver* s, int node, int which, int* out, int cap, int* len);
rs_status rs_tree_bounds(const rs_solver* s, double* min_coord, double* max_coord);
rs_status rs_allskel(const rs_solver* s, int* out, int cap, int* len);

/* Device-event timing on the handle's stream, for benchmarks. */
rs_status rs_timer_start(rs_solver* s);
rs_status rs_timer_stop(rs_solver* s, float* ms);
rs_status rs_synchronize(rs_solver* s);

/* Last error message of this handle (static storage for NULL handles). */
const char* rs_last_error(const rs_solver* s);

#ifdef __cplusplus
}
#endif
#endif
