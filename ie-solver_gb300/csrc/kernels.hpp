// Launch interfaces of the CUDA kernels (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "plan.hpp"

namespace rskel {

struct IdParams {
  Geo<double> geo;
  int pde, sd, npp;
  double tol;
  const IdTask* tasks;
  const int* dofs;
  const double* pxy_cos;
  const double* pxy_sin;
  int* ranks;      // per slot
  int* perm;       // written at act_off (n entries per task)
  void* fac;       // T output (Real)
  void* scratch;   // global tiles for large boxes (Real)
  const double* dense;  // matrices for rs_id_batched (column major)
  long long* phase_clk; // optional: per-task cycle counts {fill, fold, cpqr, z} (trace mode)
  int direct;           // 1: pivoted QR on the whole matrix in the task's global tile
  float* sketch_y;      // FP32 randomized ID in two kernels: sketch, then warp-per-box QR
  // Learned sketch sizes (IdTask::ell): per-slot flags set by a box whose
  // truncated sketch could not settle its rank, and the second pass that
  // redoes exactly those boxes with the full n + 16 rows.  nullptr: no
  // learned sizes in this launch.
  int* redo;
  int redo_pass;
  // Residual judge of a learned pass (redo != nullptr, redo_pass == 0): a
  // truncated sketch also forms kIdTestRows test rows with independent
  // signs, and a box whose estimated interpolation residual (per redundant
  // column, from the test rows) exceeds judge_factor * tol * (the largest
  // column norm of its ID matrix) is redone (flag 2).  judge_factor <= 0:
  // no test rows.  judge_ratio (optional, per slot, filled with NaN by the
  // caller): the judged boxes' worst estimate over tol * that norm.
  float judge_factor;
  float* judge_ratio;
  // FP32 sketched ID: 1 = the sketch on the tensor cores (tcgen05), 0 = on
  // the CUDA cores.  status: raised when a tensor-core wait gave up.
  int tc;
  int* status;
  // FP32 sketched ID: levels of at least this many boxes run the pivoted QR
  // one warp per box (id_cpqr_warp_kernel), smaller ones one CTA per box
  int split_min_tasks;
  // FP32 sketched ID of a level of few boxes: row_groups >= 2 splits each
  // box's ID matrix rows (its 64-row chunks, round robin) over that many
  // CTAs, each writing a partial sketch at sketch_y + y_off + g *
  // y_group_stride; the CTA-per-box QR then sums the y_parts partial
  // sketches in order instead of forming the sketch itself.
  int row_groups;
  int y_parts;
  int64_t y_group_stride;
};

struct DecoupleParams {
  Geo<double> geo;
  int pde, sd;
  const DecoupleTask* tasks;
  const int* dofs;
  const int* ranks;
  const int* perm;
  void* fac;       // T in, L/U/X_rr LU out (Real)
  int* piv;
  void* epool;     // E blocks in/out (Real)
  void* scratch;
  int* status;     // non-zero on singular pivot / non-finite value
  // trace only (else null): per box of the launch, clock cycles of the
  // assembly, the T products, the X_rr inverse or LU and the rest, then n, k
  long long* phase_clk;
};

// Sweep modes (solve_kernels.cu).
enum SweepMode : int {
  kUpSolve = 0,   // x_r -= T^T x_s; x_s -= L x_r; x_r = X_rr^{-1} x_r
  kUpPlain = 1,   // x_r -= T^T x_s; x_s -= L x_r
  kUpTransU = 2,  // x_r -= T^T x_s; x_s -= U^T x_r
  kDiagOnly = 3,  // x_r = X_rr^{-1} x_r
  kDown = 4       // x_r -= U x_s; x_s -= T x_r
};

struct SweepParams {
  const SweepTask* tasks;
  const int* dofs;
  const void* fac;  // Real
  const int* piv;
  void* x;          // Real, D x nrhs, column major
  int ld, nrhs;
  int mode;
  int stage_fac;    // set by launch_sweep: each box's factor record staged in shared memory
};

size_t id_kernel_smem(int n, bool fp32, bool tile_in_smem);
// Doubles of global tile a direct-QR task with m rows and n columns needs.
size_t id_direct_tile(int m, int n);
size_t decouple_kernel_smem(int n, bool fp32, bool tile_in_smem);

// Floats of sketch storage one FP32 task of n columns needs (split ID).
size_t id_sketch_y_size(int n);
constexpr int kIdTestRows = 8;  // test rows of the residual judge
// Shared-memory attribute set-up of the FP64 ID kernels on the current device.
cudaError_t id_noalloc_prepare();
int launch_id(const IdParams& p, int num_tasks, int nmax, size_t smem, bool fp32,
               cudaStream_t st);
// FP32 wide ID of num_tasks tasks (all of more than 128 columns; tasks with
// m_dense > 0 are sketched through `items` into `part`, the others factor
// their ID matrix directly): partial sketches, their sum into each task's
// scratch tile, then pivoted QR and Z.  Returns the kernels launched.
int launch_id_wide(const IdParams& p, int num_tasks, int nmax, const WideItem* items,
                   int num_items, float* part, cudaStream_t st);
size_t id_wide_tile(int m, int n);  // scratch floats of a wide task (m: rows factored)
int id_sketch_rows(int n);
void launch_decouple(const DecoupleParams& p, int num_tasks, size_t smem, bool fp32,
                     cudaStream_t st, int threads, int num_sms);
void launch_sweep(const SweepParams& p, int num_tasks, int nmax, bool fp32, cudaStream_t st);

// Dense LU with partial pivoting of an n x n column-major matrix (one CTA),
// and the corresponding solve on gathered rows of x.
// A forest's root blocks: E block at base[a_off] (n x n), pivots at
// piv[piv_off], the block's DOFs at dofs[idx_off].
struct RootTask {
  int64_t a_off;
  int n;
  int piv_off;
  int idx_off;
  int pad;
};
void launch_dense_lu_batched(void* base, bool fp32, const RootTask* tasks, int count, int nmax,
                             int* piv, int* status, cudaStream_t st);
void launch_dense_solve_batched(const void* base, bool fp32, const RootTask* tasks, int count,
                                int nmax, const int* piv, const int* dofs, void* x, int ld,
                                int nrhs, cudaStream_t st);
// FP32 root blocks of at most kRootInvMax DOFs: explicit inverse in place
// of the block (Gauss-Jordan with partial pivoting), then x[idx, :] =
// A^{-1} x[idx, :] as one product per application.
constexpr int kRootInvMax = 128;
void launch_root_inverse(float* base, const RootTask* tasks, int count, int* status,
                         cudaStream_t st);
void launch_root_apply(const float* base, const RootTask* tasks, int count, const int* dofs,
                       float* x, int ld, int nrhs, cudaStream_t st);
// One large block (the bordered system's S): explicit inverse by all SMs
// (cooperative launch, Gauss-Jordan with partial pivoting; a is overwritten,
// ainv receives A^{-1}, column major).  bar: one unsigned of scratch; err:
// raised if a grid barrier times out; status: raised for a singular block.
// Returns cudaErrorInvalidValue when n is too large for the kernel's shared
// memory (the caller then factors with LU).
cudaError_t launch_coop_inverse(float* a, int n, float* ainv, unsigned* bar, int* err,
                                int* status, cudaStream_t st);
cudaError_t launch_coop_inverse(double* a, int n, double* ainv, unsigned* bar, int* err,
                                int* status, cudaStream_t st);
size_t coop_inverse_smem(int n, int grid, size_t elem_bytes);
// y = ainv x (n x n column major, x and y distinct).
void launch_dense_gemv(const float* ainv, int n, const float* x, float* y, cudaStream_t st);
void launch_dense_gemv(const double* ainv, int n, const double* x, double* y, cudaStream_t st);
void launch_dense_lu(double* a, int n, int* piv, int* status, cudaStream_t st);
void launch_dense_lu_f32(float* a, int n, int* piv, int* status, cudaStream_t st);
// x[idx, :] = LU^{-1} x[idx, :] (idx == nullptr: rows 0..n-1); x is Real.
void launch_dense_solve_gather(const void* lu, bool fp32, int n, const int* piv,
                               const int* idx, void* x, int ld, int nrhs, cudaStream_t st);
// Precision conversions and residual update for refinement.
void launch_d2f(const double* in, float* out, size_t n, cudaStream_t st);
void launch_add_f2d(double* acc, const float* inc, size_t n, cudaStream_t st);
void launch_f2d(const float* in, double* out, size_t n, cudaStream_t st);

// Dense double-layer block K(I, J) (FP64), column major.
void launch_kernel_block(const Geo<double>& g, int pde, int sd, const int* I, int nI,
                         const int* J, int nJ, double* out, cudaStream_t st);
// y = K x over all DOFs, FP64.
void launch_matvec(const Geo<double>& g, int pde, int sd, int npts, const double* x,
                   int nrhs, double* y, cudaStream_t st);

// Elementwise helpers.
void launch_axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st);

// Flexible GMRES block vectors (krylov.cu): nrhs vectors of the bordered
// system stored as a D x nrhs block then an nb x nrhs block.
constexpr int kKrylovMaxBasis = 32;
int krylov_dot_blocks(int D, int nb);
// h[c * kKrylovMaxBasis + j] = <V_j(c), w(c)> for j < nv; part holds
// nrhs * krylov_dot_blocks(D, nb) * kKrylovMaxBasis partial sums.
void launch_mdot(const double* V, size_t vstride, int nv, const double* w, int D, int nb, int nrhs,
                 double* part, double* h, cudaStream_t st);
// w += sign * sum_j h[c * kKrylovMaxBasis + j] V_j(c)
void launch_maxpy(double* w, const double* V, size_t vstride, int nv, const double* h, double sign,
                  int D, int nb, int nrhs, cudaStream_t st);
// w(c) = x(c) * s[c]
void launch_kscale(double* w, const double* x, const double* s, int D, int nb, int nrhs,
                   cudaStream_t st);

}  // namespace rskel
