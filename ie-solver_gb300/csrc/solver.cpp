// Host orchestration of the GB300 recursive-skeletonization solver and the
// C ABI declared in include/rskel.h.
//
// Factorization (SkelFactorization::skeletonize, ie_solver/skel_factorization/
// skel_factorization.cpp:140-310) runs level by level from the leaves up.  For
// each level the host
//   1. forms every box's active DOF list from its children's skeletons
//      (QuadTree::remove_inactive_dofs_at_level, quadtree.cpp:997-1074) and the
//      row-source lists of the ID matrices (Kernel::get_id_mat, kernel.cpp:293-423);
//   2. uploads one packed plan and launches two batched kernels over all boxes
//      of the level (ID, then Schur elimination), binned by box size;
//   3. reads back the ranks and pivots (a few KB) to plan the next level.
// The device keeps the geometry, every factor block and every Schur-
// complemented diagonal block; nothing is recomputed on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <omp.h>

#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/rskel.h"
#include "border.hpp"
#include "devbuf.hpp"
#include "domain.hpp"
#include "fmm.hpp"
#include "kernels.hpp"
#include "plan.hpp"
#include "rank_model.hpp"
#include "tree.hpp"

using namespace rskel;

namespace {

constexpr size_t kSmemMax = 227 * 1024;
constexpr int kWideMaxN = 1024;  // FP32 wide ID up to this many columns (wider: Householder fold)

struct NodeState {
  int compressed = 0;
  int k = 0, r = 0;
  std::vector<int> active, skel, red, near_, perm, rows;
  int use_proxy = 0;
  int64_t fac_off = -1, piv_off = -1, e_off = -1;
  int e_ld = 0;  // leading dimension of this box's block E (0: none, use the kernel)
  int slot = -1;
};

template <class Real>
struct Factor {
  DevBuf<Real> fac, epool, scratch, x, tmp, mU, mP, S, M, nv;
  DevBuf<Real> Sinv, Mt;  // bordered system: S^{-1} and the product's output
  size_t fac_used = 0, e_used = 0;
};

// An allocator whose value-less construct leaves elements uninitialised:
// the DOF pool of a large batch grows by tens of MB per level, and every
// element it gains is written by the list copies right after, so the zero
// fill of a plain resize was pure cost (about 5 ms per level on the
// 512-boundary batch).
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = DefaultInitAlloc<U>;
  };
  DefaultInitAlloc() = default;
  template <class U>
  DefaultInitAlloc(const DefaultInitAlloc<U>&) {}
  template <class U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};

// memcpy split over the OpenMP team when large (the uploads of a large
// batch's level are tens of MB); a plain memcpy below 4 MB.
void copy_in(void* dst, const void* src, size_t bytes) {
  constexpr size_t kPar = size_t(4) << 20, kChunkBytes = size_t(1) << 20;
  if (bytes < kPar) {
    std::memcpy(dst, src, bytes);
    return;
  }
  const long nch = (long)((bytes + kChunkBytes - 1) / kChunkBytes);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nch; ++c) {
    const size_t o = (size_t)c * kChunkBytes;
    std::memcpy(static_cast<char*>(dst) + o, static_cast<const char*>(src) + o,
                std::min(kChunkBytes, bytes - o));
  }
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

}  // namespace

struct rs_solver {
  rs_config cfg;
  std::string err;
  int n = 0, D = 0, sd = 1, nh = 0;
  std::vector<double> pts, nrm, w, kap, hc, hr;
  QuadTree tree;
  bool tree_built = false;
  std::vector<NodeState> st;
  bool factored = false;
  bool fp32 = false;

  bool dev_ready = false;
  int num_sms = 152;  // of the handle's device; sizes the wide ID's work split
  // launch shapes the autotuner (rs_autotune) picks: the level size from
  // which the FP32 sketched ID's pivoted QR runs one warp per box, and the
  // wide ID's CTAs per SM
  int split_min_tasks = 512;
  int wide_ctas_per_sm = 2;
  // threads per box of the Schur eliminations: 128, 256, or 0 (per launch:
  // 128 when 256-thread CTAs would take more than one wave)
  int elim_threads = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // read-back of ranks while eliminations run
  cudaEvent_t ev_c = nullptr;
  std::vector<cudaEvent_t> lv_ev;  // per level: ID start, ID end, Schur end
  std::vector<int> timed_levels;
  cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr, ev_a = nullptr, ev_b = nullptr;
  cudaEvent_t ev_f0 = nullptr, ev_f1 = nullptr;
  DevBuf<double> gx, gy, gnx, gny, gw, gk, pxy_c, pxy_s;
  bool geo_on_dev = false;

  std::vector<int, DefaultInitAlloc<int>> pool;  // host mirror of the device DOF pool
  DevBuf<int> dofs, perm, ranks, piv, status;
  DevBuf<IdTask> id_tasks;
  DevBuf<DecoupleTask> dc_tasks;
  // a level's ID and elimination task records, uploaded together (one copy)
  DevBuf<unsigned char> lvl_tasks;
  HostBuf<int> h_ranks, h_perm, h_status;
  size_t piv_used = 0;
  Factor<double> F64;
  Factor<float> F32;

  std::vector<SweepTask> sweeps;
  std::vector<int> sweep_ids;  // the box of each sweep task
  size_t sweep_pool = 0;       // pool entries of the sweep tasks' lists
  std::vector<int> sweep_off, sweep_cnt, sweep_nmax;  // per level
  DevBuf<SweepTask> sweep_dev;
  int ns = 0;
  std::vector<int> allskel;
  int allskel_off = -1;
  int64_t root_e_off = -1;  // the first root's E block (the bordered system uses it)
  DevBuf<int> root_piv;
  // one root block per tree: the root tasks (E block, pivots, DOF list) of
  // the dense LU and solve, and the largest root
  std::vector<RootTask> roots_h;
  DevBuf<RootTask> roots_dev;
  int root_nmax = 0;
  bool root_inv = false;  // FP32 root blocks hold explicit inverses (else LU + pivots)
  // boundaries held by the handle (rs_set_geometry_batch) and their point
  // offsets; per-boundary DOF offsets on the device for the norms
  int nprob = 1;
  std::vector<int> prob_pt;
  DevBuf<int> prob_dof;

  // bordered system
  int nb = 0;
  DevBuf<double> U0, PsiT0, G, g1, hole_dev;
  DevBuf<unsigned char> red_mask, skel_mask, ones_mask;
  DevBuf<int> S_piv;
  DevBuf<unsigned> coop_bar;  // grid-barrier counter of the cooperative inverse
  DevBuf<double> cross_part;  // partial sums of masked_cross
  bool s_inv = false;         // the bordered system holds S^{-1} instead of LU + pivots

  // solve buffers
  DevBuf<double> f_dev, mu_dev, alpha_dev, r64, acc64, nrm_dev, x64, xa64, g64;
  HostBuf<double> h_io;
  // flexible GMRES: bases V, Z, work vector, right-hand side, dot partials,
  // coefficients (device) and their host copies
  DevBuf<double> kv, kz, kw, kb, kpart, kh;
  HostBuf<double> hk_up, hk_dn;

  FmmPlan fmm;
  HostBuf<unsigned char> stage;  // pinned staging of a factorization's host-to-device uploads
  HostBuf<double> geo_stage;     // pinned staging of the boundary data (upload_geometry)
  size_t stage_used = 0;
  bool incremental = false;      // next rs_factor keeps the boxes rs_perturb left compressed
  size_t full_fac_used = 0;      // factor storage of the last full factorization
  DevBuf<float> sketch_y;  // FP32 split ID: per-level sketches
  DevBuf<WideItem> wide_items;  // FP32 wide ID: work items and partial sketches of a level
  DevBuf<float> wide_part;
  // Learned sketch sizes: model weights on the device, a level's features
  // (sorted task order), the redo flags per slot, and the last
  // factorization's (features, k/n) samples for training.
  bool rank_model_on = false;
  DevBuf<float> rank_w, rank_feat;
  DevBuf<int> redo, ell_slot;
  DevBuf<float> judge_ratio;  // trace mode: the residual judge's ratio per slot
  HostBuf<int> h_redo, h_ell;
  // the last factorization's rank samples: the ID boxes in order and their
  // k / n (features are formed on request from the boxes' kept lists)
  std::vector<int> samp_box;
  std::vector<float> samp_target;
  double samp_tol = 0;
  double host_plan_ms = 0, host_wait_ms = 0, host_post_ms = 0;

  // CUDA graph of the factorization's inverse (no holes): the level sweeps
  // and the root solves, captured on first use for a (buffer, columns,
  // precision) and replayed; dropped at every factorization.
  struct InvGraph {
    cudaGraphExec_t exec = nullptr;
    const void* x = nullptr;
    int nrhs = 0;
    int fp32 = 0;
    int kernels = 0;
  };
  InvGraph inv_graph;

  rs_stats stats;
  int launches = 0;
  bool trace = false;  // RSKEL_TRACE=1: per-level timing on stderr
  DevBuf<long long> clk;
  DevBuf<long long> dclk;  // trace: the eliminations' phase clocks
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
namespace {

rs_status fail(rs_solver* s, rs_status code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

#define RSCHK(expr)                 \
  do {                              \
    rs_status rc_ = (expr);         \
    if (rc_ != RS_OK) return rc_;   \
  } while (0)

#define CU(expr)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(s, RS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Fresh per-box state for every box of the tree; the lists keep their
// storage, so a handle that factors one geometry after another reallocates
// nothing here.
void reset_states(rs_solver* s) {
  s->st.resize(s->tree.nodes.size());
  for (NodeState& S : s->st) {
    S.compressed = 0;
    S.k = S.r = 0;
    S.active.clear();
    S.skel.clear();
    S.red.clear();
    S.near_.clear();
    S.perm.clear();
    S.rows.clear();
    S.use_proxy = 0;
    S.fac_off = S.piv_off = S.e_off = -1;
    S.e_ld = 0;
    S.slot = -1;
  }
}

rs_status ensure_device(rs_solver* s) {
  if (s->dev_ready) return RS_OK;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0)
    return fail(s, RS_ERR_NO_DEVICE, "no CUDA device available (there is no CPU fallback)");
  if (s->cfg.device < 0 || s->cfg.device >= count) return fail(s, RS_ERR_ARG, "bad device ordinal");
  CU(cudaSetDevice(s->cfg.device));
  CU(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->cfg.device));
  CU(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  CU(cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking));
  CU(cudaEventCreateWithFlags(&s->ev_c, cudaEventDisableTiming));
  CU(cudaEventCreate(&s->ev_t0));
  CU(cudaEventCreate(&s->ev_t1));
  CU(cudaEventCreate(&s->ev_a));
  CU(cudaEventCreate(&s->ev_b));
  CU(cudaEventCreate(&s->ev_f0));
  CU(cudaEventCreate(&s->ev_f1));
  CU(s->status.ensure(4));
  CU(s->h_status.ensure(4));
  s->dev_ready = true;
  return RS_OK;
}

// The boundary data as six device arrays (x, y, n_x, n_y, w, kappa) and the
// proxy-circle directions (kernel.cpp:432-441), gathered in a pinned buffer
// and sent with one asynchronous copy each on the handle's stream.
rs_status upload_geometry(rs_solver* s) {
  if (s->geo_on_dev) return RS_OK;
  const int n = s->n, npp = s->cfg.num_proxy_points;
  CU(s->geo_stage.ensure(6 * (size_t)n + 2 * (size_t)npp));
  double* h = s->geo_stage.p;
  for (int i = 0; i < n; ++i) {
    h[i] = s->pts[2 * i];
    h[n + i] = s->pts[2 * i + 1];
    h[2 * n + i] = s->nrm[2 * i];
    h[3 * n + i] = s->nrm[2 * i + 1];
  }
  std::memcpy(h + 4 * (size_t)n, s->w.data(), n * 8);
  std::memcpy(h + 5 * (size_t)n, s->kap.data(), n * 8);
  for (int i = 0; i < npp; ++i) {
    const double ang = 2 * M_PI * i * (1.0 / npp);
    h[6 * (size_t)n + i] = std::cos(ang);
    h[6 * (size_t)n + npp + i] = std::sin(ang);
  }
  DevBuf<double>* dst[6] = {&s->gx, &s->gy, &s->gnx, &s->gny, &s->gw, &s->gk};
  for (int a = 0; a < 6; ++a) {
    CU(dst[a]->ensure(n));
    CU(cudaMemcpyAsync(dst[a]->p, h + (size_t)a * n, n * 8, cudaMemcpyHostToDevice, s->stream));
  }
  CU(s->pxy_c.ensure(npp));
  CU(s->pxy_s.ensure(npp));
  CU(cudaMemcpyAsync(s->pxy_c.p, h + 6 * (size_t)n, npp * 8, cudaMemcpyHostToDevice, s->stream));
  CU(cudaMemcpyAsync(s->pxy_s.p, h + 6 * (size_t)n + npp, npp * 8, cudaMemcpyHostToDevice,
                     s->stream));
  s->geo_on_dev = true;
  return RS_OK;
}

Geo<double> geo_of(const rs_solver* s) {
  return Geo<double>{s->gx.p, s->gy.p, s->gnx.p, s->gny.p, s->gw.p, s->gk.p};
}

// Surviving DOFs of a box after its level: skeleton when compressed.
const std::vector<int>& surviving(const NodeState& ns) {
  return ns.compressed ? ns.skel : ns.active;
}

// A box's children's runs in its active list (compute_active's order) and
// the children's Schur-complemented blocks; a leaf is one run of kernel
// entries.
void set_child_runs(const rs_solver* s, const TreeNode& nd, DecoupleTask* d) {
  if (nd.is_leaf) {
    for (int c = 0; c < 4; ++c) {
      d->cstart[c] = c == 0 ? 0 : d->n;
      d->cld[c] = 0;
      d->ce[c] = -1;
    }
    return;
  }
  int o = 0;
  for (int c = 0; c < 4; ++c) {
    const NodeState& C = s->st[nd.children[c]];
    d->cstart[c] = o;
    d->cld[c] = C.e_ld;
    d->ce[c] = C.e_ld > 0 ? C.e_off : (int64_t)-1;
    o += (int)surviving(C).size();
  }
}

// QuadTree::remove_inactive_dofs_at_box (quadtree.cpp:1032-1055)
void compute_active(rs_solver* s, int id) {
  NodeState& S = s->st[id];
  const TreeNode& nd = s->tree.nodes[id];
  S.active.clear();
  if (nd.is_leaf) {
    S.active = nd.original;
  } else {
    for (int c = 0; c < 4; ++c) {
      const std::vector<int>& v = surviving(s->st[nd.children[c]]);
      S.active.insert(S.active.end(), v.begin(), v.end());
    }
  }
}

// near lists, quadtree.cpp:1005-1024
void compute_near(rs_solver* s, int id) {
  NodeState& S = s->st[id];
  const TreeNode& nd = s->tree.nodes[id];
  S.near_.clear();
  for (int nb : nd.neighbors) {
    const TreeNode& o = s->tree.nodes[nb];
    if (o.level > nd.level) continue;
    const std::vector<int>& v = o.is_leaf ? o.original : s->st[nb].active;
    S.near_.insert(S.near_.end(), v.begin(), v.end());
  }
}

// Row-source DOFs of a box's ID matrix (kernel.cpp:300-394).
void id_rows(rs_solver* s, int id, std::vector<int>* rows, int* use_proxy) {
  rows->clear();
  const TreeNode& nd = s->tree.nodes[id];
  const int lv = nd.level;
  *use_proxy = 0;
  if (lv == 1 || lv == 2) {
    // (in a forest, the boxes of the same tree: a contiguous run of the
    // level list, which holds the trees in order)
    const int tid = nd.tree_id;
    auto same_tree = [&](const std::vector<int>& lvl) {
      const auto lo = std::partition_point(lvl.begin(), lvl.end(), [&](int o) {
        return s->tree.nodes[o].tree_id < tid;
      });
      const auto hi = std::partition_point(lo, lvl.end(), [&](int o) {
        return s->tree.nodes[o].tree_id == tid;
      });
      return std::make_pair(lo, hi);
    };
    const auto r = same_tree(s->tree.levels[lv]);
    for (auto it = r.first; it != r.second; ++it)
      if (*it != id) {
        const std::vector<int>& v = s->st[*it].active;
        rows->insert(rows->end(), v.begin(), v.end());
      }
    const auto r1 = same_tree(s->tree.levels[1]);
    if (lv == 2)
      for (auto it = r1.first; it != r1.second; ++it)
        if (const int o = *it; s->tree.nodes[o].is_leaf) {
          const std::vector<int>& v = s->tree.nodes[o].original;
          rows->insert(rows->end(), v.begin(), v.end());
        }
    return;
  }
  const double cx = nd.corners[0] + nd.side / 2.0;
  const double cy = nd.corners[1] + nd.side / 2.0;
  const double lim = s->cfg.radius_ratio * nd.side;
  // The reference's test is sqrt(dx^2 + dy^2) < lim; squared distances well
  // away from lim^2 decide it without the square root.
  const double lim2 = lim * lim, lo = lim2 * (1.0 - 1e-12), hi = lim2 * (1.0 + 1e-12);
  for (int mi : s->st[id].near_) {
    const int pv = (mi / s->sd) * 2;
    const double dx = cx - s->pts[pv], dy = cy - s->pts[pv + 1];
    const double d2 = dx * dx + dy * dy;
    if (d2 < lo || (d2 <= hi && std::sqrt(d2) < lim)) rows->push_back(mi);
  }
  *use_proxy = 1;
}

// Input features of the rank model for one box's ID (kRankFeatures values,
// each of order one): sizes of the ID matrix, the box's place in the tree,
// the tolerance and kernel, and the shape of the boundary piece the active
// DOFs sample (curvature relative to the box, spread, quadrature mass).
void rank_features(const rs_solver* s, const TreeNode& nd, const NodeState& S, int m, double tol,
                   float* f) {
  const int n = (int)S.active.size();
  const double side = nd.side > 0 ? nd.side : 1.0;
  const double root = s->tree.max > s->tree.min ? s->tree.max - s->tree.min : 1.0;
  double ksum = 0, kmax = 0, wsum = 0, cx = 0, cy = 0;
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  for (int dof : S.active) {
    const int p = dof / s->sd;
    const double k = std::fabs(s->kap[p]) * side;
    ksum += k;
    kmax = std::max(kmax, k);
    wsum += s->w[p];
    const double x = s->pts[2 * p], y = s->pts[2 * p + 1];
    cx += x;
    cy += y;
    x0 = std::min(x0, x);
    x1 = std::max(x1, x);
    y0 = std::min(y0, y);
    y1 = std::max(y1, y);
  }
  const double inv = n > 0 ? 1.0 / n : 0.0;
  const double kmean = ksum * inv;
  const double bx = nd.corners[0] + side / 2, by = nd.corners[1] + side / 2;
  f[0] = (float)(n / 128.0);
  f[1] = (float)(std::log2(std::max(n, 1)) / 8.0);
  f[2] = (float)(std::log2(std::max(m, 1)) / 12.0);
  f[3] = (float)(std::min(8.0, (double)S.rows.size() / std::max(n, 1)) / 8.0);
  f[4] = (float)S.use_proxy;
  f[5] = (float)(nd.level / 16.0);
  f[6] = (float)(std::log2(side / root) / 16.0);
  f[7] = (float)(-std::log10(tol) / 16.0);
  f[8] = (float)(s->cfg.pde / 2.0);
  f[9] = (float)nd.is_leaf;
  f[10] = (float)(kmean / (1.0 + kmean));
  f[11] = (float)(kmax / (1.0 + kmax));
  f[12] = (float)(std::min(4.0, wsum / (s->sd * side)) / 4.0);
  f[13] = n > 0 ? (float)(std::max(x1 - x0, y1 - y0) / side) : 0.f;
  f[14] = n > 0 ? (float)(std::hypot(cx * inv - bx, cy * inv - by) / side) : 0.f;
  f[15] = (float)(std::log2(std::max(s->D, 1)) / 20.0);
}

// Host-to-device copy through the pinned staging buffer: a copy from pinned
// memory is asynchronous, so a level's uploads no longer wait for the DMA.
// Regions are handed out in order during one factorization (which ends with
// a stream synchronisation), so no region is reused while its copy is in
// flight; growing the buffer waits for the stream first.
cudaError_t stage_copy(rs_solver* s, void* dst, const void* src, size_t bytes) {
  if (!bytes) return cudaSuccess;
  size_t off = (s->stage_used + 255) & ~size_t(255);
  if (off + bytes > s->stage.cap) {
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return e;
    e = s->stage.ensure(std::max<size_t>(2 * s->stage.cap, bytes + 4096));
    if (e != cudaSuccess) return e;
    off = 0;
  }
  copy_in(s->stage.p + off, src, bytes);
  s->stage_used = off + bytes;
  return cudaMemcpyAsync(dst, s->stage.p + off, bytes, cudaMemcpyHostToDevice, s->stream);
}

// Two host arrays to one device buffer, the second at byte offset off2 of
// it, through the staging ring with one copy.
cudaError_t stage_copy2(rs_solver* s, void* dst, const void* src1, size_t bytes1,
                        const void* src2, size_t off2, size_t bytes2) {
  const size_t bytes = bytes2 ? off2 + bytes2 : bytes1;
  if (!bytes) return cudaSuccess;
  size_t off = (s->stage_used + 255) & ~size_t(255);
  if (off + bytes > s->stage.cap) {
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return e;
    e = s->stage.ensure(std::max<size_t>(2 * s->stage.cap, bytes + 4096));
    if (e != cudaSuccess) return e;
    off = 0;
  }
  if (bytes1) copy_in(s->stage.p + off, src1, bytes1);
  if (bytes2) copy_in(s->stage.p + off + off2, src2, bytes2);
  s->stage_used = off + bytes;
  return cudaMemcpyAsync(dst, s->stage.p + off, bytes, cudaMemcpyHostToDevice, s->stream);
}

rs_status upload_pool(rs_solver* s, size_t from) {
  size_t to = s->pool.size();
  if (to == from) return RS_OK;
  CU(s->dofs.ensure_keep(to, from, s->stream));
  CU(s->perm.ensure_keep(to, from, s->stream));
  CU(stage_copy(s, s->dofs.p + from, s->pool.data() + from, (to - from) * sizeof(int)));
  return RS_OK;
}

double id_flops(int m, int n, int k, int pde) {
  const double per = pde == kStokes ? 20.0 : 10.0;
  const double r = n - k;
  return per * m * n + 4.0 * m * n * k - 2.0 * k * k * (m + n) + 4.0 * k * k * k / 3.0 +
         (double)k * k * r;
}
// One pass of the FP32 randomized ID of a box (ell sketch rows): the ID
// matrix fill, the +-1 sketch (2 ell m n, none when the matrix is no taller
// than ell and is factored itself), pivoted QR of the min(m, ell) x n tile
// to the rank, and Z.
double sketch_id_flops(int m, int n, int k, int ell, int pde) {
  const double per = pde == kStokes ? 20.0 : 10.0;
  const double mr = std::min(m, ell), r = n - k;
  return per * m * n + (m > ell ? 2.0 * ell * m * n : 0.0) + 4.0 * mr * n * k -
         2.0 * k * k * (mr + n) + 4.0 * k * k * k / 3.0 + (double)k * k * r;
}
double dec_flops(int k, int r) {
  const double K = k, R = r;
  return 2.0 * (R * K * K + 2 * R * R * K + R * K * K + K * K * R) + 2.0 / 3.0 * R * R * R +
         4.0 * R * R * K + 2.0 * K * K * R;
}

template <class Real>
Factor<Real>& factor_of(rs_solver* s);
template <>
Factor<double>& factor_of<double>(rs_solver* s) { return s->F64; }
template <>
Factor<float>& factor_of<float>(rs_solver* s) { return s->F32; }

// Splits a level's tasks (sorted by n) into at most three launches: boxes of
// up to 64 DOFs, larger boxes whose tiles fit in shared memory, and boxes
// that need global-memory tiles.  Few launches keep every box of a level in
// flight at once; the shared-memory request of each launch is its largest box.
// merge: the first two classes go in one launch (the larger class's
// configuration serves both).  For a level of fewer boxes than SMs, whose
// launches each last about one box's latency and run one after the other,
// that saves a whole launch.
template <class Task, class Fits, class Launch>
void launch_binned(const std::vector<Task>& tasks, const Task* dev_tasks, Fits&& fits,
                   Launch&& fn, bool merge = false) {
  auto cls = [&](int n) { return !fits(n) ? 2 : (n <= 64 && !merge ? 0 : 1); };
  size_t i = 0;
  while (i < tasks.size()) {
    const int c = cls(tasks[i].n);
    size_t j = i;
    int nmax = 0;
    while (j < tasks.size() && cls(tasks[j].n) == c) {
      nmax = std::max(nmax, tasks[j].n);
      ++j;
    }
    fn(dev_tasks + i, (int)(j - i), nmax);
    i = j;
  }
}

template <class Real>
rs_status factor_border(rs_solver* s);

// The stable order of tasks by their size n, by counting sort: the order
// std::stable_sort by n gives, in time linear in the tasks and the largest n.
template <class Task>
void order_by_n(const std::vector<Task>& v, std::vector<size_t>* o, std::vector<int>* cnt) {
  int nmax = 0;
  for (const Task& t : v) nmax = std::max(nmax, t.n);
  cnt->assign((size_t)nmax + 2, 0);
  for (const Task& t : v) ++(*cnt)[t.n + 1];
  for (int i = 1; i <= nmax + 1; ++i) (*cnt)[i] += (*cnt)[i - 1];
  o->resize(v.size());
  for (size_t i = 0; i < v.size(); ++i) (*o)[(*cnt)[v[i].n]++] = i;
}

template <class Real>
rs_status factor_impl(rs_solver* s) {
  constexpr bool f32 = sizeof(Real) == 4;
  Factor<Real>& F = factor_of<Real>(s);
  const int L = (int)s->tree.levels.size();
  const double tol = f32 ? std::max(s->cfg.id_tol, s->cfg.fp32_id_tol) : s->cfg.id_tol;
  // After rs_perturb the boxes still compressed keep their factors, E blocks
  // and pivots where they are (skel_factorization.cpp:157 skips them); new
  // ones are appended.  Once the appended storage reaches eight times a full
  // factorization's, everything is factored afresh (which reclaims it).
  const bool incr = s->incremental && F.fac_used > 0 && F.fac_used < 8 * s->full_fac_used + 1024;
  if (s->trace)
    std::fprintf(stderr, "[rskel] factor: incremental %d (requested %d, storage %zu of %zu)\n",
                 (int)incr, (int)s->incremental, F.fac_used, s->full_fac_used);
  s->incremental = false;
  if (!incr) {
    reset_states(s);
    F.fac_used = 0;
    F.e_used = 0;
    s->piv_used = 0;
  }
  s->stage_used = 0;
  s->pool.clear();
  s->stats.id_flops = 0;
  s->stats.decouple_flops = 0;
  s->stats.id_ms = 0;
  s->stats.decouple_ms = 0;
  s->launches = 0;
  s->stats.max_active = 0;
  s->stats.max_rank = 0;
  s->stats.max_rows = 0;
  s->stats.boxes_factored = 0;
  CU(cudaMemsetAsync(s->status.p, 0, sizeof(int) * 4, s->stream));
  std::vector<IdTask> idt;
  std::vector<DecoupleTask> dct;
  std::vector<int> rows;
  std::vector<int> cand_ids, dc_ids;
  std::vector<int> m_of_slot;
  std::vector<float> feat, feat_s;  // rank-model features per slot, and in sorted order
  std::vector<double> slot_work;    // per slot: ID flops, sketch rows, Schur flops
  std::vector<size_t> oi, od;       // a level's tasks in size order
  std::vector<int> sort_cnt;
  std::vector<IdTask> idt_s;
  std::vector<DecoupleTask> dct_s;
  const bool model = f32 && s->rank_model_on;
  s->samp_box.clear();
  s->samp_target.clear();
  s->samp_tol = tol;
  s->stats.rank_predicted = 0;
  s->stats.rank_redo = 0;
  s->stats.rank_redo_judge = 0;
  s->stats.sketch_rows = 0;
  // Contents below these marks are live and survive buffer growth.
  size_t fac_prev = F.fac_used, e_prev = F.e_used, piv_prev = s->piv_used;
  double t_plan = 0, t_wait = 0, t_post = 0;
  double t_detail[4] = {0, 0, 0, 0};  // lists, task records, sorting/scratch, uploads+launches
  while ((int)s->lv_ev.size() < 3 * L) {
    cudaEvent_t e;
    CU(cudaEventCreate(&e));
    s->lv_ev.push_back(e);
  }
  s->timed_levels.clear();
  for (int lv = L - 1; lv >= 1; --lv) {
    const double h0 = now_ms();
    const std::vector<int>& lvl = s->tree.levels[lv];
    const int nl = (int)lvl.size();
    // Per-box list construction is independent across the boxes of a level.
#pragma omp parallel for schedule(dynamic, 16) if (nl > 96)
    for (int q = 0; q < nl; ++q)
      if (!s->st[lvl[q]].compressed) compute_active(s, lvl[q]);
#pragma omp parallel for schedule(dynamic, 16) if (nl > 96)
    for (int q = 0; q < nl; ++q) {
      const int id = lvl[q];
      compute_near(s, id);
      NodeState& S = s->st[id];
      if (!S.compressed && (int)S.active.size() >= s->cfg.min_dofs_to_compress)
        id_rows(s, id, &S.rows, &S.use_proxy);
    }
    const double h_lists = now_ms();
    idt.clear();
    dct.clear();
    cand_ids.clear();
    dc_ids.clear();
    m_of_slot.clear();
    const size_t seg0 = s->pool.size();
    const int npp = s->cfg.num_proxy_points;
    const int prow = (s->cfg.pde == kStokes ? 2 : 1) * npp;
    // Offsets first (a serial prefix pass), then the task records and the
    // pool / block-reference copies, which are independent across boxes.
    struct Slots {
      int kind = 0;  // 0: nothing to do, 1: Schur assembly only, 2: ID + elimination
      int slot = -1, dci = -1;
      size_t act_off = 0, rows_off = 0;
    };
    std::vector<Slots> pl(nl);
    size_t pool_end = seg0;
    int nslots = 0, ndc = 0;
    for (int q = 0; q < nl; ++q) {
      const int id = lvl[q];
      NodeState& S = s->st[id];
      if (S.compressed) continue;  // kept from before rs_perturb
      const TreeNode& nd = s->tree.nodes[id];
      const int n = (int)S.active.size();
      const bool cand = n >= s->cfg.min_dofs_to_compress;
      if (!cand && nd.is_leaf) {
        S.e_ld = 0;
        continue;
      }
      Slots& P = pl[q];
      P.kind = cand ? 2 : 1;
      P.act_off = pool_end;
      pool_end += n;
      S.fac_off = -1;
      S.slot = -1;
      if (cand) {
        P.rows_off = pool_end;
        pool_end += S.rows.size();
        P.slot = nslots++;
        S.slot = P.slot;
        S.fac_off = (int64_t)F.fac_used;
        F.fac_used += fac_reserve(n);
      }
      P.dci = ndc++;
      S.piv_off = (int64_t)s->piv_used;
      s->piv_used += n;
      S.e_off = (int64_t)F.e_used;
      F.e_used += (size_t)n * n;
      s->stats.max_active = std::max(s->stats.max_active, n);
    }
    // Learned sketch sizes on levels of at least one box per SM: there the
    // ID is throughput-bound and shorter sketches save work; a level of fewer
    // boxes runs each box on an SM of its own, so its time is one box's
    // latency, which a truncated sketch barely shortens and a redone box
    // doubles.
    const bool learned = model && nslots >= s->num_sms;
    s->pool.resize(pool_end);
    idt.resize(nslots);
    m_of_slot.resize(nslots);
    cand_ids.resize(nslots);
    dct.resize(ndc);
    dc_ids.resize(ndc);
    feat.resize((size_t)nslots * kRankFeatures);
    int max_rows = s->stats.max_rows;
#pragma omp parallel for schedule(dynamic, 16) reduction(max : max_rows) if (nl > 96)
    for (int q = 0; q < nl; ++q) {
      const Slots& P = pl[q];
      if (P.kind == 0) continue;
      const int id = lvl[q];
      const NodeState& S = s->st[id];
      const TreeNode& nd = s->tree.nodes[id];
      const int n = (int)S.active.size();
      std::copy(S.active.begin(), S.active.end(), s->pool.begin() + P.act_off);
      if (P.kind == 2) {
        std::copy(S.rows.begin(), S.rows.end(), s->pool.begin() + P.rows_off);
        IdTask t{};
        t.n = n;
        t.act_off = (int)P.act_off;
        t.q = (int)S.rows.size();
        t.rows_off = (int)P.rows_off;
        t.use_proxy = S.use_proxy;
        t.slot = P.slot;
        t.cx = nd.corners[0] + nd.side / 2.0;
        t.cy = nd.corners[1] + nd.side / 2.0;
        t.pr = nd.side * s->cfg.radius_ratio;
        t.fac_off = S.fac_off;
        t.scratch_off = -1;
        t.dense_off = -1;
        t.m_dense = 0;
        const int m = 2 * t.q + (S.use_proxy ? 2 * prow : 0);
        m_of_slot[P.slot] = m;
        if (learned)  // (samples compute theirs on request: rs_rank_samples)
          rank_features(s, nd, S, m, tol, feat.data() + (size_t)P.slot * kRankFeatures);
        max_rows = std::max(max_rows, m);
        idt[P.slot] = t;
        cand_ids[P.slot] = id;
      }
      DecoupleTask d{};
      d.n = n;
      d.act_off = (int)P.act_off;
      d.slot = S.slot;
      d.perm_off = (int)P.act_off;
      d.fac_off = S.fac_off;
      d.piv_off = S.piv_off;
      d.e_off = S.e_off;
      d.scratch_off = -1;
      set_child_runs(s, nd, &d);
      dct[P.dci] = d;
      dc_ids[P.dci] = id;
    }
    s->stats.max_rows = max_rows;
    const double h_tasks = now_ms();
    if (dct.empty()) continue;
    // sort by size for binned launches (slots keep their identity)
    order_by_n(idt, &oi, &sort_cnt);
    order_by_n(dct, &od, &sort_cnt);
    idt_s.resize(idt.size());
    dct_s.resize(dct.size());
    for (size_t i = 0; i < oi.size(); ++i) idt_s[i] = idt[oi[i]];
    if (learned) {
      feat_s.resize(feat.size());
      for (size_t i = 0; i < oi.size(); ++i)
        std::memcpy(feat_s.data() + i * kRankFeatures, feat.data() + oi[i] * kRankFeatures,
                    sizeof(float) * kRankFeatures);
    }
    for (size_t i = 0; i < od.size(); ++i) dct_s[i] = dct[od[i]];
    // global-memory tiles for boxes whose tiles do not fit in shared memory
    size_t scratch_need = 0;
    // FP32 wide ID: boxes of 129..kWideMaxN columns, a contiguous range of
    // the size-sorted tasks.  Work items split each sketched box into
    // column blocks and row ranges so that the level fills the GPU.
    std::vector<WideItem> witems;
    size_t w0 = idt_s.size(), w1 = idt_s.size(), part_need = 0;
    if (f32) {
      w0 = 0;
      while (w0 < idt_s.size() && idt_s[w0].n <= 128) ++w0;
      w1 = w0;
      while (w1 < idt_s.size() && idt_s[w1].n <= kWideMaxN) ++w1;
      int blocks = 0;
      for (size_t i = w0; i < w1; ++i) {
        const IdTask& t = idt_s[i];
        const int m = 2 * t.q + (t.use_proxy ? 2 * prow : 0);
        if (m > id_sketch_rows(t.n)) blocks += (t.n + kWideCols - 1) / kWideCols;
      }
      const int want =
          blocks > 0 ? (s->wide_ctas_per_sm * s->num_sms + blocks - 1) / blocks : 1;
      for (size_t i = w0; i < w1; ++i) {
        IdTask& t = idt_s[i];
        const int m = 2 * t.q + (t.use_proxy ? 2 * prow : 0), ell = id_sketch_rows(t.n);
        t.m_dense = m > ell ? ell : 0;
        t.wide_split = 0;
        t.scratch_off = (int64_t)scratch_need;
        scratch_need += id_wide_tile(m > ell ? ell : m, t.n);
        if (m <= ell) continue;
        // row ranges of whole chunks, at least two chunks each
        const int chunks = (m + 63) / 64;
        int ns = std::max(1, std::min(want, chunks / 2));
        const int per = (chunks + ns - 1) / ns;
        ns = (chunks + per - 1) / per;
        t.wide_split = ns;
        t.y_off = (int64_t)part_need;
        const int ncb = (t.n + kWideCols - 1) / kWideCols;
        const int sbk = wide_sketch_block(ell);
        for (int jb = 0; jb < ncb; ++jb)
          for (int q = 0; q < ns; ++q)
            for (int s0 = 0; s0 < ell; s0 += sbk) {
              WideItem it;
              it.task = (int)(i - w0);
              it.j0 = jb * kWideCols;
              it.r0 = q * per * 64;
              it.r1 = std::min(m, (q + 1) * per * 64);
              it.s0 = s0;
              it.s1 = std::min(ell, s0 + sbk);
              it.part_off = t.y_off + ((int64_t)(jb * ns + q) * ell) * kWideCols;
              witems.push_back(it);
            }
        part_need += (size_t)ncb * ns * ell * kWideCols;
      }
    }
    for (size_t ti = 0; ti < idt_s.size(); ++ti) {
      IdTask& t = idt_s[ti];
      if (ti >= w0 && ti < w1) continue;  // wide: placed above
      if (!f32) {  // FP64: direct pivoted QR on the whole ID matrix
        const int m = 2 * t.q + (t.use_proxy ? 2 * prow : 0);
        t.scratch_off = (int64_t)scratch_need;
        scratch_need += id_direct_tile(m, t.n);
      } else if (id_kernel_smem(t.n, f32, true) > kSmemMax) {
        t.scratch_off = (int64_t)scratch_need;
        scratch_need += (size_t)(t.n + 32) * (t.n + 64) + 64;
      }
    }
    // FP32: sketches of the split randomized ID (boxes of at most 128
    // columns); the wide tasks' y_off (their partial sketches) is set above
    size_t y_need = 0;
    for (size_t ti = 0; ti < idt_s.size(); ++ti) {
      IdTask& t = idt_s[ti];
      if (ti >= w0 && ti < w1) continue;
      t.y_off = -1;
      if (f32 && t.n <= 128) {
        t.y_off = (int64_t)y_need;
        y_need += id_sketch_y_size(t.n);
      }
    }
    if (y_need) CU(s->sketch_y.ensure(y_need));
    for (DecoupleTask& t : dct_s)
      if (decouple_kernel_smem(t.n, f32, true) > kSmemMax) {
        t.scratch_off = (int64_t)scratch_need;
        scratch_need += (size_t)(t.n + 1) * (t.n + 1) * 2;
      }
    // upload
    const double h_sort = now_ms();
    RSCHK(upload_pool(s, seg0));
    CU(F.fac.ensure_keep(F.fac_used, fac_prev, s->stream));
    CU(F.epool.ensure_keep(F.e_used, e_prev, s->stream));
    CU(s->piv.ensure_keep(s->piv_used, piv_prev, s->stream));
    fac_prev = F.fac_used;
    e_prev = F.e_used;
    piv_prev = s->piv_used;
    if (scratch_need) CU(F.scratch.ensure(scratch_need));
    // the level's ID and elimination task records in one buffer, one copy
    const size_t idt_bytes = idt_s.size() * sizeof(IdTask);
    const size_t dct_off = (std::max<size_t>(idt_bytes, 1) + 255) & ~size_t(255);
    CU(s->lvl_tasks.ensure(dct_off + std::max<size_t>(dct_s.size(), 1) * sizeof(DecoupleTask)));
    IdTask* const d_idt = reinterpret_cast<IdTask*>(s->lvl_tasks.p);
    DecoupleTask* const d_dct = reinterpret_cast<DecoupleTask*>(s->lvl_tasks.p + dct_off);
    CU(s->ranks.ensure(std::max<size_t>(idt_s.size(), 1)));
    CU(stage_copy2(s, s->lvl_tasks.p, idt_s.data(), idt_bytes, dct_s.data(), dct_off,
                   dct_s.size() * sizeof(DecoupleTask)));
    if (!witems.empty()) {
      CU(s->wide_items.ensure(witems.size()));
      CU(s->wide_part.ensure(part_need));
      CU(stage_copy(s, s->wide_items.p, witems.data(), witems.size() * sizeof(WideItem)));
    }
    if (learned && !idt_s.empty()) {
      // predicted sketch sizes written into the uploaded task records
      CU(s->rank_feat.ensure(feat_s.size()));
      CU(s->redo.ensure(idt_s.size()));
      CU(s->ell_slot.ensure(idt_s.size()));
      CU(stage_copy(s, s->rank_feat.p, feat_s.data(), feat_s.size() * sizeof(float)));
      CU(cudaMemsetAsync(s->redo.p, 0, idt_s.size() * sizeof(int), s->stream));
      CU(rank_infer_ell(s->rank_w.p, s->rank_feat.p, d_idt, (int)idt_s.size(),
                        s->ell_slot.p, (float)s->cfg.rank_headroom, s->cfg.rank_extra_rows,
                        s->stream));
      ++s->launches;
    }
    // ID launches
    IdParams ip{};
    ip.geo = geo_of(s);
    ip.pde = s->cfg.pde;
    ip.sd = s->sd;
    ip.npp = s->cfg.num_proxy_points;
    ip.tol = tol;
    ip.tasks = d_idt;
    ip.dofs = s->dofs.p;
    ip.pxy_cos = s->pxy_c.p;
    ip.pxy_sin = s->pxy_s.p;
    ip.ranks = s->ranks.p;
    ip.perm = s->perm.p;
    ip.fac = F.fac.p;
    ip.scratch = F.scratch.p;
    ip.dense = nullptr;
    ip.direct = f32 ? 0 : 1;
    ip.sketch_y = y_need ? s->sketch_y.p : nullptr;
    ip.redo = learned && !idt_s.empty() ? s->redo.p : nullptr;
    ip.redo_pass = 0;
    ip.judge_factor = ip.redo != nullptr ? (float)s->cfg.rank_judge : 0.f;
    ip.judge_ratio = nullptr;
    if (s->trace && ip.redo != nullptr) {
      CU(s->judge_ratio.ensure(idt_s.size()));
      CU(cudaMemsetAsync(s->judge_ratio.p, 0xff, idt_s.size() * sizeof(float), s->stream));
      ip.judge_ratio = s->judge_ratio.p;
    }
    ip.split_min_tasks = s->split_min_tasks;
    ip.tc = s->cfg.tensor_cores;
    ip.status = s->status.p + 2;
    ip.phase_clk = nullptr;
    if (s->trace) {
      CU(s->clk.ensure(4 * std::max<size_t>(idt.size(), 1)));
      CU(cudaMemsetAsync(s->clk.p, 0, 4 * idt.size() * sizeof(long long), s->stream));
      ip.phase_clk = s->clk.p;
    }
    CU(cudaEventRecord(s->lv_ev[3 * lv], s->stream));
    s->timed_levels.push_back(lv);
    auto id_fits = [&](int n) { return id_kernel_smem(n, f32, true) <= kSmemMax; };
    auto dc_fits = [&](int n) { return decouple_kernel_smem(n, f32, true) <= kSmemMax; };
    const bool small_level = (int)idt_s.size() < s->num_sms;
    // A level of fewer ID boxes than SMs (no learned sizes there): each box's
    // ID matrix rows go to several CTAs, about two CTAs per SM in all, at
    // most one per 64-row chunk.
    ip.row_groups = 1;
    ip.y_parts = 0;
    ip.y_group_stride = (int64_t)y_need;
    if (f32 && small_level && ip.redo == nullptr && y_need > 0 && s->cfg.id_row_groups != 0 &&
        s->cfg.id_row_groups != 1) {
      int chunks = 1;
      for (const IdTask& t : idt_s)
        chunks = std::max(chunks, (2 * t.q + (t.use_proxy ? 2 * prow : 0) + 63) / 64);
      const int want = s->cfg.id_row_groups > 0
                           ? s->cfg.id_row_groups
                           : (2 * s->num_sms) / std::max<int>(1, (int)idt_s.size());
      ip.row_groups = std::max(1, std::min({chunks, want, 16}));
      if (ip.row_groups > 1) CU(s->sketch_y.ensure((size_t)ip.row_groups * y_need));
      ip.sketch_y = s->sketch_y.p;
    }
    auto id_launch = [&](const IdTask* dt, int cnt, int nmax) {
      IdParams q = ip;
      q.tasks = dt;
      bool in_smem = !ip.direct && id_kernel_smem(nmax, f32, true) <= kSmemMax;
      s->launches += launch_id(q, cnt, nmax, id_kernel_smem(nmax, f32, in_smem), f32, s->stream);
    };
    if (w0 < w1) {
      // the three ranges: up to 128 columns, wide, wider
      const std::vector<IdTask> lo(idt_s.begin(), idt_s.begin() + w0);
      const std::vector<IdTask> hi(idt_s.begin() + w1, idt_s.end());
      launch_binned(lo, d_idt, id_fits, id_launch, small_level);
      IdParams q = ip;
      q.tasks = d_idt + w0;
      s->launches += launch_id_wide(q, (int)(w1 - w0), idt_s[w1 - 1].n, s->wide_items.p,
                                    (int)witems.size(), s->wide_part.p, s->stream);
      launch_binned(hi, d_idt + w1, id_fits, id_launch, small_level);
    } else {
      launch_binned(idt_s, d_idt, id_fits, id_launch, small_level);
    }
    CU(cudaGetLastError());
    CU(cudaEventRecord(s->lv_ev[3 * lv + 1], s->stream));
    // ranks and pivots come back on the side stream while the eliminations run
    const size_t seg1 = s->pool.size();
    CU(s->h_ranks.ensure(std::max<size_t>(idt.size(), 1)));
    CU(s->h_perm.ensure(seg1 - seg0 + 1));
    CU(cudaStreamWaitEvent(s->stream2, s->lv_ev[3 * lv + 1], 0));
    if (!idt.empty())
      CU(cudaMemcpyAsync(s->h_ranks.p, s->ranks.p, idt.size() * sizeof(int),
                         cudaMemcpyDeviceToHost, s->stream2));
    if (ip.redo != nullptr) {
      CU(s->h_redo.ensure(idt.size()));
      CU(cudaMemcpyAsync(s->h_redo.p, s->redo.p, idt.size() * sizeof(int), cudaMemcpyDeviceToHost,
                         s->stream2));
      CU(s->h_ell.ensure(idt.size()));
      CU(cudaMemcpyAsync(s->h_ell.p, s->ell_slot.p, idt.size() * sizeof(int),
                         cudaMemcpyDeviceToHost, s->stream2));
    }
    CU(cudaMemcpyAsync(s->h_perm.p, s->perm.p + seg0, (seg1 - seg0) * sizeof(int),
                       cudaMemcpyDeviceToHost, s->stream2));
    CU(cudaEventRecord(s->ev_c, s->stream2));
    // decouple launches
    DecoupleParams dp{};
    dp.geo = geo_of(s);
    dp.pde = s->cfg.pde;
    dp.sd = s->sd;
    dp.tasks = d_dct;
    dp.dofs = s->dofs.p;
    dp.ranks = s->ranks.p;
    dp.perm = s->perm.p;
    dp.fac = F.fac.p;
    dp.piv = s->piv.p;
    dp.epool = F.epool.p;
    dp.scratch = F.scratch.p;
    dp.status = s->status.p;
    dp.phase_clk = nullptr;
    if (s->trace) {
      CU(s->dclk.ensure(6 * std::max<size_t>(dct_s.size(), 1)));
      CU(cudaMemsetAsync(s->dclk.p, 0, 6 * dct_s.size() * sizeof(long long), s->stream));
    }
    launch_binned(dct_s, d_dct, dc_fits, [&](const DecoupleTask* dt, int cnt, int nmax) {
      DecoupleParams q = dp;
      q.tasks = dt;
      if (s->trace) q.phase_clk = s->dclk.p + 6 * (dt - d_dct);
      bool in_smem = decouple_kernel_smem(nmax, f32, true) <= kSmemMax;
      launch_decouple(q, cnt, decouple_kernel_smem(nmax, f32, in_smem), f32, s->stream,
                      s->elim_threads, s->num_sms);
      ++s->launches;
    }, (int)dct_s.size() < s->num_sms);
    CU(cudaGetLastError());
    CU(cudaEventRecord(s->lv_ev[3 * lv + 2], s->stream));
    const double h1 = now_ms();
    t_detail[0] += h_lists - h0;
    t_detail[1] += h_tasks - h_lists;
    t_detail[2] += h_sort - h_tasks;
    t_detail[3] += h1 - h_sort;
    CU(cudaEventSynchronize(s->ev_c));
    const double h2 = now_ms();
    t_plan += h1 - h0;
    t_wait += h2 - h1;
    if (s->trace) {
      CU(cudaStreamSynchronize(s->stream));
      float ms_id = 0, ms_dc = 0;
      cudaEventElapsedTime(&ms_id, s->lv_ev[3 * lv], s->lv_ev[3 * lv + 1]);
      cudaEventElapsedTime(&ms_dc, s->lv_ev[3 * lv + 1], s->lv_ev[3 * lv + 2]);
      std::vector<long long> clk(4 * idt.size());
      CU(cudaMemcpy(clk.data(), s->clk.p, clk.size() * sizeof(long long), cudaMemcpyDeviceToHost));
      double ph[4] = {0, 0, 0, 0}, mx[4] = {0, 0, 0, 0};
      for (size_t q = 0; q < idt.size(); ++q)
        for (int z = 0; z < 4; ++z) {
          ph[z] += (double)clk[4 * q + z];
          mx[z] = std::max(mx[z], (double)clk[4 * q + z]);
        }
      const double cnt = idt.empty() ? 1.0 : (double)idt.size();
      std::fprintf(stderr, "[rskel]   ID cycles per box avg/max: fill %.0f/%.0f fold|qr-head %.0f/%.0f cpqr %.0f/%.0f z %.0f/%.0f\n",
                   ph[0] / cnt, mx[0], ph[1] / cnt, mx[1], ph[2] / cnt, mx[2], ph[3] / cnt, mx[3]);
      {
        // the eliminations: phase cycles per box (average, and the slowest
        // box's phases with its n and k)
        const size_t nd = dct_s.size();
        std::vector<long long> dc(6 * nd);
        CU(cudaMemcpy(dc.data(), s->dclk.p, dc.size() * sizeof(long long), cudaMemcpyDeviceToHost));
        double av[4] = {0, 0, 0, 0};
        size_t worst = 0;
        long long wt = -1;
        for (size_t q = 0; q < nd; ++q) {
          long long tot = 0;
          for (int z = 0; z < 4; ++z) {
            av[z] += (double)dc[6 * q + z];
            tot += dc[6 * q + z];
          }
          if (tot > wt) {
            wt = tot;
            worst = q;
          }
        }
        const double dn = nd ? (double)nd : 1.0;
        if (nd)
          std::fprintf(stderr,
                       "[rskel]   Schur cycles per box avg: assemble %.0f products %.0f inverse %.0f rest %.0f;"
                       " slowest (n %lld k %lld): %lld %lld %lld %lld\n",
                       av[0] / dn, av[1] / dn, av[2] / dn, av[3] / dn, dc[6 * worst + 4],
                       dc[6 * worst + 5], dc[6 * worst], dc[6 * worst + 1], dc[6 * worst + 2],
                       dc[6 * worst + 3]);
      }
      if (ip.judge_ratio != nullptr) {
        // residual judge: estimated residual / (tol |a_max|) of the judged boxes
        std::vector<float> jr(idt.size());
        CU(cudaMemcpy(jr.data(), s->judge_ratio.p, jr.size() * sizeof(float),
                      cudaMemcpyDeviceToHost));
        std::vector<float> v;
        for (float x : jr)
          if (x == x) v.push_back(x);  // NaN: not judged
        std::sort(v.begin(), v.end());
        if (!v.empty())
          std::fprintf(stderr,
                       "[rskel]   judge: %zu boxes, ratio median %.3g p90 %.3g p99 %.3g max %.3g, "
                       "%d above %.3g\n",
                       v.size(), v[v.size() / 2], v[v.size() * 9 / 10], v[v.size() * 99 / 100],
                       v.back(), (int)(v.end() - std::upper_bound(v.begin(), v.end(),
                                                                   (float)s->cfg.rank_judge)),
                       s->cfg.rank_judge);
      }
      int mmax = 0, nmax = 0;
      double msum = 0;
      for (size_t q = 0; q < idt.size(); ++q) {
        mmax = std::max(mmax, m_of_slot[q]);
        nmax = std::max(nmax, idt[q].n);
        msum += m_of_slot[q];
      }
      std::fprintf(stderr,
                   "[rskel] level %2d: %5zu ID boxes (m max %5d avg %6.0f, n max %4d), %5zu "
                   "eliminations; ID %.3f ms, Schur %.3f ms\n",
                   lv, idt.size(), mmax, idt.empty() ? 0.0 : msum / idt.size(), nmax, dct.size(),
                   ms_id, ms_dc);
    }
    // Per-box bookkeeping after the read-back, independent across boxes:
    // samples and work counts go to per-slot entries (summed in slot order
    // below, so the totals do not depend on the thread count).
    const int nc = (int)cand_ids.size();
    const size_t sbase = s->samp_target.size();
    s->samp_box.resize(sbase + nc);
    s->samp_target.resize(sbase + nc);
    slot_work.assign(3 * (size_t)nc, 0.0);  // {id flops, sketch rows, Schur flops}
    int n_pred = 0, n_redo = 0, n_redo_judge = 0, n_fac = 0, k_max = s->stats.max_rank;
#pragma omp parallel for schedule(dynamic, 32) if (nc > 96) \
    reduction(+ : n_pred, n_redo, n_redo_judge, n_fac) reduction(max : k_max)
    for (int c = 0; c < nc; ++c) {
      const int id = cand_ids[c];
      NodeState& S = s->st[id];
      const int k = s->h_ranks.p[S.slot];
      const int n = (int)S.active.size();
      s->samp_box[sbase + c] = id;
      s->samp_target[sbase + c] = k > 0 ? (float)k / (float)n : 1.f;
      const int m = m_of_slot[S.slot];
      double* wk = slot_work.data() + 3 * (size_t)c;
      if (f32 && n > 128 && n <= kWideMaxN) {
        wk[1] = std::min(m, n + 16);
        wk[0] = sketch_id_flops(m, n, k, n + 16, s->cfg.pde);
      } else if (f32 && n <= 128) {
        // rows the randomized ID sketched (m when the matrix is no taller)
        const int full = n + 16;
        int ell = full;
        bool again = false;
        int tests = 0;  // the residual judge's test rows
        if (ip.redo != nullptr) {
          ++n_pred;
          again = s->h_redo.p[S.slot] != 0;
          n_redo += again;
          n_redo_judge += s->h_redo.p[S.slot] == 2;
          ell = std::min(s->h_ell.p[S.slot], full);
          if (ip.judge_factor > 0.f && ell < full && m > ell) tests = kIdTestRows;
        }
        wk[1] = std::min(m, ell) + tests + (again ? std::min(m, full) : 0);
        wk[0] = sketch_id_flops(m, n, k, ell, s->cfg.pde) + (tests ? 2.0 * tests * m * n : 0.0) +
                (again ? sketch_id_flops(m, n, k, full, s->cfg.pde) : 0.0);
      } else {
        wk[0] = id_flops(m, n, k, s->cfg.pde);
      }
      if (k <= 0) {
        S.e_ld = n;
        continue;
      }
      const int act_off = idt[S.slot].act_off;
      S.compressed = 1;
      S.k = k;
      S.r = n - k;
      S.perm.assign(s->h_perm.p + (act_off - seg0), s->h_perm.p + (act_off - seg0) + n);
      S.skel.resize(k);
      S.red.resize(n - k);
      for (int i = 0; i < k; ++i) S.skel[i] = S.active[S.perm[i]];
      for (int i = k; i < n; ++i) S.red[i - k] = S.active[S.perm[i]];
      S.e_ld = k;
      k_max = std::max(k_max, k);
      wk[2] = dec_flops(k, n - k);
      ++n_fac;
    }
    for (int c = 0; c < nc; ++c) {
      s->stats.id_flops += slot_work[3 * (size_t)c];
      s->stats.sketch_rows += slot_work[3 * (size_t)c + 1];
      s->stats.decouple_flops += slot_work[3 * (size_t)c + 2];
    }
    s->stats.rank_predicted += n_pred;
    s->stats.rank_redo += n_redo;
    s->stats.rank_redo_judge += n_redo_judge;
    s->stats.boxes_factored += n_fac;
    s->stats.max_rank = k_max;
    for (int id : dc_ids) {
      NodeState& S = s->st[id];
      if (S.slot < 0) S.e_ld = (int)S.active.size();
    }
    t_post += now_ms() - h2;
    if (s->trace)
      std::fprintf(stderr,
                   "[rskel]   host level %2d: lists %.3f tasks %.3f sort %.3f launch %.3f wait %.3f "
                   "post %.3f ms\n",
                   lv, h_lists - h0, h_tasks - h_lists, h_sort - h_tasks, h1 - h_sort, h2 - h1,
                   now_ms() - h2);
  }
  s->host_plan_ms = t_plan;
  s->host_wait_ms = t_wait;
  s->host_post_ms = t_post;
  if (s->trace)
    std::fprintf(stderr,
                 "[rskel] host: plan+launch %.3f ms (lists %.3f, tasks %.3f, sort %.3f, upload+launch "
                 "%.3f), wait %.3f ms, post %.3f ms\n",
                 t_plan, t_detail[0], t_detail[1], t_detail[2], t_detail[3], t_wait, t_post);
  const double h3 = now_ms();
  // remove_inactive_dofs_at_all_boxes (quadtree.cpp:989-995): only the root
  // (and level-0 bookkeeping) changes for a fresh factorization.  A forest
  // (a batch of boundaries) has one root per tree.
  for (int r : s->tree.roots) {
    compute_active(s, r);
    compute_near(s, r);
  }
  // root blocks (skel_factorization.cpp:174-186), one per tree
  const size_t seg0 = s->pool.size();
  s->allskel_off = (int)seg0;
  s->allskel.clear();
  s->roots_h.clear();
  s->root_nmax = 0;
  std::vector<DecoupleTask> rdt;
  int piv_total = 0;
  for (int r : s->tree.roots) {
    const NodeState& R = s->st[r];
    RootTask rt{};
    rt.n = (int)R.active.size();
    rt.idx_off = (int)s->pool.size();
    rt.piv_off = piv_total;
    rt.a_off = (int64_t)F.e_used;
    s->pool.insert(s->pool.end(), R.active.begin(), R.active.end());
    s->allskel.insert(s->allskel.end(), R.active.begin(), R.active.end());
    if (rt.n == 0) continue;
    piv_total += rt.n;
    F.e_used += (size_t)rt.n * rt.n;
    DecoupleTask d{};
    d.n = rt.n;
    d.act_off = rt.idx_off;
    d.slot = -1;
    d.perm_off = rt.idx_off;
    d.e_off = rt.a_off;
    d.scratch_off = -1;
    set_child_runs(s, s->tree.nodes[r], &d);
    rdt.push_back(d);
    s->roots_h.push_back(rt);
    s->root_nmax = std::max(s->root_nmax, rt.n);
  }
  s->ns = (int)s->allskel.size();
  s->root_e_off = s->roots_h.empty() ? 0 : s->roots_h[0].a_off;
  // solve plan: compressed boxes per level, skeleton / redundant lists
  s->sweeps.clear();
  s->sweep_ids.clear();
  s->sweep_pool = 0;
  s->sweep_off.assign(L, 0);
  s->sweep_cnt.assign(L, 0);
  s->sweep_nmax.assign(L, 0);
  // (a serial pass for the tasks' pool offsets, then the lists are copied
  // in parallel: a batch of boundaries has hundreds of thousands of boxes)
  for (int lv = L - 1; lv >= 1; --lv) {
    s->sweep_off[lv] = (int)s->sweeps.size();
    for (int id : s->tree.levels[lv]) {
      const NodeState& S = s->st[id];
      if (!S.compressed) continue;
      SweepTask t{};
      t.k = S.k;
      t.r = S.r;
      t.skel_off = (int)(s->pool.size() + s->sweep_pool);
      t.red_off = t.skel_off + S.k;
      s->sweep_pool += (size_t)S.k + S.r;
      t.fac_off = S.fac_off;
      t.piv_off = S.piv_off;
      s->sweeps.push_back(t);
      s->sweep_ids.push_back(id);
      s->sweep_nmax[lv] = std::max(s->sweep_nmax[lv], S.k + S.r);
    }
    s->sweep_cnt[lv] = (int)s->sweeps.size() - s->sweep_off[lv];
  }
  {
    const size_t base = s->pool.size();
    s->pool.resize(base + s->sweep_pool);
    const int nsw = (int)s->sweeps.size();
#pragma omp parallel for schedule(dynamic, 64) if (nsw > 512)
    for (int i = 0; i < nsw; ++i) {
      const NodeState& S = s->st[s->sweep_ids[i]];
      std::copy(S.skel.begin(), S.skel.end(), s->pool.begin() + s->sweeps[i].skel_off);
      std::copy(S.red.begin(), S.red.end(), s->pool.begin() + s->sweeps[i].red_off);
    }
  }
  RSCHK(upload_pool(s, seg0));
  CU(s->sweep_dev.ensure(std::max<size_t>(s->sweeps.size(), 1)));
  if (!s->sweeps.empty())
    CU(cudaMemcpyAsync(s->sweep_dev.p, s->sweeps.data(), s->sweeps.size() * sizeof(SweepTask),
                       cudaMemcpyHostToDevice, s->stream));
  CU(F.epool.ensure_keep(F.e_used, e_prev, s->stream));
  if (!rdt.empty()) {
    // root E blocks: the same assembly as a level's uncompressed boxes,
    // every tree's root in one launch (binned by size)
    std::stable_sort(rdt.begin(), rdt.end(),
                     [](const DecoupleTask& a, const DecoupleTask& b) { return a.n < b.n; });
    size_t rscratch = 0;
    for (DecoupleTask& d : rdt)
      if (decouple_kernel_smem(d.n, f32, true) > kSmemMax) {
        d.scratch_off = (int64_t)rscratch;
        rscratch += (size_t)(d.n + 1) * (d.n + 1) * 2;
      }
    if (rscratch) CU(F.scratch.ensure(rscratch));
    CU(s->dc_tasks.ensure(rdt.size()));
    CU(stage_copy(s, s->dc_tasks.p, rdt.data(), rdt.size() * sizeof(DecoupleTask)));
    DecoupleParams dp{};
    dp.geo = geo_of(s);
    dp.pde = s->cfg.pde;
    dp.sd = s->sd;
    dp.tasks = s->dc_tasks.p;
    dp.dofs = s->dofs.p;
    dp.ranks = s->ranks.p;
    dp.perm = s->perm.p;
    dp.fac = F.fac.p;
    dp.piv = s->piv.p;
    dp.epool = F.epool.p;
    dp.scratch = F.scratch.p;
    dp.status = s->status.p;
    auto dc_fits = [&](int n) { return decouple_kernel_smem(n, f32, true) <= kSmemMax; };
    launch_binned(rdt, s->dc_tasks.p, dc_fits, [&](const DecoupleTask* dt, int cnt, int nmax) {
      DecoupleParams q = dp;
      q.tasks = dt;
      bool in_smem = decouple_kernel_smem(nmax, f32, true) <= kSmemMax;
      launch_decouple(q, cnt, decouple_kernel_smem(nmax, f32, in_smem), f32, s->stream,
                      s->elim_threads, s->num_sms);
      ++s->launches;
    });
    CU(cudaGetLastError());
  }
  CU(s->root_piv.ensure(std::max(piv_total, 1)));
  if (!s->roots_h.empty()) {
    CU(s->roots_dev.ensure(s->roots_h.size()));
    CU(stage_copy(s, s->roots_dev.p, s->roots_h.data(), s->roots_h.size() * sizeof(RootTask)));
  }
  s->nb = 0;
  s->root_inv = false;
  if (s->nh > 0 && s->cfg.pde != kLaplaceNeumann) {
    // bordered system, skel_factorization.cpp:188-305
    rs_status rc = factor_border<Real>(s);
    if (rc != RS_OK) return rc;
  } else if (!s->roots_h.empty()) {
    s->root_inv = f32 && s->cfg.root_inverse != 0 && s->root_nmax <= kRootInvMax;
    if (s->root_inv)
      launch_root_inverse((float*)F.epool.p, s->roots_dev.p, (int)s->roots_h.size(),
                          s->status.p, s->stream);
    else
      launch_dense_lu_batched(F.epool.p, f32, s->roots_dev.p, (int)s->roots_h.size(),
                              s->root_nmax, s->root_piv.p, s->status.p, s->stream);
    ++s->launches;
  }
  CU(cudaGetLastError());
  if (!incr) s->full_fac_used = F.fac_used;
  if (s->trace) std::fprintf(stderr, "[rskel] host: root + solve plan %.3f ms\n", now_ms() - h3);
  return RS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// bordered system (holes): linear_solve.cpp:20-112 and
// skel_factorization.cpp:188-305, 596-777
// ---------------------------------------------------------------------------
namespace {

template <class Real>
void sweep_levels(rs_solver* s, Real* x, int ld, int nrhs, int mode, bool up) {
  Factor<Real>& F = factor_of<Real>(s);
  const int L = (int)s->tree.levels.size();
  SweepParams sp{};
  sp.dofs = s->dofs.p;
  sp.fac = F.fac.p;
  sp.piv = s->piv.p;
  sp.x = x;
  sp.ld = ld;
  sp.nrhs = nrhs;
  sp.mode = mode;
  // trace mode: CUDA-event time of each level's launch
  std::vector<std::pair<int, cudaEvent_t>> marks;
  auto mark = [&](int lv) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) == cudaSuccess) {
      cudaEventRecord(e, s->stream);
      marks.emplace_back(lv, e);
    }
  };
  for (int step = 0; step < L - 1; ++step) {
    const int lv = up ? L - 1 - step : 1 + step;
    if (!s->sweep_cnt[lv]) continue;
    if (s->trace) mark(lv);
    sp.tasks = s->sweep_dev.p + s->sweep_off[lv];
    launch_sweep(sp, s->sweep_cnt[lv], s->sweep_nmax[lv], sizeof(Real) == 4, s->stream);
    ++s->launches;
  }
  if (s->trace && !marks.empty()) {
    mark(-1);
    cudaEventSynchronize(marks.back().second);
    std::fprintf(stderr, "[rskel] %s sweep (mode %d) per level:", up ? "up" : "down", mode);
    for (size_t i = 0; i + 1 < marks.size(); ++i) {
      float ms = 0;
      cudaEventElapsedTime(&ms, marks[i].second, marks[i + 1].second);
      std::fprintf(stderr, " L%d %d boxes %.1fus;", marks[i].first, s->sweep_cnt[marks[i].first],
                   ms * 1e3);
    }
    std::fprintf(stderr, "\n");
    for (auto& m : marks) cudaEventDestroy(m.second);
  }
}

template <class Real>
rs_status factor_border(rs_solver* s) {
  Factor<Real>& F = factor_of<Real>(s);
  s->nb = s->cfg.pde == kStokes ? 3 * s->nh : s->nh;
  const int D = s->D, nb = s->nb, ns = s->ns;
  std::vector<unsigned char> red(D, 1), sk(D, 0);
  for (int i : s->allskel) {
    red[i] = 0;
    sk[i] = 1;
  }
  bool any_red = false;
  for (unsigned char c : red) any_red |= c != 0;
  if (!any_red) return fail(s, RS_ERR_NO_COMPRESSION, "No compression possible");
  CU(s->red_mask.ensure(D));
  CU(s->skel_mask.ensure(D));
  CU(stage_copy(s, s->red_mask.p, red.data(), D));
  CU(stage_copy(s, s->skel_mask.p, sk.data(), D));
  CU(s->U0.ensure((size_t)D * nb));
  CU(s->PsiT0.ensure((size_t)D * nb));
  CU(s->hole_dev.ensure(3 * (size_t)s->nh));
  CU(stage_copy(s, s->hole_dev.p, s->hc.data(), 2 * (size_t)s->nh * sizeof(double)));
  CU(stage_copy(s, s->hole_dev.p + 2 * s->nh, s->hr.data(), (size_t)s->nh * sizeof(double)));
  border_fill(s->gx.p, s->gy.p, s->gw.p, s->n, s->cfg.pde, s->hole_dev.p,
              s->hole_dev.p + 2 * s->nh, s->nh, s->U0.p, s->PsiT0.p, s->stream);
  CU(F.mU.ensure((size_t)D * nb));
  CU(F.mP.ensure((size_t)D * nb));
  CU(F.tmp.ensure((size_t)D * nb));
  convert_from_double<Real>(s->U0.p, F.mU.p, (size_t)D * nb, s->stream);
  convert_from_double<Real>(s->PsiT0.p, F.mP.p, (size_t)D * nb, s->stream);
  s->launches += 3;
  // sweeps on U (with L) and Psi^T (with U^T), skel_factorization.cpp:229-266
  sweep_levels<Real>(s, F.mU.p, D, nb, kUpPlain, true);
  sweep_levels<Real>(s, F.mP.p, D, nb, kUpTransU, true);
  // D^{-1} C on a copy of the modified U (redundant rows), :268-285
  CU(cudaMemcpyAsync(F.tmp.p, F.mU.p, (size_t)D * nb * sizeof(Real), cudaMemcpyDeviceToDevice,
                     s->stream));
  sweep_levels<Real>(s, F.tmp.p, D, nb, kDiagOnly, true);
  CU(s->G.ensure((size_t)nb * nb));
  CU(s->cross_part.ensure(masked_cross_scratch(nb, nb, D)));
  masked_cross<Real>(F.mP.p, D, nb, F.tmp.p, D, nb, s->red_mask.p, D, s->G.p, nb,
                     s->cross_part.p, s->stream);
  const int SN = ns + nb;
  CU(F.S.ensure((size_t)SN * SN));
  assemble_s<Real>(F.S.p, ns, nb, F.epool.p + s->root_e_off, F.mU.p, F.mP.p, D,
                   s->dofs.p + s->allskel_off, s->G.p, s->stream);
  CU(s->S_piv.ensure(SN));
  // S^{-1} by all SMs (Gauss-Jordan with partial pivoting); LU with partial
  // pivoting by one CTA (dgetrf, as the reference factors S) only when S is
  // too large for the cooperative kernel's shared memory
  s->s_inv = false;
  CU(F.Sinv.ensure((size_t)SN * SN));
  CU(F.Mt.ensure(SN));
  CU(s->coop_bar.ensure(1));
  const cudaError_t ce = launch_coop_inverse(F.S.p, SN, F.Sinv.p, s->coop_bar.p,
                                             s->status.p + 1, s->status.p, s->stream);
  if (ce == cudaSuccess) s->s_inv = true;
  else if (ce != cudaErrorInvalidValue) CU(ce);
  else (void)cudaGetLastError();
  if (!s->s_inv) {
    if constexpr (sizeof(Real) == 4)
      launch_dense_lu_f32(F.S.p, SN, s->S_piv.p, s->status.p, s->stream);
    else
      launch_dense_lu(F.S.p, SN, s->S_piv.p, s->status.p, s->stream);
  }
  s->launches += 4;
  CU(cudaGetLastError());
  return RS_OK;
}

// multiply_connected_solve (skel_factorization.cpp:596-777) for one column x
// (device, Real, length D) with second-block right-hand side g (nb, may be
// null = 0).  On return x = mu and alpha (device, Real, nb) is set.
template <class Real>
rs_status solve_border_col(rs_solver* s, Real* x, Real* alpha, const double* g) {
  Factor<Real>& F = factor_of<Real>(s);
  const int D = s->D, nb = s->nb, ns = s->ns, SN = ns + nb;
  CU(F.nv.ensure(D));
  CU(F.M.ensure(SN));
  CU(s->g1.ensure(2 * (size_t)nb));
  sweep_levels<Real>(s, x, D, 1, kUpPlain, true);
  CU(cudaMemcpyAsync(F.nv.p, x, D * sizeof(Real), cudaMemcpyDeviceToDevice, s->stream));
  sweep_levels<Real>(s, F.nv.p, D, 1, kDiagOnly, true);
  CU(s->cross_part.ensure(masked_cross_scratch(nb, nb, D)));
  masked_cross<Real>(F.mP.p, D, nb, F.nv.p, D, 1, s->red_mask.p, D, s->g1.p, nb,
                     s->cross_part.p, s->stream);
  if (g) launch_axpby(s->g1.p, g, -1.0, 1.0, nb, s->stream);  // g1 <- g1 - g
  border_rhs<Real>(F.M.p, ns, nb, x, s->dofs.p + s->allskel_off, s->g1.p, s->stream);
  if (s->s_inv) {
    launch_dense_gemv(F.Sinv.p, SN, F.M.p, F.Mt.p, s->stream);
    CU(cudaMemcpyAsync(F.M.p, F.Mt.p, SN * sizeof(Real), cudaMemcpyDeviceToDevice, s->stream));
  } else {
    launch_dense_solve_gather(F.S.p, sizeof(Real) == 4, SN, s->S_piv.p, nullptr, F.M.p, SN, 1,
                              s->stream);
  }
  CU(cudaMemcpyAsync(alpha, F.M.p + ns, nb * sizeof(Real), cudaMemcpyDeviceToDevice, s->stream));
  border_sub<Real>(F.nv.p, x, F.mU.p, D, nb, alpha, s->red_mask.p, s->stream);
  sweep_levels<Real>(s, F.nv.p, D, 1, kDiagOnly, true);
  border_merge<Real>(x, F.nv.p, s->red_mask.p, D, s->dofs.p + s->allskel_off, F.M.p, ns,
                     s->stream);
  sweep_levels<Real>(s, x, D, 1, kDown, false);
  s->launches += 8;
  CU(cudaGetLastError());
  return RS_OK;
}

// Applies the factorization inverse in place to x (device, Real, D x nrhs);
// alpha (device, Real, nb x nrhs) for bordered systems; g (device, double,
// nb x nrhs) is the second-block right-hand side (null = 0).
void drop_inverse_graph(rs_solver* s) {
  if (s->inv_graph.exec) cudaGraphExecDestroy(s->inv_graph.exec);
  s->inv_graph = rs_solver::InvGraph();
}

template <class Real>
rs_status apply_inverse(rs_solver* s, Real* x, int nrhs, Real* alpha, const double* g);

// The inverse without holes as one CUDA graph launch (cfg.use_graphs): the
// first call for a buffer and column count captures the launches into a
// graph, later calls replay it.
template <class Real>
rs_status apply_inverse_graph(rs_solver* s, Real* x, int nrhs) {
  rs_solver::InvGraph& G = s->inv_graph;
  const int fp32 = sizeof(Real) == 4;
  if (!(G.exec && G.x == x && G.nrhs == nrhs && G.fp32 == fp32)) {
    drop_inverse_graph(s);
    const int before = s->launches;
    CU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    rs_status rc = apply_inverse<Real>(s, x, nrhs, nullptr, nullptr);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
    if (rc != RS_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CU(e);
    const cudaError_t ei = cudaGraphInstantiate(&G.exec, graph, 0);
    cudaGraphDestroy(graph);
    CU(ei);
    G.x = x;
    G.nrhs = nrhs;
    G.fp32 = fp32;
    G.kernels = s->launches - before;
    s->launches = before;
  }
  CU(cudaGraphLaunch(G.exec, s->stream));
  s->launches += G.kernels;
  return RS_OK;
}

template <class Real>
rs_status apply_inverse(rs_solver* s, Real* x, int nrhs, Real* alpha, const double* g) {
  Factor<Real>& F = factor_of<Real>(s);
  if (s->nb == 0 && s->cfg.use_graphs && !s->trace) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(s->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone) return apply_inverse_graph<Real>(s, x, nrhs);
  }
  if (s->nb == 0) {
    sweep_levels<Real>(s, x, s->D, nrhs, kUpSolve, true);
    if (!s->roots_h.empty()) {
      if constexpr (sizeof(Real) == 4) {
        if (s->root_inv)
          launch_root_apply(F.epool.p, s->roots_dev.p, (int)s->roots_h.size(), s->dofs.p, x,
                            s->D, nrhs, s->stream);
      }
      if (!s->root_inv || sizeof(Real) != 4)
        launch_dense_solve_batched(F.epool.p, sizeof(Real) == 4, s->roots_dev.p,
                                   (int)s->roots_h.size(), s->root_nmax, s->root_piv.p,
                                   s->dofs.p, x, s->D, nrhs, s->stream);
      ++s->launches;
    }
    sweep_levels<Real>(s, x, s->D, nrhs, kDown, false);
    CU(cudaGetLastError());
    return RS_OK;
  }
  for (int c = 0; c < nrhs; ++c) {
    rs_status rc = solve_border_col<Real>(s, x + (size_t)s->D * c, alpha + (size_t)s->nb * c,
                                          g ? g + (size_t)s->nb * c : nullptr);
    if (rc != RS_OK) return rc;
  }
  return RS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// solves and FP64 refinement
// ---------------------------------------------------------------------------
namespace rskel {
void launch_col_norms(const double* x, int rows, int cols, double* out, cudaStream_t st);
void launch_seg_norms(const double* x, int rows, int cols, const int* seg, int np, double* out,
                      cudaStream_t st);
void launch_gemv_sub(double* r, const double* U, const double* a, int D, int nb, cudaStream_t st);
}  // namespace rskel

namespace {

// r = f - K mu - U alpha;  rg = alpha - Psi mu  (bordered operator of
// ie_solver_test.cpp:43-83, [K U; Psi -I]).
// Multipole plan for the refinement residual (Laplace).  FP64 order from the
// configuration, or matched to the refinement tolerance: on the 65536-point
// star the product's relative error is about 10^(-0.36 p - 2.1) (order 20:
// 1.2e-9, 28: 1.8e-12, 32: 6.5e-14), and the residual needs it ten times
// below refine_tol.  FP32 products of corrections at order 16 at most (the
// plan's FP32 table), lower for the later, smaller corrections.
// The Stokes product also evaluates derivatives of the expansions (about
// 30x the Laplace error at the same order on the 16-hole, 131072-point
// geometry), so it takes four more terms.
constexpr int kFmmOrder32 = 16;
int auto_fmm_order(double refine_tol, int pde) {
  const double want = std::max(refine_tol, 1e-15) / 10.0;
  const int p = (int)std::ceil((-std::log10(want) - 2.1) / 0.36) + (pde == kStokes ? 4 : 0);
  return std::min(48, std::max(12, p));
}
// Error of the FP32 product (order kFmmOrder32) of a refinement correction,
// relative to |mu|/|f| times the residual the correction came from, with a
// margin over what refinement runs show: Laplace (65536-point star) 1.4e-8
// -> 6e-8; Stokes (131072 points, 16 holes) 4.7e-7 -> 8e-7.  (On test
// vectors the products measure 1.5e-8 rough / 1.4e-7 smooth for Laplace,
// 7.8e-8 / 3.9e-7 for Stokes.)  The refinement takes the FP32 product of a
// correction only while this bound stays below half the tolerance, and
// sums the bounds.
double fmm32_error(int pde) { return pde == kStokes ? 8e-7 : 6e-8; }
// Below order kFmmOrder32 the FP32 product's error grows with the
// truncation of the expansions: by about 10^0.36 per order dropped (the
// slope of the multipole error over the orders, measured on the 65536-point
// star; the same geometric rate bounds well-separated interactions).
double fmm32_order_factor(int p) { return std::pow(10.0, 0.36 * (kFmmOrder32 - p)); }
constexpr int kFmmOrder32Min = 4;
int fmm32_fixed(const rs_solver* s) {
  return s->cfg.fmm_order32 > 0 ? s->cfg.fmm_order32 : kFmmOrder32;
}
// Relative residual the inner GMRES of GMRES-IR aims for (its FP32
// products and preconditioner are good to about 1e-7).
constexpr double kGmresInnerTol = 1e-6;
int fmm_order_of(const rs_solver* s) {
  return s->cfg.fmm_order > 0 ? s->cfg.fmm_order : auto_fmm_order(s->cfg.refine_tol, s->cfg.pde);
}
rs_status build_fmm(rs_solver* s) {
  const int p = fmm_order_of(s);
  if (p > 64) return fail(s, RS_ERR_ARG, "fmm_order above 64");
  if (!fmm_build(s->fmm, s->tree, s->pts.data(), s->n, p, kFmmOrder32, s->stream))
    return fail(s, RS_ERR_CUDA, "fast multipole plan failed");
  return RS_OK;
}

rs_status residual(rs_solver* s, const double* f, const double* mu, const double* alpha,
                   int nrhs, double* r, double* rg) {
  const int D = s->D;
  if (s->fmm.built) {
    CU(fmm_apply(s->fmm, s->cfg.pde, geo_of(s), mu, nrhs, r, 0.0, 1.0, kFmmDF, s->stream));
    s->launches += fmm_launches(s->fmm, s->cfg.pde, nrhs);
  } else {
    launch_matvec(geo_of(s), s->cfg.pde, s->sd, s->n, mu, nrhs, r, s->stream);
  }
  launch_axpby(r, f, 1.0, -1.0, (size_t)D * nrhs, s->stream);
  s->launches += 2;
  if (s->nb > 0) {
    const int nb = s->nb;
    for (int c = 0; c < nrhs; ++c) {
      launch_gemv_sub(r + (size_t)D * c, s->U0.p, alpha + (size_t)nb * c, D, nb, s->stream);
      CU(s->cross_part.ensure(masked_cross_scratch(nb, nb, D)));
      masked_cross<double>(s->PsiT0.p, D, nb, mu + (size_t)D * c, D, 1, s->ones_mask.p, D,
                           rg + (size_t)nb * c, nb, s->cross_part.p, s->stream);
      launch_axpby(rg + (size_t)nb * c, alpha + (size_t)nb * c, 1.0, -1.0, nb, s->stream);
      s->launches += 3;
    }
  }
  CU(cudaGetLastError());
  return RS_OK;
}

// Residual recurrence for a refinement correction (x, xa) of (mu, alpha):
// r -= K x + U xa and rg -= Psi x - xa, with K x from the FP32 multipole
// variant (the full residual uses the float-float variant) (the correction is ~1e-6 of the solution, so FP32 accuracy of the
// product leaves the residual exact to ~1e-13 of the data).
rs_status residual_update(rs_solver* s, const double* x, const double* xa, int nrhs, double* r,
                          double* rg, double* g, int p32) {
  const int D = s->D;
  if (!fmm_set_order32(s->fmm, p32)) return fail(s, RS_ERR_ARG, "bad FP32 multipole order");
  CU(fmm_apply(s->fmm, s->cfg.pde, geo_of(s), x, nrhs, r, 1.0, -1.0, kFmmF32, s->stream));
  s->launches += fmm_launches(s->fmm, s->cfg.pde, nrhs);
  if (s->nb > 0) {
    const int nb = s->nb;
    for (int c = 0; c < nrhs; ++c) {
      launch_gemv_sub(r + (size_t)D * c, s->U0.p, xa + (size_t)nb * c, D, nb, s->stream);
      CU(s->cross_part.ensure(masked_cross_scratch(nb, nb, D)));
      masked_cross<double>(s->PsiT0.p, D, nb, x + (size_t)D * c, D, 1, s->ones_mask.p, D,
                           g + (size_t)nb * c, nb, s->cross_part.p, s->stream);
      launch_axpby(rg + (size_t)nb * c, g + (size_t)nb * c, -1.0, 1.0, nb, s->stream);
      launch_axpby(rg + (size_t)nb * c, xa + (size_t)nb * c, 1.0, 1.0, nb, s->stream);
      s->launches += 4;
    }
  }
  CU(cudaGetLastError());
  return RS_OK;
}

// y = -(A z) for a block vector z (mu block, then alpha block) through the
// FP32 multipole product: the bordered operator [K U; Psi -I] (the residual
// recurrence's update applied to a zero residual).
rs_status apply_neg_op(rs_solver* s, const double* z, int nrhs, double* y) {
  const int D = s->D, nb = s->nb;
  const size_t nd = (size_t)D * nrhs;
  CU(cudaMemsetAsync(y, 0, (nd + (size_t)nb * nrhs) * 8, s->stream));
  return residual_update(s, z, nb ? z + nd : nullptr, nrhs, y, nb ? y + nd : nullptr, s->g64.p,
                         fmm32_fixed(s));
}

// z = M^{-1} v with the FP32 factorization (block vectors; the alpha block
// of v is the second-block right-hand side of the bordered solve).
rs_status apply_prec(rs_solver* s, const double* v, int nrhs, double* z) {
  Factor<float>& F = s->F32;
  const int D = s->D, nb = s->nb;
  const size_t nd = (size_t)D * nrhs;
  launch_d2f(v, F.x.p, nd, s->stream);
  rs_status rc = apply_inverse<float>(s, F.x.p, nrhs, F.tmp.p, nb ? v + nd : nullptr);
  if (rc != RS_OK) return rc;
  launch_f2d(F.x.p, z, nd, s->stream);
  if (nb) launch_f2d(F.tmp.p, z + nd, (size_t)nb * nrhs, s->stream);
  s->launches += nb ? 3 : 2;
  return RS_OK;
}

// Flexible GMRES (Saad 1993) on A d = b for the block vector b: right
// preconditioned by the FP32 factorization, FP32 multipole products, FP64
// basis vectors orthogonalised by classical Gram-Schmidt applied twice, one
// Krylov space per right-hand side advanced in lockstep.  Stops when every
// right-hand side's residual estimate is below rtol of its |b|, or after m
// steps (no restart: the refinement around it restarts from a fresh
// residual).  d gets the correction; *steps the steps taken.
rs_status fgmres(rs_solver* s, const double* b, int nrhs, double rtol, int m, double* d,
                 int* steps) {
  const int D = s->D, nb = s->nb;
  const size_t nblk = ((size_t)D + nb) * nrhs;
  m = std::max(1, std::min(m, kKrylovMaxBasis - 1));
  CU(s->kv.ensure((size_t)(m + 1) * nblk));
  CU(s->kz.ensure((size_t)m * nblk));
  CU(s->kw.ensure(nblk));
  CU(s->kpart.ensure((size_t)nrhs * krylov_dot_blocks(D, nb) * kKrylovMaxBasis));
  CU(s->kh.ensure((size_t)kKrylovMaxBasis * nrhs));
  CU(s->hk_up.ensure((size_t)kKrylovMaxBasis * nrhs));
  CU(s->hk_dn.ensure((size_t)kKrylovMaxBasis * nrhs));
  double *V = s->kv.p, *Z = s->kz.p, *W = s->kw.p, *kh = s->kh.p;
  const int KB = kKrylovMaxBasis;
  auto read_h = [&](int nv) -> rs_status {
    CU(cudaMemcpyAsync(s->hk_dn.p, kh, sizeof(double) * KB * nrhs, cudaMemcpyDeviceToHost,
                       s->stream));
    CU(cudaStreamSynchronize(s->stream));
    (void)nv;
    return RS_OK;
  };
  auto upload_scale = [&](const std::vector<double>& v) -> rs_status {
    for (int c = 0; c < nrhs; ++c) s->hk_up.p[c] = v[c];
    CU(cudaMemcpyAsync(kh, s->hk_up.p, sizeof(double) * nrhs, cudaMemcpyHostToDevice, s->stream));
    return RS_OK;
  };
  // beta = |b| per right-hand side, v_0 = b / beta
  launch_mdot(b, 0, 1, b, D, nb, nrhs, s->kpart.p, kh, s->stream);
  RSCHK(read_h(1));
  std::vector<double> beta(nrhs), inv(nrhs);
  for (int c = 0; c < nrhs; ++c) {
    beta[c] = std::sqrt(std::max(0.0, s->hk_dn.p[c * KB]));
    inv[c] = beta[c] > 0 ? 1.0 / beta[c] : 0.0;
  }
  RSCHK(upload_scale(inv));
  launch_kscale(V, b, kh, D, nb, nrhs, s->stream);
  s->launches += 3;
  // per right-hand side: Hessenberg columns (after rotations), Givens, rhs g
  std::vector<double> H((size_t)nrhs * (m + 1) * m, 0.0), cs((size_t)nrhs * m), sn((size_t)nrhs * m),
      g((size_t)nrhs * (m + 1), 0.0), h1((size_t)nrhs * KB);
  auto Hc = [&](int c, int i, int j) -> double& { return H[((size_t)c * (m + 1) + i) * m + j]; };
  for (int c = 0; c < nrhs; ++c) g[(size_t)c * (m + 1)] = beta[c];
  int k = 0;
  for (int j = 0; j < m; ++j) {
    double* Vj = V + (size_t)j * nblk;
    double* Zj = Z + (size_t)j * nblk;
    RSCHK(apply_prec(s, Vj, nrhs, Zj));
    RSCHK(apply_neg_op(s, Zj, nrhs, W));
    // classical Gram-Schmidt, twice
    launch_mdot(V, nblk, j + 1, W, D, nb, nrhs, s->kpart.p, kh, s->stream);
    launch_maxpy(W, V, nblk, j + 1, kh, -1.0, D, nb, nrhs, s->stream);
    RSCHK(read_h(j + 1));
    std::copy(s->hk_dn.p, s->hk_dn.p + (size_t)KB * nrhs, h1.begin());
    launch_mdot(V, nblk, j + 1, W, D, nb, nrhs, s->kpart.p, kh, s->stream);
    launch_maxpy(W, V, nblk, j + 1, kh, -1.0, D, nb, nrhs, s->stream);
    RSCHK(read_h(j + 1));
    for (size_t e = 0; e < h1.size(); ++e) h1[e] += s->hk_dn.p[e];
    launch_mdot(W, 0, 1, W, D, nb, nrhs, s->kpart.p, kh, s->stream);
    RSCHK(read_h(1));
    s->launches += 10;
    bool done = true;
    for (int c = 0; c < nrhs; ++c) {
      const double wn = std::sqrt(std::max(0.0, s->hk_dn.p[c * KB]));
      inv[c] = wn > 0 ? 1.0 / wn : 0.0;
      // A z_j = sum_i (-h_i) v_i - |w| v_{j+1}  (w holds -A z_j)
      for (int i = 0; i <= j; ++i) Hc(c, i, j) = -h1[(size_t)c * KB + i];
      Hc(c, j + 1, j) = -wn;
      for (int i = 0; i < j; ++i) {  // earlier rotations
        const double a = Hc(c, i, j), bb = Hc(c, i + 1, j);
        Hc(c, i, j) = cs[(size_t)c * m + i] * a + sn[(size_t)c * m + i] * bb;
        Hc(c, i + 1, j) = -sn[(size_t)c * m + i] * a + cs[(size_t)c * m + i] * bb;
      }
      const double a = Hc(c, j, j), bb = Hc(c, j + 1, j);
      const double r = std::hypot(a, bb);
      const double cj = r > 0 ? a / r : 1.0, sj = r > 0 ? bb / r : 0.0;
      cs[(size_t)c * m + j] = cj;
      sn[(size_t)c * m + j] = sj;
      Hc(c, j, j) = r;
      Hc(c, j + 1, j) = 0.0;
      const double gj = g[(size_t)c * (m + 1) + j];
      g[(size_t)c * (m + 1) + j] = cj * gj;
      g[(size_t)c * (m + 1) + j + 1] = -sj * gj;
      if (beta[c] > 0 && std::fabs(g[(size_t)c * (m + 1) + j + 1]) > rtol * beta[c]) done = false;
    }
    k = j + 1;
    if (done || j + 1 == m) break;
    RSCHK(upload_scale(inv));
    launch_kscale(V + (size_t)(j + 1) * nblk, W, kh, D, nb, nrhs, s->stream);
    ++s->launches;
  }
  // y = R^{-1} g per right-hand side; d = Z y
  for (int c = 0; c < nrhs; ++c) {
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; --i) {
      double t = g[(size_t)c * (m + 1) + i];
      for (int l = i + 1; l < k; ++l) t -= Hc(c, i, l) * y[l];
      y[i] = Hc(c, i, i) != 0.0 ? t / Hc(c, i, i) : 0.0;
    }
    for (int i = 0; i < KB; ++i) s->hk_up.p[(size_t)c * KB + i] = i < k ? y[i] : 0.0;
  }
  CU(cudaMemcpyAsync(kh, s->hk_up.p, sizeof(double) * KB * nrhs, cudaMemcpyHostToDevice,
                     s->stream));
  CU(cudaMemsetAsync(d, 0, nblk * 8, s->stream));
  launch_maxpy(d, Z, nblk, k, kh, 1.0, D, nb, nrhs, s->stream);
  ++s->launches;
  *steps = k;
  CU(cudaGetLastError());
  return RS_OK;
}

rs_status solve_device_impl(rs_solver* s, const double* f, int nrhs, double* mu, double* alpha) {
  const int D = s->D, nb = s->nb;
  const size_t nd = (size_t)D * nrhs;
  if (!s->fp32) {
    Factor<double>& F = s->F64;
    CU(F.x.ensure(nd));
    CU(F.M.ensure(std::max<size_t>((size_t)nb * nrhs, 1)));
    CU(cudaMemcpyAsync(F.x.p, f, nd * 8, cudaMemcpyDeviceToDevice, s->stream));
    rs_status rc = apply_inverse<double>(s, F.x.p, nrhs, alpha, nullptr);
    if (rc != RS_OK) return rc;
    CU(cudaMemcpyAsync(mu, F.x.p, nd * 8, cudaMemcpyDeviceToDevice, s->stream));
    s->stats.refine_iters = 0;
    s->stats.krylov_steps = 0;
    return RS_OK;
  }
  // FP32 factorization + FP64 iterative refinement
  Factor<float>& F = s->F32;
  CU(F.x.ensure(nd));
  CU(F.tmp.ensure(std::max<size_t>((size_t)nb * nrhs, 1)));
  CU(s->r64.ensure(nd));
  CU(s->acc64.ensure(std::max<size_t>(2 * (size_t)nb * nrhs, 1)));
  // Norms per column, or per boundary and column for a batch (each boundary
  // is its own system): ncol entries into h_io.
  const int np = s->nprob;
  const int ncol = np * nrhs;
  CU(s->nrm_dev.ensure(65 * (size_t)nrhs + 2 + (size_t)ncol));  // norms + partial sums
  CU(s->h_io.ensure(4 * (size_t)nrhs + 4 + (size_t)ncol));
  if (np > 1) {
    std::vector<int> seg(np + 1);
    for (int q = 0; q <= np; ++q) seg[q] = s->prob_pt[q] * s->sd;
    CU(s->prob_dof.ensure(np + 1));
    CU(cudaMemcpyAsync(s->prob_dof.p, seg.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice,
                       s->stream));
    CU(cudaStreamSynchronize(s->stream));
  }
  auto launch_norms = [&](const double* x) {
    if (np > 1) launch_seg_norms(x, D, nrhs, s->prob_dof.p, np, s->nrm_dev.p, s->stream);
    else launch_col_norms(x, D, nrhs, s->nrm_dev.p, s->stream);
  };
  double* rg = s->acc64.p;
  double* a64 = alpha;
  CU(cudaMemsetAsync(mu, 0, nd * 8, s->stream));
  if (nb) CU(cudaMemsetAsync(a64, 0, (size_t)nb * nrhs * 8, s->stream));
  CU(cudaMemcpyAsync(s->r64.p, f, nd * 8, cudaMemcpyDeviceToDevice, s->stream));
  launch_norms(f);
  CU(cudaMemcpyAsync(s->h_io.p, s->nrm_dev.p, ncol * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  std::vector<double> fn(s->h_io.p, s->h_io.p + ncol);
  s->stats.residual64_ms = 0;
  s->stats.residual32_ms = 0;
  int it = 0;
  double worst = 0, prev = 1.0;
  const int max_it = std::max(1, s->cfg.refine_max_iters);
  const bool recur = s->fmm.built;
  // FP32 product error relative to the residual a correction came from: the
  // product's own error times |delta| / |r|, which is about |mu| / |f| (set
  // after the first step)
  double eps32 = fmm32_error(s->cfg.pde);
  if (recur) {
    CU(s->x64.ensure(nd));
    CU(s->xa64.ensure(std::max<size_t>((size_t)nb * nrhs, 1)));
    CU(s->g64.ensure(std::max<size_t>((size_t)nb * nrhs, 1)));
  }
  // worst relative residual of r64 (and its event time into the given stat)
  auto measure = [&](double* stat) -> rs_status {
    CU(cudaEventRecord(s->ev_b, s->stream));
    launch_norms(s->r64.p);
    CU(cudaMemcpyAsync(s->h_io.p, s->nrm_dev.p, ncol * 8, cudaMemcpyDeviceToHost, s->stream));
    CU(cudaStreamSynchronize(s->stream));
    float ms_res = 0;
    CU(cudaEventElapsedTime(&ms_res, s->ev_a, s->ev_b));
    if (stat) *stat += ms_res;
    worst = 0;
    for (int c = 0; c < ncol; ++c)
      worst = std::max(worst, fn[c] > 0 ? s->h_io.p[c] / fn[c] : s->h_io.p[c]);
    return RS_OK;
  };
  auto fresh = [&]() -> rs_status {
    CU(cudaEventRecord(s->ev_a, s->stream));
    RSCHK(residual(s, f, mu, a64, nrhs, s->r64.p, rg));
    return measure(&s->stats.residual64_ms);
  };
  // GMRES-IR: the correction equation solved by flexible GMRES instead of
  // one application of the FP32 factorization (refine_solver 2, or 0 once
  // the stationary iteration contracts by less than a factor 10)
  bool krylov = s->cfg.refine_solver == 2;
  int ksteps = 0;
  double rec_err = 0;  // bound on the recurrence's accumulated error (FP32 products)
  const size_t kbl = nd + (size_t)nb * nrhs;
  if (nb) CU(cudaMemsetAsync(rg, 0, (size_t)nb * nrhs * 8, s->stream));
  for (it = 0; it < max_it; ++it) {
    const double before = prev;
    bool upd = false;
    int p32 = fmm32_fixed(s);  // order of this step's FP32 product
    if (krylov) {
      CU(s->kb.ensure(kbl));
      CU(s->x64.ensure(kbl));
      CU(cudaMemcpyAsync(s->kb.p, s->r64.p, nd * 8, cudaMemcpyDeviceToDevice, s->stream));
      if (nb)
        CU(cudaMemcpyAsync(s->kb.p + nd, rg, (size_t)nb * nrhs * 8, cudaMemcpyDeviceToDevice,
                           s->stream));
      int steps = 0;
      RSCHK(fgmres(s, s->kb.p, nrhs, kGmresInnerTol, kKrylovMaxBasis - 1, s->x64.p, &steps));
      ksteps += steps;
      launch_axpby(mu, s->x64.p, 1.0, 1.0, nd, s->stream);
      if (nb) launch_axpby(a64, s->x64.p + nd, 1.0, 1.0, (size_t)nb * nrhs, s->stream);
      s->launches += nb ? 2 : 1;
      RSCHK(fresh());
    } else {
      launch_d2f(s->r64.p, F.x.p, nd, s->stream);
      rs_status rc = apply_inverse<float>(s, F.x.p, nrhs, F.tmp.p, it == 0 || !nb ? nullptr : rg);
      if (rc != RS_OK) return rc;
      CU(cudaEventRecord(s->ev_a, s->stream));
      // residual recurrence with the FP32 product of the correction (x ~
      // prev relative to the data) only while its error, eps32 * prev, is
      // below half the tolerance; otherwise a fresh float-float residual
      upd = recur && it > 0 &&
            eps32 * fmm32_order_factor(fmm32_fixed(s)) * prev <= 0.5 * s->cfg.refine_tol;
      // the correction's product at the lowest order whose error bound stays
      // within a quarter of the recurrence's remaining slack (half the
      // tolerance less the bounds already summed), or within what order 16
      // gives: once the slack is spent, every product is at order 16, so
      // the lower orders never make the bound call for a confirming residual
      if (upd && s->cfg.fmm_order32 == 0) {
        const double slack = 0.5 * s->cfg.refine_tol - rec_err;
        const double budget = std::max(eps32 * prev, 0.25 * slack);
        while (p32 > kFmmOrder32Min && eps32 * fmm32_order_factor(p32 - 1) * prev <= budget)
          --p32;
      }
      if (upd) {
        launch_f2d(F.x.p, s->x64.p, nd, s->stream);
        launch_axpby(mu, s->x64.p, 1.0, 1.0, nd, s->stream);
        if (nb) {
          launch_f2d(F.tmp.p, s->xa64.p, (size_t)nb * nrhs, s->stream);
          launch_axpby(a64, s->xa64.p, 1.0, 1.0, (size_t)nb * nrhs, s->stream);
        }
        s->launches += 4;
        rec_err += eps32 * fmm32_order_factor(p32) * prev;
        RSCHK(residual_update(s, s->x64.p, s->xa64.p, nrhs, s->r64.p, rg, s->g64.p, p32));
        RSCHK(measure(&s->stats.residual32_ms));
      } else {
        launch_add_f2d(mu, F.x.p, nd, s->stream);
        if (nb) launch_add_f2d(a64, F.tmp.p, (size_t)nb * nrhs, s->stream);
        s->launches += 3;
        RSCHK(residual(s, f, mu, a64, nrhs, s->r64.p, rg));
        RSCHK(measure(&s->stats.residual64_ms));
      }
    }
    prev = worst;
    if (s->trace)
      std::fprintf(stderr, "[rskel] refine %d: %s, %s residual %.3e (FP32 order %d)\n", it,
                   krylov ? "GMRES" : "stationary", upd ? "recurrence" : "fresh", worst, p32);
    if (it == 0 && recur) {
      // The multipole errors scale with |mu| while the tolerance is relative
      // to |f|: on an ill-conditioned system (|mu| >> |f|) the float-float
      // product needs more terms and FP32 products of corrections count for
      // more.
      launch_norms(mu);
      CU(cudaMemcpyAsync(s->h_io.p, s->nrm_dev.p, ncol * 8, cudaMemcpyDeviceToHost, s->stream));
      CU(cudaStreamSynchronize(s->stream));
      double amp = 0;
      for (int c = 0; c < ncol; ++c) amp = std::max(amp, fn[c] > 0 ? s->h_io.p[c] / fn[c] : 0.0);
      eps32 *= std::max(amp, 1.0);
      const int want = auto_fmm_order(s->cfg.refine_tol / std::max(amp, 1.0), s->cfg.pde);
      if (s->cfg.fmm_order == 0 && amp > 4.0 && want > s->fmm.p) {
        if (!fmm_set_order(s->fmm, want, s->stream))
          return fail(s, RS_ERR_CUDA, "multipole order update failed");
        if (s->trace)
          std::fprintf(stderr, "[rskel] |mu|/|f| = %.1f: multipole order %d\n", amp, want);
        RSCHK(fresh());
        prev = worst;
      }
    }
    if (worst <= s->cfg.refine_tol && upd &&
        (s->cfg.refine_verify == 2 ||
         (s->cfg.refine_verify == 1 && worst + rec_err > s->cfg.refine_tol))) {
      // the recurrence says converged, but its error bound does not settle
      // it (or confirmation is always asked for): confirm with a fresh residual
      RSCHK(fresh());
      prev = worst;
      rec_err = 0;
    }
    if (worst <= s->cfg.refine_tol) { ++it; break; }
    if (!krylov && s->cfg.refine_solver == 0 && recur && it >= 1 && worst > 0.1 * before) {
      krylov = true;
      if (upd) {  // GMRES works on the true residual
        RSCHK(fresh());
        prev = worst;
        rec_err = 0;
      }
    }
  }
  s->stats.krylov_steps = ksteps;
  s->stats.refine_iters = it;
  s->stats.refine_residual = worst;
  return RS_OK;
}

rs_status check_solver(rs_solver* s) {
  if (!s) return RS_ERR_ARG;
  return RS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void rs_config_default(rs_config* c) {
  if (!c) return;
  c->pde = RS_LAPLACE;
  c->solution_dimension = 1;
  c->domain_dimension = 2;
  c->id_tol = 1e-6;
  c->max_leaf_dofs = 32;
  c->num_proxy_points = 128;
  c->radius_ratio = 1.5;
  c->min_dofs_to_compress = 16;
  c->is_strong_admissibility = 0;
  c->precision = RS_FP64;
  c->refine_tol = 1e-12;
  c->refine_max_iters = 10;
  c->fp32_id_tol = 1e-6;
  c->device = 0;
  c->fmm_order = 0;
  c->rank_headroom = 1.25;
  c->rank_extra_rows = 12;
  c->refine_verify = 1;
  c->refine_solver = 0;
  c->use_graphs = 1;
  c->root_inverse = 1;
  c->rank_judge = 4.0;
  c->tensor_cores = 1;
  c->id_row_groups = -1;
  c->fmm_order32 = 0;
}

rs_status rs_create(const rs_config* cfg, rs_solver** out) {
  if (!cfg || !out) return RS_ERR_ARG;
  *out = nullptr;
  if (cfg->pde < 0 || cfg->pde > 2) return RS_ERR_ARG;
  const int want_sd = cfg->pde == RS_STOKES ? 2 : 1;
  if (cfg->solution_dimension != want_sd || cfg->domain_dimension != 2) return RS_ERR_ARG;
  if (!(cfg->id_tol > 0) || cfg->max_leaf_dofs < 1 || cfg->num_proxy_points < 1 ||
      !(cfg->radius_ratio > 0) || cfg->min_dofs_to_compress < 1)
    return RS_ERR_ARG;
  if (cfg->is_strong_admissibility) return RS_ERR_ARG;
  if (cfg->precision != RS_FP64 && cfg->precision != RS_FP32_REFINE) return RS_ERR_ARG;
  if (!(cfg->rank_headroom >= 1.0 && cfg->rank_headroom <= 4.0) || cfg->rank_extra_rows < 0 ||
      cfg->rank_extra_rows > 128 || cfg->refine_solver < 0 || cfg->refine_solver > 2 ||
      !(cfg->rank_judge >= 0.0 && cfg->rank_judge <= 1e6) || cfg->tensor_cores < 0 ||
      cfg->tensor_cores > 1 || cfg->id_row_groups < -1 || cfg->id_row_groups > 16 ||
      cfg->fmm_order32 < 0 || cfg->fmm_order32 == 1 || cfg->fmm_order32 > 16)
    return RS_ERR_ARG;
  rs_solver* s = new rs_solver();
  s->cfg = *cfg;
  const char* tr = std::getenv("RSKEL_TRACE");
  s->trace = tr && tr[0] == '1';
  s->sd = want_sd;
  s->fp32 = cfg->precision == RS_FP32_REFINE;
  if (s->fp32 && !(s->cfg.fp32_id_tol > 0)) s->cfg.fp32_id_tol = 1e-6;
  std::memset(&s->stats, 0, sizeof(s->stats));
  *out = s;
  return RS_OK;
}

rs_status rs_destroy(rs_solver* s) {
  if (!s) return RS_ERR_ARG;
  if (s->dev_ready) {
    cudaSetDevice(s->cfg.device);
    cudaStreamSynchronize(s->stream);
    drop_inverse_graph(s);
    cudaEventDestroy(s->ev_t0);
    cudaEventDestroy(s->ev_t1);
    cudaEventDestroy(s->ev_a);
    cudaEventDestroy(s->ev_b);
    cudaEventDestroy(s->ev_f0);
    cudaEventDestroy(s->ev_f1);
    cudaEventDestroy(s->ev_c);
    for (cudaEvent_t e : s->lv_ev) cudaEventDestroy(e);
    if (s->stream2) cudaStreamDestroy(s->stream2);
  }
  cudaStream_t st = s->stream;
  delete s;  // device buffers free themselves
  if (st) cudaStreamDestroy(st);
  return RS_OK;
}

rs_status rs_set_geometry(rs_solver* s, int num_points, const double* points,
                          const double* normals, const double* weights, const double* curvatures,
                          int num_holes, const double* hole_centers, const double* hole_radii) {
  if (!s || num_points <= 0 || !points || !normals || !weights || !curvatures || num_holes < 0)
    return fail(s, RS_ERR_ARG, "bad geometry arguments");
  if (num_holes > 0 && (!hole_centers || !hole_radii))
    return fail(s, RS_ERR_ARG, "holes need centres and radii");
  int bad_xy = 0, bad_wk = 0;  // validated before anything of the handle changes
#pragma omp parallel for reduction(| : bad_xy, bad_wk) if (num_points >= 16384)
  for (int i = 0; i < num_points; ++i) {
    bad_xy |= !std::isfinite(points[2 * i]) || !std::isfinite(points[2 * i + 1]) ||
              !std::isfinite(normals[2 * i]) || !std::isfinite(normals[2 * i + 1]);
    bad_wk |= !std::isfinite(weights[i]) || !std::isfinite(curvatures[i]);
  }
  if (bad_xy) return fail(s, RS_ERR_NUMERIC, "non-finite point or normal");
  if (bad_wk) return fail(s, RS_ERR_NUMERIC, "non-finite weight or curvature");
  s->n = num_points;
  s->D = num_points * s->sd;
  s->pts.assign(points, points + 2 * (size_t)num_points);
  s->nrm.assign(normals, normals + 2 * (size_t)num_points);
  s->w.assign(weights, weights + num_points);
  s->kap.assign(curvatures, curvatures + num_points);
  s->nh = num_holes;
  s->nprob = 1;
  s->prob_pt.assign({0, num_points});
  s->hc.assign(hole_centers ? hole_centers : points, hole_centers ? hole_centers + 2 * num_holes : points);
  s->hr.assign(hole_radii ? hole_radii : points, hole_radii ? hole_radii + num_holes : points);
  s->tree_built = false;
  s->factored = false;
  s->geo_on_dev = false;
  s->fmm.built = false;
  if (s->dev_ready) drop_inverse_graph(s);
  return RS_OK;
}

rs_status rs_set_geometry_batch(rs_solver* s, int count, const int* num_points,
                                const double* points, const double* normals,
                                const double* weights, const double* curvatures) {
  if (!s || count < 1 || !num_points) return fail(s, RS_ERR_ARG, "bad batch arguments");
  long long total = 0;
  for (int t = 0; t < count; ++t) {
    if (num_points[t] <= 0) return fail(s, RS_ERR_ARG, "empty boundary in batch");
    total += num_points[t];
  }
  if (total > (1LL << 30) / s->sd) return fail(s, RS_ERR_CAPACITY, "batch too large");
  rs_status rc = rs_set_geometry(s, (int)total, points, normals, weights, curvatures, 0, nullptr,
                                 nullptr);
  if (rc != RS_OK) return rc;
  s->nprob = count;
  s->prob_pt.assign(count + 1, 0);
  for (int t = 0; t < count; ++t) s->prob_pt[t + 1] = s->prob_pt[t] + num_points[t];
  return RS_OK;
}

rs_status rs_build_tree(rs_solver* s) {
  if (!s) return RS_ERR_ARG;
  if (s->n <= 0) return fail(s, RS_ERR_STATE, "no geometry");
  double t0 = now_ms();
  if (s->nprob > 1) {
    // one tree per boundary, merged into a forest (independent problems)
    std::vector<QuadTree> parts(s->nprob);
    std::vector<int> dof_off(s->nprob);
    bool ok = true;
#pragma omp parallel for schedule(dynamic, 4) reduction(&& : ok)
    for (int t = 0; t < s->nprob; ++t) {
      const int p0 = s->prob_pt[t], np = s->prob_pt[t + 1] - p0;
      ok = parts[t].build(s->pts.data() + 2 * (size_t)p0, np, s->sd, s->cfg.max_leaf_dofs) && ok;
      dof_off[t] = p0 * s->sd;
    }
    if (!ok) return fail(s, RS_ERR_ARG, "tree build failed");
    s->tree.merge(parts, dof_off);
  } else if (!s->tree.build(s->pts.data(), s->n, s->sd, s->cfg.max_leaf_dofs)) {
    return fail(s, RS_ERR_ARG, "tree build failed");
  }
  s->fmm.built = false;
  s->tree_built = true;
  s->factored = false;
  reset_states(s);
  s->stats.t_tree_ms = now_ms() - t0;
  s->stats.num_levels = (int)s->tree.levels.size();
  s->stats.num_nodes = (int)s->tree.nodes.size();
  return RS_OK;
}

namespace {
struct PointKey {
  uint64_t x, y;
  bool operator==(const PointKey& o) const { return x == o.x && y == o.y; }
};
struct PointKeyHash {
  size_t operator()(const PointKey& k) const {
    return (size_t)(k.x * 0x9E3779B97F4A7C15ull ^ (k.y + 0x7F4A7C159E3779B9ull + (k.x << 6)));
  }
};
PointKey point_key(const double* p) {
  PointKey k;
  std::memcpy(&k.x, p, 8);
  std::memcpy(&k.y, p + 1, 8);
  return k;
}
}  // namespace

rs_status rs_perturb(rs_solver* s, int num_points, const double* points, const double* normals,
                     const double* weights, const double* curvatures, int num_holes,
                     const double* hole_centers, const double* hole_radii) {
  if (!s) return RS_ERR_ARG;
  if (s->nprob > 1) return fail(s, RS_ERR_ARG, "rs_perturb of a batch");
  if (!s->tree_built)  // nothing to update
    return rs_set_geometry(s, num_points, points, normals, weights, curvatures, num_holes,
                           hole_centers, hole_radii);
  const std::vector<double> old_pts = s->pts;
  const int n_old = s->n, sd = s->sd;
  rs_status rc = rs_set_geometry(s, num_points, points, normals, weights, curvatures, num_holes,
                                 hole_centers, hole_radii);
  if (rc != RS_OK) return rc;
  // old point -> new point by exact coordinates (quadtree.cpp:529-561)
  std::unordered_map<PointKey, int, PointKeyHash> where;
  where.reserve(2 * (size_t)num_points);
  for (int i = 0; i < num_points; ++i) where[point_key(points + 2 * i)] = i;
  std::vector<int> old_to_new(n_old, -1);
  for (int p = 0; p < n_old; ++p) {
    auto it = where.find(point_key(old_pts.data() + 2 * p));
    if (it != where.end()) old_to_new[p] = it->second;
  }
  std::vector<int> id_map;
  std::vector<char> marked;
  s->tree.perturb(old_pts.data(), points, num_points, old_to_new, &id_map, &marked);
  // Boxes left compressed keep their factorization with renumbered DOF
  // lists; everything else starts afresh.
  std::vector<NodeState> st(s->tree.nodes.size());
  std::vector<char> dropped(st.size(), 0);  // compressed before, refactored now
  for (size_t old = 0; old < id_map.size() && old < s->st.size(); ++old) {
    const int nw = id_map[old];
    if (nw < 0 || !s->st[old].compressed) continue;
    if (marked[nw]) {
      dropped[nw] = 1;
      continue;
    }
    NodeState& S = st[nw];
    S = std::move(s->st[old]);
    bool ok = true;
    auto renumber = [&](std::vector<int>& v) {
      for (int& d : v) {
        const int q = old_to_new[d / sd];
        if (q < 0) ok = false;
        else d = sd * q + d % sd;
      }
    };
    renumber(S.active);
    renumber(S.skel);
    renumber(S.red);
    S.near_.clear();
    S.rows.clear();
    if (!ok) {
      S = NodeState();
      dropped[nw] = 1;
    }
  }
  // A box's ID sees everything inside its proxy circle exactly (kernel.cpp:
  // 360-394) and, at levels 1 and 2, every other box of its level
  // (kernel.cpp:300-350).  Besides the reference's marking through neighbour
  // lists, drop every kept box whose proxy circle holds a changed point (old
  // or new position), and all of levels 1 and 2 when anything changed.
  std::vector<double> changed;
  for (int p = 0; p < n_old; ++p)
    if (old_to_new[p] < 0) changed.insert(changed.end(), {old_pts[2 * p], old_pts[2 * p + 1]});
  {
    std::vector<char> found(num_points, 0);
    for (int p = 0; p < n_old; ++p)
      if (old_to_new[p] >= 0) found[old_to_new[p]] = 1;
    for (int i = 0; i < num_points; ++i)
      if (!found[i]) changed.insert(changed.end(), {points[2 * i], points[2 * i + 1]});
  }
  const size_t nch = changed.size() / 2;
  if (nch > 0) {
    // boxes of a level on a grid of their side; a changed point can only be
    // inside the proxy circles of boxes within a few cells of its own
    const TreeNode& rt = s->tree.nodes[s->tree.root];
    const double x0 = rt.corners[0], y0 = rt.corners[1];
    const int reach = (int)std::ceil(s->cfg.radius_ratio) + 1;
    for (size_t lv = 0; lv < s->tree.levels.size(); ++lv) {
      const std::vector<int>& lvl = s->tree.levels[lv];
      if (lvl.empty()) continue;
      const double side = s->tree.nodes[lvl[0]].side;
      const double rad = s->cfg.radius_ratio * side * (1.0 + 1e-9);
      std::unordered_map<int64_t, int> cell;
      cell.reserve(2 * lvl.size());
      auto key = [](int64_t ix, int64_t iy) { return (ix << 32) ^ (iy & 0xffffffffll); };
      for (int id : lvl) {
        const TreeNode& nd = s->tree.nodes[id];
        cell[key((int64_t)std::floor((nd.corners[0] - x0) / side + 0.5),
                 (int64_t)std::floor((nd.corners[1] - y0) / side + 0.5))] = id;
      }
      for (size_t q = 0; q < nch; ++q) {
        const double px = changed[2 * q], py = changed[2 * q + 1];
        const int64_t cx = (int64_t)std::floor((px - x0) / side);
        const int64_t cy = (int64_t)std::floor((py - y0) / side);
        for (int64_t dx = -reach; dx <= reach; ++dx)
          for (int64_t dy = -reach; dy <= reach; ++dy) {
            auto it = cell.find(key(cx + dx, cy + dy));
            if (it == cell.end() || !st[it->second].compressed) continue;
            const TreeNode& nd = s->tree.nodes[it->second];
            const double ex = px - (nd.corners[0] + side / 2.0);
            const double ey = py - (nd.corners[1] + side / 2.0);
            if (lv <= 2 || ex * ex + ey * ey <= rad * rad) {
              st[it->second] = NodeState();
              dropped[it->second] = 1;
            }
          }
      }
      if (lv <= 2)
        for (int id : lvl)
          if (st[id].compressed) {
            st[id] = NodeState();
            dropped[id] = 1;
          }
    }
  }
  // a box whose factorization was dropped drops its ancestors' too
  for (size_t id = 0; id < st.size(); ++id) {
    if (!dropped[id]) continue;
    for (int a = s->tree.nodes[id].parent; a >= 0; a = s->tree.nodes[a].parent)
      if (st[a].compressed) st[a] = NodeState();
  }
  s->st.swap(st);
  s->tree_built = true;
  s->incremental = true;
  s->stats.num_levels = (int)s->tree.levels.size();
  s->stats.num_nodes = (int)s->tree.nodes.size();
  return RS_OK;
}

rs_status rs_factor(rs_solver* s) {
  if (!s) return RS_ERR_ARG;
  if (!s->tree_built) {
    rs_status rc = rs_build_tree(s);
    if (rc != RS_OK) return rc;
  }
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  CU(cudaSetDevice(s->cfg.device));
  rc = upload_geometry(s);
  if (rc != RS_OK) return rc;
  if (s->fp32 && s->nprob > 1 && s->cfg.pde != kLaplace)
    return fail(s, RS_ERR_ARG, "refinement of a batch supports the Laplace double layer only");
  // The multipole plan is needed by the solve only: its host part is built
  // on another thread while the factorization runs, and uploaded after.
  FmmHostPlan fhp;
  std::thread plan_thread;
  const bool need_fmm = s->fp32 && !s->fmm.built;
  // the factorization's OpenMP team leaves a core to the plan thread
  const int omp_threads = omp_get_max_threads();
  if (need_fmm && omp_threads > 2) omp_set_num_threads(omp_threads - 1);
  if (need_fmm) {
    if (fmm_order_of(s) > 64) return fail(s, RS_ERR_ARG, "fmm_order above 64");
    plan_thread = std::thread([s, &fhp] {
      fmm_plan_host(fhp, s->tree, s->pts.data(), s->n, fmm_order_of(s), kFmmOrder32);
    });
  }
  struct Joiner {
    std::thread& t;
    int omp_threads;
    ~Joiner() {
      if (t.joinable()) t.join();
      omp_set_num_threads(omp_threads);
    }
  } joiner{plan_thread, omp_threads};
  double t0 = now_ms();
  drop_inverse_graph(s);
  CU(cudaEventRecord(s->ev_f0, s->stream));
  s->factored = false;
  rc = s->fp32 ? factor_impl<float>(s) : factor_impl<double>(s);
  if (rc != RS_OK) return rc;
  if (s->nh > 0 && s->cfg.pde != kLaplaceNeumann) {
    // the residual's Psi product runs over every DOF: an all-ones mask
    CU(s->ones_mask.ensure(s->D));
    CU(cudaMemsetAsync(s->ones_mask.p, 1, s->D, s->stream));
  }
  CU(cudaEventRecord(s->ev_f1, s->stream));
  if (need_fmm) {
    plan_thread.join();
    if (!fmm_plan_upload(s->fmm, fhp, s->stream))
      return fail(s, RS_ERR_CUDA, "fast multipole plan failed");
  }
  CU(cudaMemcpyAsync(s->h_status.p, s->status.p, 3 * sizeof(int), cudaMemcpyDeviceToHost,
                     s->stream));
  CU(cudaStreamSynchronize(s->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, s->ev_f0, s->ev_f1);
  s->stats.dev_factor_ms = ms;
  s->stats.t_factor_ms = now_ms() - t0;
  s->stats.id_ms = 0;
  s->stats.decouple_ms = 0;
  s->stats.level_gap_ms = 0;
  for (size_t q = 0; q < s->timed_levels.size(); ++q) {
    const int lv = s->timed_levels[q];
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, s->lv_ev[3 * lv], s->lv_ev[3 * lv + 1]);
    cudaEventElapsedTime(&b, s->lv_ev[3 * lv + 1], s->lv_ev[3 * lv + 2]);
    s->stats.id_ms += a;
    s->stats.decouple_ms += b;
    if (q + 1 < s->timed_levels.size()) {
      // from this level's Schur end to the next level's ID start: the
      // stream waits for the host's planning of that level
      cudaEventElapsedTime(&c, s->lv_ev[3 * lv + 2], s->lv_ev[3 * s->timed_levels[q + 1]]);
      s->stats.level_gap_ms += c;
    }
  }
  int nc = 0;
  for (const NodeState& S : s->st) nc += S.compressed;
  s->stats.num_compressed = nc;
  s->stats.num_skel_root = s->ns;
  if (s->h_status.p[1] != 0) return fail(s, RS_ERR_CUDA, "grid barrier timed out");
  if (s->h_status.p[2] != 0) return fail(s, RS_ERR_CUDA, "tensor-core sketch wait gave up");
  if (s->h_status.p[0] != 0) return fail(s, RS_ERR_NUMERIC, "singular or non-finite pivot");
  s->factored = true;
  return RS_OK;
}

rs_status rs_solve_device(rs_solver* s, const double* d_f, int nrhs, double* d_mu,
                          double* d_alpha) {
  if (!s || !d_f || !d_mu || nrhs < 1) return fail(s, RS_ERR_ARG, "bad solve arguments");
  if (!s->factored) return fail(s, RS_ERR_STATE, "solve before factor");
  if (s->nb > 0 && !d_alpha) return fail(s, RS_ERR_ARG, "holes need an alpha output");
  CU(cudaSetDevice(s->cfg.device));
  CU(cudaEventRecord(s->ev_f0, s->stream));
  rs_status rc = solve_device_impl(s, d_f, nrhs, d_mu, d_alpha);
  if (rc != RS_OK) return rc;
  CU(cudaEventRecord(s->ev_f1, s->stream));
  return RS_OK;
}

rs_status rs_solve(rs_solver* s, const double* f, int nrhs, double* mu, double* alpha) {
  if (!s || !f || !mu || nrhs < 1) return fail(s, RS_ERR_ARG, "bad solve arguments");
  if (!s->factored) return fail(s, RS_ERR_STATE, "solve before factor");
  if (s->nb > 0 && !alpha) return fail(s, RS_ERR_ARG, "holes need an alpha output");
  double t0 = now_ms();
  CU(cudaSetDevice(s->cfg.device));
  const size_t nd = (size_t)s->D * nrhs;
  const size_t na = (size_t)s->nb * nrhs;
  CU(s->f_dev.ensure(nd));
  CU(s->mu_dev.ensure(nd));
  CU(s->alpha_dev.ensure(std::max<size_t>(na, 1)));
  CU(cudaMemcpyAsync(s->f_dev.p, f, nd * 8, cudaMemcpyHostToDevice, s->stream));
  rs_status rc = rs_solve_device(s, s->f_dev.p, nrhs, s->mu_dev.p, s->alpha_dev.p);
  if (rc != RS_OK) return rc;
  CU(cudaMemcpyAsync(mu, s->mu_dev.p, nd * 8, cudaMemcpyDeviceToHost, s->stream));
  if (s->nb > 0) CU(cudaMemcpyAsync(alpha, s->alpha_dev.p, na * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, s->ev_f0, s->ev_f1);
  s->stats.dev_solve_ms = ms;
  s->stats.t_solve_ms = now_ms() - t0;
  return RS_OK;
}

rs_status rs_kernel_block(rs_solver* s, const int* I, int nI, const int* J, int nJ, double* out) {
  if (!s || nI < 0 || nJ < 0 || (nI && !I) || (nJ && !J) || (nI > 0 && nJ > 0 && !out))
    return fail(s, RS_ERR_ARG, "bad kernel block arguments");
  for (int i = 0; i < nI; ++i)
    if (I[i] < 0 || I[i] >= s->D) return fail(s, RS_ERR_ARG, "row index out of range");
  for (int j = 0; j < nJ; ++j)
    if (J[j] < 0 || J[j] >= s->D) return fail(s, RS_ERR_ARG, "column index out of range");
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  rc = upload_geometry(s);
  if (rc != RS_OK) return rc;
  if (!nI || !nJ) return RS_OK;
  DevBuf<int> dI, dJ;
  DevBuf<double> dO;
  CU(dI.ensure(nI));
  CU(dJ.ensure(nJ));
  CU(dO.ensure((size_t)nI * nJ));
  CU(cudaMemcpyAsync(dI.p, I, nI * 4, cudaMemcpyHostToDevice, s->stream));
  CU(cudaMemcpyAsync(dJ.p, J, nJ * 4, cudaMemcpyHostToDevice, s->stream));
  launch_kernel_block(geo_of(s), s->cfg.pde, s->sd, dI.p, nI, dJ.p, nJ, dO.p, s->stream);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(out, dO.p, (size_t)nI * nJ * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

rs_status rs_matvec(rs_solver* s, const double* x, int nrhs, double* y) {
  if (!s || !x || !y || nrhs < 1) return fail(s, RS_ERR_ARG, "bad matvec arguments");
  if (s->n <= 0) return fail(s, RS_ERR_STATE, "no geometry");
  if (s->nprob > 1) return fail(s, RS_ERR_ARG, "dense product of a batch (use rs_matvec_fast)");
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  rc = upload_geometry(s);
  if (rc != RS_OK) return rc;
  const size_t nd = (size_t)s->D * nrhs;
  DevBuf<double> dx, dy;
  CU(dx.ensure(nd));
  CU(dy.ensure(nd));
  CU(cudaMemcpyAsync(dx.p, x, nd * 8, cudaMemcpyHostToDevice, s->stream));
  launch_matvec(geo_of(s), s->cfg.pde, s->sd, s->n, dx.p, nrhs, dy.p, s->stream);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(y, dy.p, nd * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

rs_status rs_matvec_fast(rs_solver* s, const double* x, int nrhs, double* y, int arith) {
  if (!s || !x || !y || nrhs < 1 || arith < 0 || arith > 2)
    return fail(s, RS_ERR_ARG, "bad matvec arguments");
  if (s->n <= 0) return fail(s, RS_ERR_STATE, "no geometry");
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  rc = upload_geometry(s);
  if (rc != RS_OK) return rc;
  if (!s->tree_built) {
    rc = rs_build_tree(s);
    if (rc != RS_OK) return rc;
  }
  if (!s->fmm.built) {
    rc = build_fmm(s);
    if (rc != RS_OK) return rc;
  }
  const size_t nd = (size_t)s->D * nrhs;
  DevBuf<double> dx, dy;
  CU(dx.ensure(nd));
  CU(dy.ensure(nd));
  CU(cudaMemcpyAsync(dx.p, x, nd * 8, cudaMemcpyHostToDevice, s->stream));
  if (!fmm_set_order32(s->fmm, fmm32_fixed(s))) return fail(s, RS_ERR_ARG, "bad FP32 multipole order");
  CU(fmm_apply(s->fmm, s->cfg.pde, geo_of(s), dx.p, nrhs, dy.p, 0.0, 1.0, arith, s->stream));
  CU(cudaMemcpyAsync(y, dy.p, nd * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

rs_status rs_domain_eval(rs_solver* s, int num_targets, const double* targets,
                         const unsigned char* in_domain, const double* mu, const double* alpha,
                         int nrhs, double* out) {
  if (!s || num_targets < 0 || (num_targets > 0 && !targets) || !mu || !out || nrhs < 1)
    return fail(s, RS_ERR_ARG, "bad domain evaluation arguments");
  if (s->n <= 0) return fail(s, RS_ERR_STATE, "no geometry");
  if (s->nprob > 1) return fail(s, RS_ERR_ARG, "domain evaluation of a batch");
  const int nb = (s->nh > 0 && s->cfg.pde != kLaplaceNeumann)
                     ? (s->cfg.pde == kStokes ? 3 * s->nh : s->nh) : 0;
  if (nb > 0 && !alpha) return fail(s, RS_ERR_ARG, "holes need alpha");
  if (num_targets == 0) return RS_OK;
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  rc = upload_geometry(s);
  if (rc != RS_OK) return rc;
  const int sd = s->sd, D = s->D, nt = num_targets;
  std::vector<double> txy(2 * (size_t)nt);
  for (int i = 0; i < nt; ++i) {
    txy[i] = targets[2 * i];
    txy[nt + i] = targets[2 * i + 1];
  }
  DevBuf<double> dt, dmu, dal, dhc, dout;
  DevBuf<unsigned char> dmask;
  CU(dt.ensure(2 * (size_t)nt));
  CU(dmu.ensure((size_t)D * nrhs));
  CU(dout.ensure((size_t)nt * sd * nrhs));
  CU(cudaMemcpyAsync(dt.p, txy.data(), 2 * (size_t)nt * 8, cudaMemcpyHostToDevice, s->stream));
  CU(cudaMemcpyAsync(dmu.p, mu, (size_t)D * nrhs * 8, cudaMemcpyHostToDevice, s->stream));
  if (in_domain) {
    CU(dmask.ensure(nt));
    CU(cudaMemcpyAsync(dmask.p, in_domain, nt, cudaMemcpyHostToDevice, s->stream));
  }
  if (nb > 0) {
    CU(dal.ensure((size_t)nb * nrhs));
    CU(dhc.ensure(2 * (size_t)s->nh));
    CU(cudaMemcpyAsync(dal.p, alpha, (size_t)nb * nrhs * 8, cudaMemcpyHostToDevice, s->stream));
    CU(cudaMemcpyAsync(dhc.p, s->hc.data(), 2 * (size_t)s->nh * 8, cudaMemcpyHostToDevice,
                       s->stream));
  }
  DomainParams p{};
  p.g = geo_of(s);
  p.n = s->n;
  p.sd = sd;
  p.pde = s->cfg.pde;
  p.tx = dt.p;
  p.ty = dt.p + nt;
  p.mask = in_domain ? dmask.p : nullptr;
  p.nt = nt;
  p.mu = dmu.p;
  p.ldmu = D;
  p.alpha = nb > 0 ? dal.p : nullptr;
  p.ldal = nb;
  p.hc = nb > 0 ? dhc.p : nullptr;
  p.nh = nb > 0 ? s->nh : 0;
  p.out = dout.p;
  p.ldo = nt * sd;
  CU(launch_domain_eval(p, nrhs, s->stream));
  CU(cudaMemcpyAsync(out, dout.p, (size_t)nt * sd * nrhs * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

rs_status rs_id_batched(rs_solver* s, int count, const double* mats, const int64_t* a_off,
                        const int* m, const int* n, double tol, int* ranks, int* perm,
                        const int64_t* p_off, double* Z, const int64_t* z_off) {
  if (!s || count < 0 || (count && (!mats || !a_off || !m || !n || !ranks || !perm || !p_off ||
                                    !Z || !z_off)) ||
      !(tol > 0))
    return fail(s, RS_ERR_ARG, "bad id arguments");
  if (!count) return RS_OK;
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  int64_t a_tot = 0, p_tot = 0, z_tot = 0;
  std::vector<IdTask> tasks(count);
  size_t scratch = 0;
  for (int i = 0; i < count; ++i) {
    if (m[i] < 1 || n[i] < 1 || n[i] > 4096) return fail(s, RS_ERR_ARG, "bad matrix size");
    a_tot = std::max<int64_t>(a_tot, a_off[i] + (int64_t)m[i] * n[i]);
    p_tot = std::max<int64_t>(p_tot, p_off[i] + n[i]);
    z_tot = std::max<int64_t>(z_tot, z_off[i] + (int64_t)n[i] * n[i]);
    IdTask& t = tasks[i];
    t = IdTask{};
    t.n = n[i];
    t.act_off = (int)p_off[i];
    t.slot = i;
    t.fac_off = z_off[i];
    t.scratch_off = -1;
    t.dense_off = a_off[i];
    t.m_dense = m[i];
  }
  std::vector<size_t> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return tasks[a].n < tasks[b].n; });
  std::vector<IdTask> sorted(count);
  for (int i = 0; i < count; ++i) sorted[i] = tasks[order[i]];
  for (IdTask& t : sorted)
    if (id_kernel_smem(t.n, false, true) > kSmemMax) {
      t.scratch_off = (int64_t)scratch;
      scratch += (size_t)(t.n + 32) * (t.n + 64) + 64;
    }
  DevBuf<double> dA, dZ, dS;
  DevBuf<int> dP, dR;
  DevBuf<IdTask> dT;
  CU(dA.ensure(a_tot));
  CU(dZ.ensure(z_tot));
  CU(dS.ensure(std::max<size_t>(scratch, 1)));
  CU(dP.ensure(p_tot));
  CU(dR.ensure(count));
  CU(dT.ensure(count));
  CU(cudaMemcpyAsync(dA.p, mats, a_tot * 8, cudaMemcpyHostToDevice, s->stream));
  CU(cudaMemsetAsync(dZ.p, 0, z_tot * 8, s->stream));
  CU(cudaMemcpyAsync(dT.p, sorted.data(), count * sizeof(IdTask), cudaMemcpyHostToDevice, s->stream));
  IdParams ip{};
  ip.tol = tol;
  ip.ranks = dR.p;
  ip.perm = dP.p;
  ip.fac = dZ.p;
  ip.scratch = dS.p;
  ip.dense = dA.p;
  ip.direct = 0;
  ip.phase_clk = nullptr;
  ip.sd = 1;
  ip.npp = 1;
  auto id_fits = [&](int nn) { return id_kernel_smem(nn, false, true) <= kSmemMax; };
  launch_binned(sorted, dT.p, id_fits, [&](const IdTask* dt, int cnt, int nmax) {
    IdParams q = ip;
    q.tasks = dt;
    bool in_smem = id_kernel_smem(nmax, false, true) <= kSmemMax;
    launch_id(q, cnt, nmax, id_kernel_smem(nmax, false, in_smem), false, s->stream);
  });
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(ranks, dR.p, count * 4, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaMemcpyAsync(perm, dP.p, p_tot * 4, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaMemcpyAsync(Z, dZ.p, z_tot * 8, cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

rs_status rs_get_stats(const rs_solver* s, rs_stats* out) {
  if (!s || !out) return RS_ERR_ARG;
  *out = s->stats;
  out->kernel_launches = s->launches;
  out->host_plan_ms = s->host_plan_ms;
  out->host_wait_ms = s->host_wait_ms;
  out->host_post_ms = s->host_post_ms;
  out->residual64_ms = s->stats.residual64_ms;
  out->residual32_ms = s->stats.residual32_ms;
  return RS_OK;
}

rs_status rs_autotune(rs_solver* s, int reps, int* split_min_tasks, int* wide_ctas_per_sm,
                      int* elim_threads) {
  if (!s || reps < 1) return RS_ERR_ARG;
  // each candidate: the median device time of `reps` factorizations of the
  // handle's geometry; one knob at a time, the other at its current value.
  // An FP32 factorization is timed with one refined solve after it: the
  // launch shapes change the factorization's rounding, and with it the
  // number of refinement steps a solve takes, which can cost more than a
  // faster factorization saves.  The data are kTuneRhs columns of the
  // potential of a point source, log |x - c_q|, at points c_q on the circle
  // of 1.25 times the half-diagonal of the geometry's bounding box around
  // its centre, outside the geometry (the same in every component for
  // Stokes): close enough to the boundary to show the factorization's
  // accuracy, as a solve's own data do.
  rs_status rc = rs_factor(s);  // warm-up (plans, buffers, first launches)
  if (rc != RS_OK) return rc;
  const bool with_solve = s->fp32;
  constexpr int kTuneRhs = 8;
  DevBuf<double> df, dmu, dal;
  if (with_solve) {
    double x0 = s->pts[0], x1 = x0, y0 = s->pts[1], y1 = y0;
    for (int p = 0; p < s->n; ++p) {
      x0 = std::min(x0, s->pts[2 * p]);
      x1 = std::max(x1, s->pts[2 * p]);
      y0 = std::min(y0, s->pts[2 * p + 1]);
      y1 = std::max(y1, s->pts[2 * p + 1]);
    }
    const double cx = 0.5 * (x0 + x1), cy = 0.5 * (y0 + y1);
    const double rad = 1.25 * std::max(0.5 * std::hypot(x1 - x0, y1 - y0), 1e-300);
    std::vector<double> f((size_t)s->D * kTuneRhs);
    for (int q = 0; q < kTuneRhs; ++q) {
      const double a = 0.3 + 2.0 * 3.14159265358979323846 * q / kTuneRhs;
      const double sx = cx + rad * std::cos(a), sy = cy + rad * std::sin(a);
      for (int i = 0; i < s->D; ++i) {
        const int pt = i / s->sd;
        f[i + (size_t)s->D * q] = std::log(std::hypot(s->pts[2 * pt] - sx, s->pts[2 * pt + 1] - sy));
      }
    }
    CU(df.ensure(f.size()));
    CU(dmu.ensure(f.size()));
    CU(dal.ensure(std::max<size_t>((size_t)s->nb * kTuneRhs, 1)));
    CU(cudaMemcpy(df.p, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  auto time_factor = [&](double* ms) -> rs_status {
    std::vector<double> t;
    for (int r = 0; r < reps; ++r) {
      rs_status rc2 = rs_factor(s);
      if (rc2 != RS_OK) return rc2;
      double m = s->stats.dev_factor_ms;
      if (with_solve) {
        rc2 = rs_solve_device(s, df.p, kTuneRhs, dmu.p, dal.p);
        if (rc2 != RS_OK) return rc2;
        CU(cudaStreamSynchronize(s->stream));
        float sm = 0;
        CU(cudaEventElapsedTime(&sm, s->ev_f0, s->ev_f1));
        m += sm;
      }
      t.push_back(m);
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return RS_OK;
  };
  double best = 1e300;
  int best_split = s->split_min_tasks;
  for (int cand : {1, 32, 128, 256, 512, 1024, 1 << 30}) {
    s->split_min_tasks = cand;
    double ms = 0;
    RSCHK(time_factor(&ms));
    if (ms < best) {
      best = ms;
      best_split = cand;
    }
  }
  s->split_min_tasks = best_split;
  best = 1e300;
  int best_wide = s->wide_ctas_per_sm;
  for (int cand : {1, 2, 4}) {
    s->wide_ctas_per_sm = cand;
    double ms = 0;
    RSCHK(time_factor(&ms));
    if (ms < best) {
      best = ms;
      best_wide = cand;
    }
  }
  s->wide_ctas_per_sm = best_wide;
  best = 1e300;
  int best_elim = s->elim_threads;
  for (int cand : {0, 256, 128}) {
    s->elim_threads = cand;
    double ms = 0;
    RSCHK(time_factor(&ms));
    if (ms < best) {
      best = ms;
      best_elim = cand;
    }
  }
  s->elim_threads = best_elim;
  s->factored = false;  // the last candidate's factors are not the chosen shape's
  if (split_min_tasks) *split_min_tasks = s->split_min_tasks;
  if (wide_ctas_per_sm) *wide_ctas_per_sm = s->wide_ctas_per_sm;
  if (elim_threads) *elim_threads = s->elim_threads;
  return RS_OK;
}

static_assert(kRankFeatures == RS_RANK_FEATURES && kRankWeights == RS_RANK_WEIGHTS,
              "rank model sizes of rskel.h and rank_model.hpp differ");

void rs_rank_model_init(uint64_t seed, float* weights) {
  if (!weights) return;
  uint64_t x = seed + 0x9E3779B97F4A7C15ull;
  auto uni = [&x]() {  // splitmix64 -> uniform in [-1, 1)
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0);
  };
  const int H = kRankHidden, F = kRankFeatures;
  float* w = weights;
  const float a1 = std::sqrt(6.f / F), a2 = std::sqrt(6.f / H), a3 = std::sqrt(1.f / H);
  for (int e = 0; e < H * F; ++e) *w++ = a1 * uni();
  for (int e = 0; e < H; ++e) *w++ = 0.f;
  for (int e = 0; e < H * H; ++e) *w++ = a2 * uni();
  for (int e = 0; e < H; ++e) *w++ = 0.f;
  for (int e = 0; e < H; ++e) *w++ = a3 * uni();
  *w++ = 0.f;
}

rs_status rs_set_rank_model(rs_solver* s, const float* weights) {
  if (!s) return RS_ERR_ARG;
  if (!weights) {
    s->rank_model_on = false;
    return RS_OK;
  }
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  CU(cudaSetDevice(s->cfg.device));
  CU(s->rank_w.ensure(kRankWeights));
  CU(cudaMemcpyAsync(s->rank_w.p, weights, sizeof(float) * kRankWeights, cudaMemcpyHostToDevice,
                     s->stream));
  CU(cudaStreamSynchronize(s->stream));
  s->rank_model_on = true;
  return RS_OK;
}

rs_status rs_rank_samples(const rs_solver* s, float* features, float* targets, int cap,
                          int* count) {
  if (!s || !count || cap < 0 || (cap > 0 && (!features || !targets))) return RS_ERR_ARG;
  const int n = (int)s->samp_target.size();
  *count = n;
  const int w = std::min(n, cap);
  if (w > 0) {
    // the features of each sample's box, from its lists as the factorization
    // left them (the same values the planning computes for a rank model)
    const int prow = (s->cfg.pde == kStokes ? 2 : 1) * s->cfg.num_proxy_points;
#pragma omp parallel for schedule(dynamic, 64) if (w > 256)
    for (int i = 0; i < w; ++i) {
      const int id = s->samp_box[i];
      const NodeState& S = s->st[id];
      const int m = 2 * (int)S.rows.size() + (S.use_proxy ? 2 * prow : 0);
      rank_features(s, s->tree.nodes[id], S, m, s->samp_tol, features + (size_t)i * kRankFeatures);
    }
    std::memcpy(targets, s->samp_target.data(), sizeof(float) * (size_t)w);
  }
  return RS_OK;
}

// Device copies of a training set for the rank-model entry points.
struct RankSet {
  DevBuf<float> w, x, y, g, m, v, loss, part;
};

static rs_status rank_upload(rs_solver* s, RankSet& R, const float* weights,
                             const float* features, const float* targets, int count) {
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  CU(cudaSetDevice(s->cfg.device));
  CU(R.w.ensure(kRankWeights));
  CU(R.g.ensure(kRankWeights));
  CU(R.loss.ensure(1));
  CU(R.x.ensure((size_t)count * kRankFeatures));
  CU(cudaMemcpyAsync(R.w.p, weights, sizeof(float) * kRankWeights, cudaMemcpyHostToDevice,
                     s->stream));
  CU(cudaMemcpyAsync(R.x.p, features, sizeof(float) * kRankFeatures * (size_t)count,
                     cudaMemcpyHostToDevice, s->stream));
  if (targets) {
    CU(R.y.ensure(count));
    CU(cudaMemcpyAsync(R.y.p, targets, sizeof(float) * (size_t)count, cudaMemcpyHostToDevice,
                       s->stream));
  }
  return RS_OK;
}

rs_status rs_rank_train(rs_solver* s, const float* features, const float* targets, int count,
                        int epochs, float lr, float* weights, float* loss) {
  if (!s || !features || !targets || !weights || count < 1 || epochs < 1 || !(lr > 0))
    return RS_ERR_ARG;
  RankSet R;
  RSCHK(rank_upload(s, R, weights, features, targets, count));
  CU(R.m.ensure(kRankWeights));
  CU(R.v.ensure(kRankWeights));
  CU(cudaMemsetAsync(R.m.p, 0, sizeof(float) * kRankWeights, s->stream));
  CU(cudaMemsetAsync(R.v.p, 0, sizeof(float) * kRankWeights, s->stream));
  CU(R.part.ensure(rank_gradient_scratch(count)));
  for (int e = 1; e <= epochs; ++e) {
    CU(rank_gradient(R.w.p, R.x.p, R.y.p, count, R.g.p, R.loss.p, R.part.p, s->stream));
    CU(rank_adam(R.w.p, R.g.p, R.m.p, R.v.p, e, lr, s->stream));
  }
  float ls = 0;
  CU(cudaMemcpyAsync(weights, R.w.p, sizeof(float) * kRankWeights, cudaMemcpyDeviceToHost,
                     s->stream));
  CU(cudaMemcpyAsync(&ls, R.loss.p, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  if (loss) *loss = ls / (float)count;
  return RS_OK;
}

rs_status rs_rank_predict(rs_solver* s, const float* weights, const float* features, int count,
                          float* out) {
  if (!s || !weights || !features || !out || count < 0) return RS_ERR_ARG;
  if (count == 0) return RS_OK;
  RankSet R;
  RSCHK(rank_upload(s, R, weights, features, nullptr, count));
  CU(R.y.ensure(count));
  CU(rank_predict(R.w.p, R.x.p, count, R.y.p, s->stream));
  CU(cudaMemcpyAsync(out, R.y.p, sizeof(float) * (size_t)count, cudaMemcpyDeviceToHost,
                     s->stream));
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

rs_status rs_rank_gradient(rs_solver* s, const float* weights, const float* features,
                           const float* targets, int count, float* grad, float* loss) {
  if (!s || !weights || !features || !targets || !grad || count < 1) return RS_ERR_ARG;
  RankSet R;
  RSCHK(rank_upload(s, R, weights, features, targets, count));
  CU(R.part.ensure(rank_gradient_scratch(count)));
  CU(rank_gradient(R.w.p, R.x.p, R.y.p, count, R.g.p, R.loss.p, R.part.p, s->stream));
  float ls = 0;
  CU(cudaMemcpyAsync(grad, R.g.p, sizeof(float) * kRankWeights, cudaMemcpyDeviceToHost,
                     s->stream));
  CU(cudaMemcpyAsync(&ls, R.loss.p, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  CU(cudaStreamSynchronize(s->stream));
  if (loss) *loss = ls / (float)count;
  return RS_OK;
}

rs_status rs_node_info(const rs_solver* s, int node, int* info, double* corners8, double* side) {
  if (!s || !info || !s->tree_built) return RS_ERR_ARG;
  if (node < 0 || node >= (int)s->tree.level_order.size()) return RS_ERR_ARG;
  const int id = s->tree.level_order[node];
  const TreeNode& nd = s->tree.nodes[id];
  info[0] = nd.level;
  info[1] = nd.is_leaf;
  info[2] = nd.parent >= 0 ? s->tree.level_rank[nd.parent] : -1;
  for (int c = 0; c < 4; ++c) info[3 + c] = nd.children[c] >= 0 ? s->tree.level_rank[nd.children[c]] : -1;
  const bool have = id < (int)s->st.size();
  info[7] = have ? s->st[id].compressed : 0;
  info[8] = have ? (int)s->st[id].skel.size() : 0;
  info[9] = have ? (int)s->st[id].red.size() : 0;
  if (corners8) std::memcpy(corners8, nd.corners, sizeof(nd.corners));
  if (side) *side = nd.side;
  return RS_OK;
}

rs_status rs_node_list(const rs_solver* s, int node, int which, int* out, int cap, int* len) {
  if (!s || !s->tree_built || !len) return RS_ERR_ARG;
  if (node < 0 || node >= (int)s->tree.level_order.size()) return RS_ERR_ARG;
  const int id = s->tree.level_order[node];
  const TreeNode& nd = s->tree.nodes[id];
  std::vector<int> tmp;
  const std::vector<int>* src = nullptr;
  const bool have = id < (int)s->st.size();
  static const std::vector<int> empty;
  switch (which) {
    case 0:
      tmp = s->tree.box_dofs(id);
      src = &tmp;
      break;
    case 1: src = have ? &s->st[id].active : &empty; break;
    case 2: src = have ? &s->st[id].skel : &empty; break;
    case 3: src = have ? &s->st[id].red : &empty; break;
    case 4: src = have ? &s->st[id].near_ : &empty; break;
    case 5:
      for (int x : nd.neighbors) tmp.push_back(s->tree.level_rank[x]);
      src = &tmp;
      break;
    case 6: src = have ? &s->st[id].perm : &empty; break;
    default: return RS_ERR_ARG;
  }
  *len = (int)src->size();
  if (out)
    for (int i = 0; i < *len && i < cap; ++i) out[i] = (*src)[i];
  return RS_OK;
}

rs_status rs_tree_bounds(const rs_solver* s, double* mn, double* mx) {
  if (!s || !s->tree_built) return RS_ERR_ARG;
  if (mn) *mn = s->tree.min;
  if (mx) *mx = s->tree.max;
  return RS_OK;
}

rs_status rs_allskel(const rs_solver* s, int* out, int cap, int* len) {
  if (!s || !len) return RS_ERR_ARG;
  *len = (int)s->allskel.size();
  if (out)
    for (int i = 0; i < *len && i < cap; ++i) out[i] = s->allskel[i];
  return RS_OK;
}

rs_status rs_timer_start(rs_solver* s) {
  if (!s) return RS_ERR_ARG;
  rs_status rc = ensure_device(s);
  if (rc != RS_OK) return rc;
  CU(cudaEventRecord(s->ev_t0, s->stream));
  return RS_OK;
}

rs_status rs_timer_stop(rs_solver* s, float* ms) {
  if (!s || !ms || !s->dev_ready) return RS_ERR_ARG;
  CU(cudaEventRecord(s->ev_t1, s->stream));
  CU(cudaEventSynchronize(s->ev_t1));
  CU(cudaEventElapsedTime(ms, s->ev_t0, s->ev_t1));
  return RS_OK;
}

rs_status rs_synchronize(rs_solver* s) {
  if (!s) return RS_ERR_ARG;
  if (!s->dev_ready) return RS_OK;
  CU(cudaStreamSynchronize(s->stream));
  return RS_OK;
}

const char* rs_last_error(const rs_solver* s) {
  static const char* none = "";
  return s ? s->err.c_str() : none;
}

}  // extern "C"
