"""ctypes binding of the solver's C ABI (include/rskel.h).

This is the Python-side caller of the C ABI, used by the tests and the
benchmark; it mirrors the reference's solve flow (build tree, skeletonize,
linear_solve).  Every call goes to the CUDA library; there is no CPU path:
if ``lib/librskel.so`` is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "librskel.so")

RS_LAPLACE, RS_LAPLACE_NEUMANN, RS_STOKES = 0, 1, 2
RS_FP64, RS_FP32_REFINE = 0, 1

STATUS = {0: "RS_OK", 1: "RS_ERR_ARG", 2: "RS_ERR_STATE", 3: "RS_ERR_CUDA",
          4: "RS_ERR_NO_DEVICE", 5: "RS_ERR_CAPACITY", 6: "RS_ERR_NUMERIC",
          7: "RS_ERR_NO_COMPRESSION"}

# Every function the C ABI exports (include/rskel.h).
EXPORTS = ["rs_config_default", "rs_create", "rs_destroy", "rs_set_geometry", "rs_perturb",
           "rs_set_geometry_batch", "rs_autotune",
           "rs_build_tree",
           "rs_factor", "rs_solve", "rs_solve_device", "rs_kernel_block", "rs_matvec",
           "rs_matvec_fast", "rs_domain_eval",
           "rs_id_batched", "rs_id_noalloc", "rs_barrier_selftest", "rs_rank_model_init", "rs_set_rank_model",
           "rs_rank_samples", "rs_rank_train", "rs_rank_predict", "rs_rank_gradient",
           "rs_get_stats", "rs_node_info", "rs_node_list", "rs_tree_bounds",
           "rs_allskel", "rs_timer_start", "rs_timer_stop", "rs_synchronize", "rs_last_error"]


class RsConfig(ctypes.Structure):
    _fields_ = [("pde", ctypes.c_int), ("solution_dimension", ctypes.c_int),
                ("domain_dimension", ctypes.c_int), ("id_tol", ctypes.c_double),
                ("max_leaf_dofs", ctypes.c_int), ("num_proxy_points", ctypes.c_int),
                ("radius_ratio", ctypes.c_double), ("min_dofs_to_compress", ctypes.c_int),
                ("is_strong_admissibility", ctypes.c_int), ("precision", ctypes.c_int),
                ("refine_tol", ctypes.c_double), ("refine_max_iters", ctypes.c_int),
                ("fp32_id_tol", ctypes.c_double), ("device", ctypes.c_int),
                ("fmm_order", ctypes.c_int), ("rank_headroom", ctypes.c_double),
                ("rank_extra_rows", ctypes.c_int), ("refine_verify", ctypes.c_int),
                ("refine_solver", ctypes.c_int), ("use_graphs", ctypes.c_int),
                ("root_inverse", ctypes.c_int), ("rank_judge", ctypes.c_double),
                ("tensor_cores", ctypes.c_int),
                ("id_row_groups", ctypes.c_int), ("fmm_order32", ctypes.c_int)]


class RsStats(ctypes.Structure):
    _fields_ = [("num_levels", ctypes.c_int), ("num_nodes", ctypes.c_int),
                ("num_compressed", ctypes.c_int), ("num_skel_root", ctypes.c_int),
                ("max_active", ctypes.c_int), ("max_rank", ctypes.c_int),
                ("max_rows", ctypes.c_int),
                ("t_tree_ms", ctypes.c_double), ("t_factor_ms", ctypes.c_double),
                ("t_solve_ms", ctypes.c_double), ("dev_factor_ms", ctypes.c_double),
                ("dev_solve_ms", ctypes.c_double), ("id_flops", ctypes.c_double),
                ("decouple_flops", ctypes.c_double), ("solve_bytes", ctypes.c_double),
                ("id_ms", ctypes.c_double), ("decouple_ms", ctypes.c_double),
                ("refine_iters", ctypes.c_int), ("refine_residual", ctypes.c_double),
                ("kernel_launches", ctypes.c_int), ("host_plan_ms", ctypes.c_double),
                ("host_wait_ms", ctypes.c_double), ("host_post_ms", ctypes.c_double),
                ("boxes_factored", ctypes.c_int),
                ("residual64_ms", ctypes.c_double), ("residual32_ms", ctypes.c_double),
                ("rank_predicted", ctypes.c_int), ("rank_redo", ctypes.c_int),
                ("sketch_rows", ctypes.c_double), ("krylov_steps", ctypes.c_int),
                ("rank_redo_judge", ctypes.c_int), ("level_gap_ms", ctypes.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


def openmp_spin_default():
    """The library's host planner runs a few short OpenMP regions per tree
    level, between waits of 0.1-0.3 ms on the GPU; with libgomp's default
    spin count its threads fall asleep in those waits and every region then
    pays their wake-up.  Unless the caller chose a policy, let them spin up
    to 1e8 iterations (a fraction of a second) before sleeping: measured on
    the 65536-point star, the factorization's device time 2.95 -> 2.74 ms in
    steady state and 3.98 -> 2.58 ms after a new geometry.  libgomp reads the
    setting when it is loaded, so this runs before the library is."""
    if "OMP_WAIT_POLICY" not in os.environ:
        os.environ.setdefault("GOMP_SPINCOUNT", "100000000")


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        openmp_spin_default()
        L = ctypes.CDLL(LIB_PATH)
        L.rs_config_default.argtypes = [ctypes.POINTER(RsConfig)]
        L.rs_config_default.restype = None
        L.rs_create.argtypes = [ctypes.POINTER(RsConfig), ctypes.POINTER(_vp)]
        L.rs_destroy.argtypes = [_vp]
        L.rs_set_geometry.argtypes = [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp]
        L.rs_perturb.argtypes = [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp]
        L.rs_set_geometry_batch.argtypes = [_vp, ctypes.c_int, _ip, _dp, _dp, _dp, _dp]
        L.rs_autotune.argtypes = [_vp, ctypes.c_int, _ip, _ip, _ip]
        L.rs_build_tree.argtypes = [_vp]
        L.rs_factor.argtypes = [_vp]
        L.rs_solve.argtypes = [_vp, _dp, ctypes.c_int, _dp, _dp]
        L.rs_solve_device.argtypes = [_vp, _vp, ctypes.c_int, _vp, _vp]
        L.rs_kernel_block.argtypes = [_vp, _ip, ctypes.c_int, _ip, ctypes.c_int, _dp]
        L.rs_matvec.argtypes = [_vp, _dp, ctypes.c_int, _dp]
        L.rs_matvec_fast.argtypes = [_vp, _dp, ctypes.c_int, _dp, ctypes.c_int]
        L.rs_id_batched.argtypes = [_vp, ctypes.c_int, _dp, _lp, _ip, _ip, ctypes.c_double, _ip,
                                    _ip, _lp, _dp, _lp]
        L.rs_domain_eval.argtypes = [_vp, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_ubyte), _dp,
                                     _dp, ctypes.c_int, _dp]
        L.rs_id_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, _vp, ctypes.c_double, _vp, _vp, _vp,
                                    _vp]
        L.rs_barrier_selftest.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_int,
                                          _ip, _ip, _ip, ctypes.POINTER(ctypes.c_float)]
        _fp = ctypes.POINTER(ctypes.c_float)
        L.rs_rank_model_init.argtypes = [ctypes.c_uint64, _fp]
        L.rs_rank_model_init.restype = None
        L.rs_set_rank_model.argtypes = [_vp, _fp]
        L.rs_rank_samples.argtypes = [_vp, _fp, _fp, ctypes.c_int, _ip]
        L.rs_rank_train.argtypes = [_vp, _fp, _fp, ctypes.c_int, ctypes.c_int, ctypes.c_float, _fp,
                                    _fp]
        L.rs_rank_predict.argtypes = [_vp, _fp, _fp, ctypes.c_int, _fp]
        L.rs_rank_gradient.argtypes = [_vp, _fp, _fp, _fp, ctypes.c_int, _fp, _fp]
        L.rs_get_stats.argtypes = [_vp, ctypes.POINTER(RsStats)]
        L.rs_node_info.argtypes = [_vp, ctypes.c_int, _ip, _dp, _dp]
        L.rs_node_list.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int, _ip]
        L.rs_tree_bounds.argtypes = [_vp, _dp, _dp]
        L.rs_allskel.argtypes = [_vp, _ip, ctypes.c_int, _ip]
        L.rs_timer_start.argtypes = [_vp]
        L.rs_timer_stop.argtypes = [_vp, ctypes.POINTER(ctypes.c_float)]
        L.rs_synchronize.argtypes = [_vp]
        L.rs_last_error.argtypes = [_vp]
        L.rs_last_error.restype = ctypes.c_char_p
        for fn in EXPORTS:
            f = getattr(L, fn)
            if fn not in ("rs_config_default", "rs_last_error", "rs_rank_model_init"):
                f.restype = ctypes.c_int
        _lib = L
    return _lib


class RsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _l(a):
    return a.ctypes.data_as(_lp)


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


RANK_FEATURES, RANK_HIDDEN = 16, 64
RANK_WEIGHTS = RANK_HIDDEN * RANK_FEATURES + RANK_HIDDEN + RANK_HIDDEN * RANK_HIDDEN + \
    RANK_HIDDEN + RANK_HIDDEN + 1


def rank_model_init(seed=0):
    """rs_rank_model_init: deterministic initial weights of the rank model."""
    w = np.zeros(RANK_WEIGHTS, dtype=np.float32)
    lib().rs_rank_model_init(seed, _f(w))
    return w


def rank_unpack(w):
    """Splits a weight vector into (W1 [64x16], b1, W2 [64x64], b2, w3, b3)."""
    H, F = RANK_HIDDEN, RANK_FEATURES
    o = 0
    out = []
    for shape in ((H, F), (H,), (H, H), (H,), (H,), (1,)):
        sz = int(np.prod(shape))
        out.append(np.asarray(w[o:o + sz]).reshape(shape))
        o += sz
    return out


def default_config(**kw):
    c = RsConfig()
    lib().rs_config_default(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


LISTS = {"original": 0, "active": 1, "skel": 2, "redundant": 3, "near": 4, "neighbors": 5,
         "permutation": 6}


class Solver:
    """One boundary problem: geometry -> quadtree -> factor -> solves."""

    def __init__(self, geo, pde, tol, leaf=64, npp=64, precision=RS_FP64, refine_tol=1e-12,
                 refine_max_iters=10, fp32_id_tol=1e-6, device=0, min_dofs=16, fmm_order=0,
                 rank_headroom=1.25, rank_extra_rows=12, refine_verify=1, refine_solver=0,
                 use_graphs=1, root_inverse=1, rank_judge=4.0, tensor_cores=1,
                 id_row_groups=-1, fmm_order32=0):
        self.sd = 2 if pde == RS_STOKES else 1
        self.cfg = default_config(pde=pde, solution_dimension=self.sd, id_tol=tol,
                                  max_leaf_dofs=leaf, num_proxy_points=npp,
                                  precision=precision, refine_tol=refine_tol,
                                  refine_max_iters=refine_max_iters, fp32_id_tol=fp32_id_tol,
                                  device=device, min_dofs_to_compress=min_dofs,
                                  fmm_order=fmm_order, rank_headroom=rank_headroom,
                                  rank_extra_rows=rank_extra_rows, refine_verify=refine_verify,
                                  refine_solver=refine_solver, use_graphs=use_graphs,
                                  root_inverse=root_inverse, rank_judge=rank_judge,
                                  tensor_cores=tensor_cores, id_row_groups=id_row_groups,
                                  fmm_order32=fmm_order32)
        h = _vp()
        self._check(lib().rs_create(ctypes.byref(self.cfg), ctypes.byref(h)), None)
        self.h = h
        self.pde = pde
        self.set_geometry(geo)

    def set_geometry(self, geo, perturb=False):
        """rs_set_geometry: a new boundary for this handle (tree and factors
        reset); with perturb=True rs_perturb, which keeps what it can."""
        self.n = geo.n
        self.D = geo.n * self.sd
        self.nh = geo.num_holes
        self.nb = 0 if geo.num_holes == 0 or self.pde == RS_LAPLACE_NEUMANN else (
            3 * geo.num_holes if self.pde == RS_STOKES else geo.num_holes)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in
                (geo.points, geo.normals, geo.weights, geo.curvatures)]
        hc = np.ascontiguousarray(geo.hole_centers if geo.num_holes else np.zeros(2))
        hr = np.ascontiguousarray(geo.hole_radii if geo.num_holes else np.zeros(1))
        fn = lib().rs_perturb if perturb else lib().rs_set_geometry
        self._check(fn(self.h, geo.n, _d(arrs[0]), _d(arrs[1]), _d(arrs[2]), _d(arrs[3]),
                       geo.num_holes, _d(hc), _d(hr)))

    def set_geometry_batch(self, geos):
        """rs_set_geometry_batch: independent boundaries (no holes) in one
        handle; vectors are the boundaries' vectors concatenated in order."""
        assert all(g.num_holes == 0 for g in geos)
        counts = np.array([g.n for g in geos], dtype=np.int32)
        self.n = int(counts.sum())
        self.D = self.n * self.sd
        self.nh = 0
        self.nb = 0
        self.batch = counts
        arrs = [np.ascontiguousarray(np.concatenate([np.asarray(getattr(g, f)).ravel()
                                                     for g in geos]), dtype=np.float64)
                for f in ("points", "normals", "weights", "curvatures")]
        self._check(lib().rs_set_geometry_batch(self.h, len(geos), _i(counts), _d(arrs[0]),
                                                _d(arrs[1]), _d(arrs[2]), _d(arrs[3])))

    def autotune(self, reps=3):
        """rs_autotune: returns (split_min_tasks, wide_ctas_per_sm,
        elim_threads) chosen."""
        a, b, c = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        self._check(lib().rs_autotune(self.h, reps, ctypes.byref(a), ctypes.byref(b),
                                      ctypes.byref(c)))
        return a.value, b.value, c.value

    def _check(self, rc, h="self"):
        if rc != 0:
            hh = self.h if h == "self" else h
            msg = lib().rs_last_error(hh).decode() if hh is not None else ""
            raise RsError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            lib().rs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_tree(self):
        self._check(lib().rs_build_tree(self.h))

    def factor(self):
        self._check(lib().rs_factor(self.h))

    def solve(self, f):
        f = np.asfortranarray(f, dtype=np.float64)
        squeeze = f.ndim == 1
        if squeeze:
            f = f[:, None]
        assert f.shape[0] == self.D
        mu = np.zeros_like(f, order="F")
        alpha = np.zeros((max(self.nb, 1), f.shape[1]), order="F")
        self._check(lib().rs_solve(self.h, _d(f), f.shape[1], _d(mu), _d(alpha)))
        a = alpha[:self.nb] if self.nb else None
        if squeeze:
            return mu[:, 0], (a[:, 0] if a is not None else None)
        return mu, a

    def solve_device(self, f_ptr, nrhs, mu_ptr, alpha_ptr=0):
        self._check(lib().rs_solve_device(self.h, f_ptr, nrhs, mu_ptr, alpha_ptr))

    # --- learned skeleton ranks (rs_rank_*) ---
    def set_rank_model(self, weights):
        """rs_set_rank_model: predicted sketch sizes for the FP32 ID from the
        next factor() on; None switches them off."""
        if weights is None:
            self._check(lib().rs_set_rank_model(self.h, None))
            return
        w = np.ascontiguousarray(weights, dtype=np.float32)
        assert w.size == RANK_WEIGHTS
        self._check(lib().rs_set_rank_model(self.h, _f(w)))

    def rank_samples(self):
        """(features [count x 16], k/n [count]) of the last factorization."""
        cnt = ctypes.c_int(0)
        self._check(lib().rs_rank_samples(self.h, None, None, 0, ctypes.byref(cnt)))
        X = np.zeros((cnt.value, RANK_FEATURES), dtype=np.float32)
        y = np.zeros(cnt.value, dtype=np.float32)
        if cnt.value:
            self._check(lib().rs_rank_samples(self.h, _f(X), _f(y), cnt.value, ctypes.byref(cnt)))
        return X, y

    def rank_train(self, X, y, weights, epochs=1000, lr=3e-3):
        """rs_rank_train: returns (trained weights, final mean loss)."""
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        w = np.array(weights, dtype=np.float32, copy=True)
        loss = ctypes.c_float(0)
        self._check(lib().rs_rank_train(self.h, _f(X), _f(y), len(y), epochs, lr, _f(w),
                                        ctypes.byref(loss)))
        return w, loss.value

    def rank_predict(self, weights, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        w = np.ascontiguousarray(weights, dtype=np.float32)
        out = np.zeros(len(X), dtype=np.float32)
        self._check(lib().rs_rank_predict(self.h, _f(w), _f(X), len(X), _f(out)))
        return out

    def rank_gradient(self, weights, X, y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        w = np.ascontiguousarray(weights, dtype=np.float32)
        g = np.zeros(RANK_WEIGHTS, dtype=np.float32)
        loss = ctypes.c_float(0)
        self._check(lib().rs_rank_gradient(self.h, _f(w), _f(X), _f(y), len(y), _f(g),
                                           ctypes.byref(loss)))
        return g, loss.value

    def domain_eval(self, targets, mu, alpha=None, in_domain=None):
        """rs_domain_eval: u at interleaved targets (2 nt,) from mu ((n sd) x nrhs)."""
        t = np.ascontiguousarray(targets, dtype=np.float64)
        mu = np.asfortranarray(mu, dtype=np.float64)
        sq = mu.ndim == 1
        if sq:
            mu = mu[:, None]
        nt = t.size // 2
        out = np.zeros((nt * self.sd, mu.shape[1]), order="F")
        mask = None
        if in_domain is not None:
            m = np.ascontiguousarray(in_domain, dtype=np.uint8)
            mask = m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))
        al = None
        if alpha is not None:
            al = np.asfortranarray(alpha, dtype=np.float64)
            if al.ndim == 1:
                al = al[:, None]
        self._check(lib().rs_domain_eval(self.h, nt, _d(t), mask, _d(mu),
                                         _d(al) if al is not None else None, mu.shape[1],
                                         _d(out)))
        return out[:, 0] if sq else out

    def kernel_block(self, I, J):
        I = np.ascontiguousarray(I, dtype=np.int32)
        J = np.ascontiguousarray(J, dtype=np.int32)
        out = np.zeros((I.size, J.size), order="F")
        self._check(lib().rs_kernel_block(self.h, _i(I), I.size, _i(J), J.size, _d(out)))
        return out

    def matvec(self, x, fast=False, fp32=False, arith=None):
        """K x: dense FP64, or (fast=True) through the fast multipole method in
        arithmetic `arith` (0 FP64, 1 FP32, 2 float-float; fp32=True is 1)."""
        x = np.asfortranarray(x, dtype=np.float64)
        sq = x.ndim == 1
        if sq:
            x = x[:, None]
        y = np.zeros_like(x, order="F")
        if fast:
            a = (1 if fp32 else 0) if arith is None else int(arith)
            self._check(lib().rs_matvec_fast(self.h, _d(x), x.shape[1], _d(y), a))
        else:
            self._check(lib().rs_matvec(self.h, _d(x), x.shape[1], _d(y)))
        return y[:, 0] if sq else y

    def stats(self):
        st = RsStats()
        self._check(lib().rs_get_stats(self.h, ctypes.byref(st)))
        return st.as_dict()

    def num_nodes(self):
        return self.stats()["num_nodes"]

    def node_info(self, i):
        info = np.zeros(10, dtype=np.int32)
        cor = np.zeros(8)
        side = np.zeros(1)
        self._check(lib().rs_node_info(self.h, i, _i(info), _d(cor), _d(side)))
        return info, cor, side[0]

    def node_list(self, i, which):
        ln = ctypes.c_int(0)
        self._check(lib().rs_node_list(self.h, i, LISTS[which], None, 0, ctypes.byref(ln)))
        out = np.zeros(max(ln.value, 1), dtype=np.int32)
        self._check(lib().rs_node_list(self.h, i, LISTS[which], _i(out), ln.value, ctypes.byref(ln)))
        return out[:ln.value]

    def tree_bounds(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(lib().rs_tree_bounds(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def allskel(self):
        ln = ctypes.c_int(0)
        self._check(lib().rs_allskel(self.h, None, 0, ctypes.byref(ln)))
        out = np.zeros(max(ln.value, 1), dtype=np.int32)
        self._check(lib().rs_allskel(self.h, _i(out), ln.value, ctypes.byref(ln)))
        return out[:ln.value]

    def timer_start(self):
        self._check(lib().rs_timer_start(self.h))

    def timer_stop(self):
        ms = ctypes.c_float()
        self._check(lib().rs_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(lib().rs_synchronize(self.h))

    def tree_dump(self):
        """Tree fields named as in oracle/ref_dump.cpp's result file."""
        nn = self.num_nodes()
        out = {k: [] for k in ("node_level", "node_leaf", "node_parent", "node_children",
                               "node_compressed", "node_corners", "node_side")}
        lists = {"nbr": "neighbors", "orig": "original", "active": "active", "skel": "skel",
                 "red": "redundant", "near": "near"}
        csr = {k: ([0], []) for k in lists}
        nlev = self.stats()["num_levels"]
        level_sizes = np.zeros(nlev, dtype=np.int32)
        for i in range(nn):
            info, cor, side = self.node_info(i)
            level_sizes[info[0]] += 1
            out["node_level"].append(info[0])
            out["node_leaf"].append(info[1])
            out["node_parent"].append(info[2])
            out["node_children"].extend(info[3:7])
            out["node_compressed"].append(info[7])
            out["node_corners"].extend(cor)
            out["node_side"].append(side)
            for key, which in lists.items():
                v = self.node_list(i, which)
                csr[key][1].extend(v.tolist())
                csr[key][0].append(len(csr[key][1]))
        res = {k: np.array(v, dtype=np.float64 if k in ("node_corners", "node_side") else np.int32)
               for k, v in out.items()}
        for key, (off, val) in csr.items():
            res[key + "_off"] = np.array(off, dtype=np.int32)
            res[key] = np.array(val, dtype=np.int32)
        res["level_sizes"] = level_sizes
        return res


def id_batched(solver, mats, tol):
    """Runs the GPU ID on a list of dense matrices; returns [(k, perm, Z)]."""
    mats = [np.asfortranarray(a, dtype=np.float64) for a in mats]
    cnt = len(mats)
    m = np.array([a.shape[0] for a in mats], dtype=np.int32)
    n = np.array([a.shape[1] for a in mats], dtype=np.int32)
    a_off = np.zeros(cnt, dtype=np.int64)
    p_off = np.zeros(cnt, dtype=np.int64)
    z_off = np.zeros(cnt, dtype=np.int64)
    for i in range(1, cnt):
        a_off[i] = a_off[i - 1] + m[i - 1] * n[i - 1]
        p_off[i] = p_off[i - 1] + n[i - 1]
        z_off[i] = z_off[i - 1] + n[i - 1] * n[i - 1]
    A = np.concatenate([a.ravel(order="F") for a in mats])
    ranks = np.zeros(cnt, dtype=np.int32)
    perm = np.zeros(int(p_off[-1] + n[-1]), dtype=np.int32)
    Z = np.zeros(int(z_off[-1] + n[-1] * n[-1]))
    solver._check(lib().rs_id_batched(solver.h, cnt, _d(A), _l(a_off), _i(m), _i(n), tol,
                                      _i(ranks), _i(perm), _l(p_off), _d(Z), _l(z_off)))
    out = []
    for i in range(cnt):
        k = int(ranks[i])
        p = perm[p_off[i]:p_off[i] + n[i]].copy()
        z = Z[z_off[i]:z_off[i] + k * (n[i] - k)].reshape((k, n[i] - k), order="F") if k else None
        out.append((k, p, z))
    return out


def barrier_selftest(device=0, skip_block=-1, spins=1 << 16, rounds=8):
    """rs_barrier_selftest: returns (err, passed_min, passed_max, ms)."""
    err, pmin, pmax = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_int(-1)
    ms = ctypes.c_float(0)
    rc = lib().rs_barrier_selftest(device, skip_block, spins, rounds, ctypes.byref(err),
                                   ctypes.byref(pmin), ctypes.byref(pmax), ctypes.byref(ms))
    if rc != 0:
        raise RsError(rc, "barrier self-test failed")
    return err.value, pmin.value, pmax.value, ms.value
