"""ctypes binding of the oracle restatement (oracle/rs_oracle.c).

Test infrastructure only: the checker used by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg.  It is built by
``make -C oracle oracle`` into oracle/_build/liboracle.so.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp,
                                 ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        for fn in ("orc_build_tree", "orc_factor", "orc_num_levels", "orc_num_nodes",
                   "orc_border_dims"):
            getattr(L, fn).argtypes = [ctypes.c_void_p]
            getattr(L, fn).restype = ctypes.c_int
        L.orc_solve.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp, _dp]
        L.orc_solve.restype = ctypes.c_int
        L.orc_node_info.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip, _dp, _dp]
        L.orc_node_list.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int]
        L.orc_node_list.restype = ctypes.c_int
        L.orc_allskel.argtypes = [ctypes.c_void_p, _ip, ctypes.c_int]
        L.orc_allskel.restype = ctypes.c_int
        L.orc_tree_min.argtypes = [ctypes.c_void_p]
        L.orc_tree_min.restype = ctypes.c_double
        L.orc_tree_max.argtypes = [ctypes.c_void_p]
        L.orc_tree_max.restype = ctypes.c_double
        L.orc_node_factors.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_node_factors.restype = ctypes.c_int
        L.orc_kernel_block.argtypes = [ctypes.c_void_p, _ip, ctypes.c_int, _ip, ctypes.c_int, _dp]
        L.orc_id_matrix.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_long, _ip]
        L.orc_id_matrix.restype = ctypes.c_int
        L.orc_id.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _ip, _dp, _dp]
        L.orc_id.restype = ctypes.c_int
        L.orc_matvec.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp]
        L.orc_border_mats.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_last_factor_seconds.argtypes = [ctypes.c_void_p]
        L.orc_last_factor_seconds.restype = ctypes.c_double
        L.orc_last_solve_seconds.argtypes = [ctypes.c_void_p]
        L.orc_last_solve_seconds.restype = ctypes.c_double
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def orc_id(A, tol):
    """Restated ie_Mat::id: returns (k, perm, Z, rdiag)."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    perm = np.zeros(n, dtype=np.int32)
    Z = np.zeros(n * n)
    rd = np.zeros(n)
    k = lib().orc_id(_d(A), m, n, tol, _i(perm), _d(Z), _d(rd))
    Zm = Z[:k * (n - k)].reshape((k, n - k), order="F") if k else np.zeros((0, 0))
    return k, perm, Zm, rd


class OracleSolver:
    """One boundary problem on the oracle restatement."""

    LISTS = {"original": 0, "active": 1, "skel": 2, "redundant": 3, "near": 4,
             "neighbors": 5, "permutation": 6}

    def __init__(self, geo, pde, sd, tol, leaf=64, npp=64, threads=1):
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in
                      (geo.points, geo.normals, geo.weights, geo.curvatures,
                       geo.hole_centers if geo.num_holes else np.zeros(1),
                       geo.hole_radii if geo.num_holes else np.zeros(1))]
        p, q, w, c, hc, hr = self._keep
        self.n, self.sd, self.pde = geo.n, sd, pde
        self.h = lib().orc_create(pde, sd, geo.n, _d(p), _d(q), _d(w), _d(c), geo.num_holes,
                                  _d(hc), _d(hr), tol, leaf, npp, threads)
        self.nb = 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def build_tree(self):
        rc = lib().orc_build_tree(self.h)
        assert rc == 0, rc

    def factor(self):
        rc = lib().orc_factor(self.h)
        if rc:
            raise RuntimeError(f"oracle factor failed ({rc})")
        self.nb = lib().orc_border_dims(self.h)
        return lib().orc_last_factor_seconds(self.h)

    def solve(self, f):
        f = np.asfortranarray(f, dtype=np.float64)
        if f.ndim == 1:
            f = f[:, None]
        mu = np.zeros_like(f, order="F")
        alpha = np.zeros(max(self.nb, 1))
        rc = lib().orc_solve(self.h, _d(f), f.shape[1], _d(mu), _d(alpha))
        if rc:
            raise RuntimeError(f"oracle solve failed ({rc})")
        return mu, (alpha[:self.nb] if self.nb else None)

    @property
    def solve_seconds(self):
        return lib().orc_last_solve_seconds(self.h)

    def num_nodes(self):
        return lib().orc_num_nodes(self.h)

    def num_levels(self):
        return lib().orc_num_levels(self.h)

    def node_info(self, i):
        info = np.zeros(10, dtype=np.int32)
        cor = np.zeros(8)
        side = np.zeros(1)
        lib().orc_node_info(self.h, i, _i(info), _d(cor), _d(side))
        return info, cor, side[0]

    def node_list(self, i, which):
        w = self.LISTS[which]
        cnt = lib().orc_node_list(self.h, i, w, None, 0)
        out = np.zeros(max(cnt, 1), dtype=np.int32)
        lib().orc_node_list(self.h, i, w, _i(out), cnt)
        return out[:cnt]

    def allskel(self):
        cnt = lib().orc_allskel(self.h, None, 0)
        out = np.zeros(max(cnt, 1), dtype=np.int32)
        lib().orc_allskel(self.h, _i(out), cnt)
        return out[:cnt]

    def tree_minmax(self):
        return lib().orc_tree_min(self.h), lib().orc_tree_max(self.h)

    def id_matrix(self, i):
        n = np.zeros(1, dtype=np.int32)
        m = lib().orc_id_matrix(self.h, i, None, 0, _i(n))
        out = np.zeros(max(m * n[0], 1))
        lib().orc_id_matrix(self.h, i, _d(out), m * n[0], _i(n))
        return out[:m * n[0]].reshape((m, n[0]), order="F")

    def kernel_block(self, I, J):
        I = np.ascontiguousarray(I, dtype=np.int32)
        J = np.ascontiguousarray(J, dtype=np.int32)
        out = np.zeros((I.size, J.size), order="F")
        lib().orc_kernel_block(self.h, _i(I), I.size, _i(J), J.size, _d(out))
        return out

    def matvec(self, x):
        x = np.asfortranarray(x, dtype=np.float64)
        if x.ndim == 1:
            x = x[:, None]
        y = np.zeros_like(x, order="F")
        lib().orc_matvec(self.h, _d(x), x.shape[1], _d(y))
        return y

    def border_mats(self):
        D = self.n * self.sd
        U = np.zeros((D, self.nb), order="F")
        P = np.zeros((self.nb, D), order="F")
        lib().orc_border_mats(self.h, _d(U), _d(P))
        return U, P

    def tree_dump(self):
        """Same field names as oracle/ref_dump.cpp's result file."""
        nn = self.num_nodes()
        out = {k: [] for k in ("node_level", "node_leaf", "node_parent", "node_children",
                               "node_compressed", "node_corners", "node_side")}
        lists = {"nbr": "neighbors", "orig": "original", "active": "active", "skel": "skel",
                 "red": "redundant", "near": "near"}
        csr = {k: ([0], []) for k in lists}
        level_sizes = np.zeros(self.num_levels(), dtype=np.int32)
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


def domain_eval(geo, pde, targets, mu, alpha=None, in_domain=None):
    """Restatement of the domain solution of boundary_integral_solve
    (ie_solver/linear_solve.cpp:140-154, 188-266): K_domain mu + U_forward
    alpha, K_domain per Initialization::InitializeDomainKernel
    (ie_solver/initialization.cpp:11-135) with the off-boundary kernels of
    ie_solver/kernel/kernel.cpp:29-104, U_forward per initialize_U_mat
    (ie_solver/linear_solve.cpp:20-64); targets outside the domain give 0.
    Dense numpy, FP64."""
    pts = geo.points.reshape(-1, 2)
    nrm = geo.normals.reshape(-1, 2)
    w = geo.weights
    t = np.asarray(targets, dtype=np.float64).reshape(-1, 2)
    nt, n = t.shape[0], pts.shape[0]
    mu = np.asarray(mu, dtype=np.float64)
    if mu.ndim == 1:
        mu = mu[:, None]
    rx = t[:, 0:1] - pts[None, :, 0]
    ry = t[:, 1:2] - pts[None, :, 1]
    r2 = rx * rx + ry * ry
    dot = rx * nrm[None, :, 0] + ry * nrm[None, :, 1]
    if pde == 2:
        c = w[None, :] / np.pi * dot / (r2 * r2)
        out = np.zeros((2 * nt, mu.shape[1]))
        m0, m1 = mu[0::2], mu[1::2]
        for q in range(mu.shape[1]):
            d = c * (rx * m0[None, :, q] + ry * m1[None, :, q])
            out[0::2, q] = (rx * d).sum(1)
            out[1::2, q] = (ry * d).sum(1)
    elif pde == 1:
        out = (w[None, :] / (2 * np.pi) * 0.5 * np.log(r2)) @ mu
    else:
        out = (-w[None, :] / (2 * np.pi) * dot / r2) @ mu
    if alpha is not None and geo.num_holes > 0 and pde != 1:
        alpha = np.asarray(alpha, dtype=np.float64)
        if alpha.ndim == 1:
            alpha = alpha[:, None]
        hc = geo.hole_centers.reshape(-1, 2)
        for h in range(hc.shape[0]):
            hx = t[:, 0] - hc[h, 0]
            hy = t[:, 1] - hc[h, 1]
            h2 = hx * hx + hy * hy
            if pde == 0:
                out += np.outer(0.5 * np.log(h2), alpha[h])
            else:
                s = 1.0 / (4 * np.pi)
                lg = -0.5 * np.log(h2)
                a0, a1, a2 = alpha[3 * h], alpha[3 * h + 1], alpha[3 * h + 2]
                out[0::2] += s * (np.outer(lg + hx * hx / h2, a0) + np.outer(hx * hy / h2, a1)
                                  + np.outer(hy / h2, a2))
                out[1::2] += s * (np.outer(hx * hy / h2, a0) + np.outer(lg + hy * hy / h2, a1)
                                  - np.outer(hx / h2, a2))
    if in_domain is not None:
        keep = np.asarray(in_domain, dtype=bool)
        sd = 2 if pde == 2 else 1
        out[np.repeat(~keep, sd)] = 0.0
    return out


def border_matrices(geo, pde):
    """U (D x nb) and Psi (nb x D) of the bordered system for a geometry with
    holes, as initialize_U_mat and initialize_Psi_mat build them
    (ie_solver/linear_solve.cpp:20-112): Laplace log|x - c_h| per hole;
    Stokes a Stokeslet pair and a rotlet per hole; Psi the quadrature
    weights of the hole's own points (first hole whose circle, radius
    + 1e-8, holds the point), plus the moment row for Stokes.  pde: 0
    Laplace, 2 Stokes."""
    xy = np.asarray(geo.points, dtype=np.float64).reshape(-1, 2)
    n = xy.shape[0]
    hc = np.asarray(geo.hole_centers, dtype=np.float64).reshape(-1, 2)
    hr = np.asarray(geo.hole_radii, dtype=np.float64).reshape(-1)
    h = len(hr)
    w = np.asarray(geo.weights, dtype=np.float64)
    stokes = pde == 2
    D = 2 * n if stokes else n
    nb = 3 * h if stokes else h
    U = np.zeros((D, nb))
    P = np.zeros((nb, D))
    member = -np.ones(n, dtype=int)
    sc = 1.0 / (4.0 * np.pi)
    for k in range(h):
        r0 = xy[:, 0] - hc[k, 0]
        r1 = xy[:, 1] - hc[k, 1]
        r2 = r0 * r0 + r1 * r1
        rn = np.sqrt(r2)
        if stokes:
            lg = np.log(1.0 / rn)
            U[0::2, 3 * k] = sc * (lg + r0 * r0 / r2)
            U[1::2, 3 * k] = sc * (r1 * r0 / r2)
            U[0::2, 3 * k + 1] = sc * (r0 * r1 / r2)
            U[1::2, 3 * k + 1] = sc * (lg + r1 * r1 / r2)
            U[0::2, 3 * k + 2] = r1 * (sc / r2)
            U[1::2, 3 * k + 2] = -r0 * (sc / r2)
        else:
            U[:, k] = np.log(rn)
        sel = (member < 0) & (rn < hr[k] + 1e-8)
        member[sel] = k
    for i in np.nonzero(member >= 0)[0]:
        k = member[i]
        if stokes:
            P[3 * k, 2 * i] = w[i]
            P[3 * k + 1, 2 * i + 1] = w[i]
            P[3 * k + 2, 2 * i] = w[i] * xy[i, 1]
            P[3 * k + 2, 2 * i + 1] = -w[i] * xy[i, 0]
        else:
            P[k, i] = w[i]
    return U, P

