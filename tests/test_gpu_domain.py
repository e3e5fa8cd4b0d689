"""GPU: solution evaluation at points off the boundary (rs_domain_eval).

* Parity with the oracle's dense restatement (initialization.cpp:11-135,
  linear_solve.cpp:20-64, 188-266) on random densities: 1e-12 relative.
* The reference's analytic-agreement tests (ie_solver_test.cpp:404-430,
  508-524): solve, evaluate on a 20 x 20 grid over the tree's box, compare
  with the exact interior solution on the points the reference's
  is_in_domain keeps (1e-2 away from the boundary), relative L2 (Laplace)
  or max-norm (Stokes) error <= 10 tol as the reference requires.
"""
import math

import numpy as np
import pytest

from conftest import golden_geometry, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["laplace_star_8192_2rhs", "laplace_annulus_512",
                                  "stokes_annulus_512", "stokes_ellipses_4096"])
def test_domain_eval_matches_oracle(name, solver_lib, oracle_lib):
    d = load_golden(name)
    geo = golden_geometry(d)
    pde, sd, leaf, npp = (int(x) for x in d["meta"][:4])
    s = solver_lib.Solver(geo, pde, float(d["tol"][0]), leaf=leaf, npp=npp)
    rng = np.random.default_rng(8)
    mu = rng.standard_normal((s.D, 3))
    alpha = rng.standard_normal((s.nb, 3)) if s.nb else None
    xy = geo.xy()
    lo, hi = xy.min(0), xy.max(0)
    t = np.empty(2 * 300)
    t[0::2] = rng.uniform(lo[0], hi[0], 300)
    t[1::2] = rng.uniform(lo[1], hi[1], 300)
    mask = rng.uniform(size=300) < 0.8
    got = s.domain_eval(t, mu, alpha, mask)
    ref = oracle_lib.domain_eval(geo, pde, t, mu, alpha, mask)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def _bounds(s):
    lo, hi = np.zeros(1), np.zeros(1)
    from rskel import capi
    capi.lib().rs_tree_bounds(s.h, capi._d(lo), capi._d(hi))
    return float(lo[0]), float(hi[0])


def _grid_points(lo, hi, size=20):
    xs = lo + (np.arange(size) / (size - 1)) * (hi - lo)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    t = np.empty(2 * size * size)
    t[0::2], t[1::2] = X.ravel(), Y.ravel()
    return t


def test_laplace_circle_analytic(solver_lib):
    from rskel import geometry as G

    tol = 1e-6  # the reference's default configuration
    geo = G.reference_circle(512)
    xy = geo.xy()
    f = np.log(np.hypot(xy[:, 0] + 3, xy[:, 1] + 2))  # SINGLE_ELECTRON (boundary.cpp:49-54)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, tol, leaf=32, npp=128)
    s.build_tree()
    s.factor()
    mu, _ = s.solve(f)
    t = _grid_points(*_bounds(s))
    T = t.reshape(-1, 2)
    inside = np.hypot(T[:, 0] - 0.5, T[:, 1] - 0.5) + 1e-2 <= 0.25  # circle.cpp:36-44
    u = s.domain_eval(t, mu, None, inside)
    truth = np.log(np.hypot(T[:, 0] + 3, T[:, 1] + 2))
    err = np.linalg.norm((u - truth)[inside]) / np.linalg.norm(truth[inside])
    assert inside.sum() > 20 and err <= 10 * tol, err


def test_laplace_annulus_analytic(solver_lib):
    from rskel import geometry as G

    tol = 1e-6
    geo = G.reference_annulus(512)
    xy = geo.xy()
    f = np.log(np.hypot(xy[:, 0] + 3, xy[:, 1] + 2))
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, tol, leaf=32, npp=128)
    s.build_tree()
    s.factor()
    mu, alpha = s.solve(f)
    t = _grid_points(*_bounds(s))
    T = t.reshape(-1, 2)
    inside = np.hypot(T[:, 0] - 0.5, T[:, 1] - 0.5) + 1e-2 <= 1.0  # annulus.cpp:69-81
    hc = geo.hole_centers.reshape(-1, 2)
    for (cx, cy), r in zip(hc, geo.hole_radii):
        inside &= np.hypot(T[:, 0] - cx, T[:, 1] - cy) - 1e-2 >= r
    u = s.domain_eval(t, mu, alpha, inside)
    truth = np.log(np.hypot(T[:, 0] + 3, T[:, 1] + 2))
    err = np.linalg.norm((u - truth)[inside]) / np.linalg.norm(truth[inside])
    assert inside.sum() > 20 and err <= 10 * tol, err


def test_stokes_circle_rotation_analytic(solver_lib):
    from rskel import geometry as G

    tol = 1e-6
    geo = G.reference_circle(512)
    f = G.tangent_data(geo)  # TANGENT_VEC: a rigid rotation of the disc
    s = solver_lib.Solver(geo, solver_lib.RS_STOKES, tol, leaf=32, npp=128)
    s.build_tree()
    s.factor()
    mu, _ = s.solve(f)
    t = _grid_points(*_bounds(s))
    T = t.reshape(-1, 2)
    inside = np.hypot(T[:, 0] - 0.5, T[:, 1] - 0.5) + 1e-2 <= 0.25
    u = s.domain_eval(t, mu, None, inside).reshape(-1, 2)
    rx, ry = T[:, 0] - 0.5, T[:, 1] - 0.5
    truth = 4.0 * np.stack([-ry, rx], 1)  # |u| = 4 r: unit speed at r = 0.25 (ie_solver_test.cpp:473-500)
    err = np.abs(u - truth)[inside].max()
    assert inside.sum() > 20 and err <= 10 * tol, err


def test_laplace_neumann_donut_analytic(solver_lib):
    """ie_solver_test.cpp:508-524 (LaplaceNeumannDonutAnalyticAgreement): the
    domain solution minus log r is constant to 10 tol."""
    from rskel import geometry as G

    tol = 1e-6
    geo = G.reference_donut(512)
    f = G.donut_neumann_data(geo)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE_NEUMANN, tol, leaf=32, npp=128)
    s.build_tree()
    s.factor()
    mu, _ = s.solve(f)
    t = _grid_points(*_bounds(s))
    T = t.reshape(-1, 2)
    r = np.hypot(T[:, 0] - 0.5, T[:, 1] - 0.5)
    inside = (r + 1e-2 <= 1.0) & (r - 1e-2 >= 0.5)  # donut.cpp:66-78
    u = s.domain_eval(t, mu, None, inside)
    dev = (u - np.log(np.where(inside, r, 1.0)))[inside]
    err = np.abs(dev - dev.mean()).max()
    assert inside.sum() > 20 and err <= 10 * tol, err


def test_laplace_neumann_solve_matches_oracle(solver_lib, oracle_lib):
    from rskel import geometry as G

    tol = 1e-8
    geo = G.reference_donut(1024)
    f = G.donut_neumann_data(geo)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE_NEUMANN, tol, leaf=64, npp=64)
    s.factor()
    mu, _ = s.solve(f)
    o = oracle_lib.OracleSolver(geo, 1, 1, tol, 64, 64, 4)
    o.build_tree()
    o.factor()
    mo, _ = o.solve(f)
    mo = np.asarray(mo).reshape(mu.shape)
    assert np.linalg.norm(mu - mo) <= 10 * tol * np.linalg.norm(mo)
    # backward error against the dense operator (ie_solver_test.cpp:82-95)
    assert np.abs(s.matvec(mu) - f).max() <= 50 * tol
