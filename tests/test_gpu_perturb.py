"""GPU: refactorization after a local boundary change (rs_perturb, the
reference's QuadTree::perturb + skeletonize keeping compressed boxes).

Mirrors the reference's update tests (ie_solver_test.cpp:577-612, 630-673,
690-730): after each change, the updated factorization's solution (and its
domain solution) agrees with a fresh factorization of the new boundary to
100 tol, the backward error against the dense operator stays <= 50 tol, and
only a fraction of the boxes is refactored (the boxes near the old and new
bump, their neighbours and ancestors).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# A smooth bump: sharper ones (width 0.1, height 0.05) put points of a larger,
# non-neighbouring leaf inside a box's proxy circle, where the reference's
# neighbour rule (quadtree.cpp:185-227) leaves them out of the ID rows and
# the fresh factorization itself loses accuracy.
BUMP = dict(width=0.2, height=0.02)


def _data(G, geo, stokes):
    if stokes:
        return G.stokeslet_velocity(geo, (2.2, 0.7), (1.0, -0.5))
    return G.laplace_point_source(geo, (2.2, 0.7))


@pytest.mark.parametrize("pde,prec,n", [(0, 0, 8192), (2, 0, 4096), (0, 1, 8192)])
def test_update_loses_no_accuracy(solver_lib, pde, prec, n):
    from rskel import geometry as G

    tol = 1e-8
    stokes = pde == solver_lib.RS_STOKES
    s = solver_lib.Solver(G.star_bump(n, center=0.0, **BUMP), pde, tol, leaf=64, npp=64,
                          precision=prec)
    s.factor()
    full = s.stats()["boxes_factored"]
    rng = np.random.default_rng(9)
    targets = np.empty(2 * 200)
    r = 0.5 * np.sqrt(rng.uniform(size=200))
    th = rng.uniform(0, 2 * np.pi, 200)
    targets[0::2], targets[1::2] = r * np.cos(th), r * np.sin(th)
    for c in (0.4, 1.3, 2.5, 4.0):
        geo = G.star_bump(n, center=c, **BUMP)
        f = _data(G, geo, stokes)
        s.set_geometry(geo, perturb=True)
        s.factor()
        part = s.stats()["boxes_factored"]
        mu, _ = s.solve(f)
        fresh = solver_lib.Solver(geo, pde, tol, leaf=64, npp=64, precision=prec)
        fresh.factor()
        mu2, _ = fresh.solve(f)
        assert np.abs(mu - mu2).max() <= 100 * tol * np.abs(mu2).max(), c
        u, u2 = s.domain_eval(targets, mu), fresh.domain_eval(targets, mu2)
        assert np.abs(u - u2).max() <= 100 * tol * max(1.0, np.abs(u2).max()), c
        assert np.abs(s.matvec(mu) - f).max() <= 50 * tol * max(1.0, np.abs(f).max()), c
        assert np.abs(fresh.matvec(mu2) - f).max() <= 50 * tol * max(1.0, np.abs(f).max()), c
        assert part < 0.7 * full, (part, full)


def test_unchanged_boundary_refactors_nothing_but_the_root(solver_lib):
    from rskel import geometry as G

    geo = G.star_bump(8192, center=1.0)
    f = G.laplace_point_source(geo, (2.2, 0.7))
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-8, leaf=64, npp=64)
    s.factor()
    mu, _ = s.solve(f)
    s.set_geometry(geo, perturb=True)
    s.factor()
    assert s.stats()["boxes_factored"] == 0
    mu2, _ = s.solve(f)
    assert np.array_equal(mu, mu2)
