"""GPU: a batch of independent boundaries in one handle (a forest of
quadtrees, every level of every boundary factored in the same launches).

* FP64: each boundary's solution equals the one its own handle computes
  (same boxes, same kernels, same operation order): |diff| <= 1e-13 |mu|.
* FP32 + refinement: every boundary's residual, recomputed by an FP64
  multipole product on an evaluator handle of the same batch (its lists
  never cross boundaries), is <= 2e-10 of that boundary's data.
* The full batch configuration: 512 seeded random stars
  r(t) = 1 + sum_{k=2..8} a_k cos(k t + phi_k), a_k ~ U[0, 0.04],
  N ~ U[1024, 16384], ID tolerance 1e-8, one point-source right-hand side
  each.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stars(g, count, seed, lo=1024, hi=16384):
    rng = np.random.default_rng(seed)
    geos = [g.random_star(int(rng.integers(lo, hi + 1)), rng) for _ in range(count)]
    F = [g.laplace_point_source(geo, (2.0 * np.cos(t), 2.0 * np.sin(t)))
         for geo, t in zip(geos, rng.uniform(0, 2 * np.pi, count))]
    return geos, F


def _per_boundary_residual(capi, geos, F, mu):
    ev = capi.Solver(geos[0], capi.RS_LAPLACE, 1e-8, leaf=64, npp=64, fmm_order=36)
    ev.set_geometry_batch(geos)
    Ff = np.concatenate(F)
    r = ev.matvec(mu[:, None], fast=True)[:, 0] - Ff
    out, o = [], 0
    for f in F:
        out.append(np.linalg.norm(r[o:o + len(f)]) / np.linalg.norm(f))
        o += len(f)
    ev.close()
    return np.array(out)


def test_batch_fp64_equals_separate_handles(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    geos, F = _stars(g, 12, 7, 1024, 6000)
    b = capi.Solver(geos[0], capi.RS_LAPLACE, 1e-8, leaf=64, npp=64)
    b.set_geometry_batch(geos)
    b.factor()
    mu, _ = b.solve(np.concatenate(F))
    launches_batch = b.stats()["kernel_launches"]
    o, launches = 0, 0
    for geo, f in zip(geos, F):
        s = capi.Solver(geo, capi.RS_LAPLACE, 1e-8, leaf=64, npp=64)
        s.factor()
        m1, _ = s.solve(f)
        launches += s.stats()["kernel_launches"]
        assert np.abs(mu[o:o + geo.n] - m1).max() <= 1e-13 * np.abs(m1).max()
        o += geo.n
        s.close()
    assert launches_batch < launches / 4


def test_batch_fp32_refined_per_boundary(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    geos, F = _stars(g, 24, 8)
    b = capi.Solver(geos[0], capi.RS_LAPLACE, 1e-8, leaf=64, npp=64,
                    precision=capi.RS_FP32_REFINE, refine_tol=1e-10)
    b.set_geometry_batch(geos)
    b.factor()
    mu, _ = b.solve(np.concatenate(F))
    assert b.stats()["refine_residual"] <= 1e-10
    assert _per_boundary_residual(capi, geos, F, mu).max() <= 2e-10


def test_batch_512_random_stars(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    geos, F = _stars(g, 512, 4)
    b = capi.Solver(geos[0], capi.RS_LAPLACE, 1e-8, leaf=64, npp=64,
                    precision=capi.RS_FP32_REFINE, refine_tol=1e-10)
    b.set_geometry_batch(geos)
    b.factor()
    mu, _ = b.solve(np.concatenate(F))
    st = b.stats()
    assert st["refine_residual"] <= 1e-10
    res = _per_boundary_residual(capi, geos, F, mu)
    assert res.max() <= 2e-10, res.max()


def test_batch_rejects_what_it_does_not_support(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    geos, F = _stars(g, 3, 9, 1024, 2048)
    b = capi.Solver(geos[0], capi.RS_LAPLACE, 1e-8)
    b.set_geometry_batch(geos)
    with pytest.raises(capi.RsError):
        b.matvec(np.ones((b.D, 1)))
    s = capi.Solver(geos[0], capi.RS_STOKES, 1e-8, precision=capi.RS_FP32_REFINE)
    s.set_geometry_batch(geos)
    with pytest.raises(capi.RsError):
        s.factor()
