"""GPU: the fast multipole products used for the refinement residual
(Laplace double layer, Laplace-Neumann, Stokes double layer), against the
dense FP64 product of the same kernel entries (rs_matvec).

Tolerances: FP64 and float-float variants, max |y_fmm - y_dense| <= 1e-10
max |y_dense| per column at the default order (31; measured ~1e-13 on the
65536-point star); lower orders must be no more accurate than higher ones.
FP32 variant (used only for products with refinement corrections): <= 2e-6
of max |y_dense|.  Below order 16 (the refinement's later corrections) the
FP32 product must stay within the error bound the refinement assumes for
it: eps16 * 10^(0.36 (16 - p)), eps16 = 6e-8 (Laplace, Neumann) or 8e-7
(Stokes), on rough vectors such as refinement corrections.
"""
import numpy as np
import pytest

from conftest import golden_geometry, load_golden

pytestmark = pytest.mark.gpu


def _rel(y, z):
    return float((np.abs(y - z).max(axis=0) / np.abs(z).max(axis=0)).max())


@pytest.mark.parametrize("name", ["laplace_circle_512", "laplace_annulus_512",
                                  "laplace_star_8192_2rhs", "laplace_unit_circle_4096"])
def test_fmm_matches_dense_golden(name, solver_lib):
    d = load_golden(name)
    geo = golden_geometry(d)
    pde, sd, leaf, npp = (int(x) for x in d["meta"][:4])
    s = solver_lib.Solver(geo, pde, float(d["tol"][0]), leaf=leaf, npp=npp)
    x = np.random.default_rng(3).standard_normal((s.D, 3))
    z = s.matvec(x)
    assert _rel(s.matvec(x, fast=True), z) <= 1e-10
    assert _rel(s.matvec(x, fast=True, arith=2), z) <= 1e-10


def test_fmm_large_star_many_rhs(solver_lib):
    from rskel import geometry as G
    geo = G.star(65536)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-8)
    x = np.random.default_rng(4).standard_normal((s.D, 10))  # two passes of at most 8
    y = s.matvec(x, fast=True)
    z = s.matvec(x)
    assert _rel(y, z) <= 1e-10
    assert _rel(s.matvec(x, fast=True, arith=2), z) <= 1e-10
    # column independence: the second pass equals a one-column product
    y9 = s.matvec(x[:, 9], fast=True)
    assert np.abs(y9 - y[:, 9]).max() <= 1e-13 * np.abs(y[:, 9]).max()


def test_fmm_order_monotone(solver_lib):
    d = load_golden("laplace_star_8192_2rhs")
    geo = golden_geometry(d)
    x = np.random.default_rng(5).standard_normal((geo.n, 2))
    errs = []
    for p in (10, 20, 40):
        s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-8, fmm_order=p)
        errs.append(_rel(s.matvec(x, fast=True), s.matvec(x)))
    assert errs[0] >= errs[1] >= errs[2] and errs[0] <= 1e-2, errs


@pytest.mark.parametrize("name", ["laplace_star_8192_2rhs", "laplace_annulus_512"])
def test_fmm_fp32_variant(name, solver_lib):
    d = load_golden(name)
    geo = golden_geometry(d)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-8)
    x = np.random.default_rng(7).standard_normal((s.D, 3))
    z = s.matvec(x)
    assert _rel(s.matvec(x, fast=True, fp32=True), z) <= 2e-6


@pytest.mark.parametrize("name", ["stokes_circle_512", "stokes_annulus_512",
                                  "stokes_ellipses_4096"])
def test_stokes_fmm_matches_dense(name, solver_lib):
    """The Stokes double layer as three Cauchy sums per density (A, B and the
    re-centred E/G channels) plus the rank-one term, against the dense
    product of the same kernel entries."""
    d = load_golden(name)
    geo = golden_geometry(d)
    s = solver_lib.Solver(geo, solver_lib.RS_STOKES, 1e-8, leaf=int(d["meta"][2]),
                          npp=int(d["meta"][3]))
    x = np.random.default_rng(6).standard_normal((s.D, 5))  # passes of 2, 2 and 1 densities
    z = s.matvec(x)
    assert _rel(s.matvec(x, fast=True), z) <= 1e-10
    assert _rel(s.matvec(x, fast=True, arith=2), z) <= 1e-10
    assert _rel(s.matvec(x, fast=True, fp32=True), z) <= 2e-6


def test_stokes_fmm_large_ellipses(solver_lib):
    from rskel import geometry as G
    geo = G.circle_with_ellipses(65536, 16, np.random.default_rng(3))
    s = solver_lib.Solver(geo, solver_lib.RS_STOKES, 1e-8)
    x = np.random.default_rng(8).standard_normal((s.D, 2))
    z = s.matvec(x)
    assert _rel(s.matvec(x, fast=True), z) <= 1e-10
    assert _rel(s.matvec(x, fast=True, arith=2), z) <= 1e-10
    assert _rel(s.matvec(x, fast=True, fp32=True), z) <= 2e-6


def test_neumann_fmm_matches_dense(solver_lib):
    from rskel import geometry as G
    for geo in (G.reference_donut(2048), G.star(16384)):
        s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE_NEUMANN, 1e-8)
        x = np.random.default_rng(9).standard_normal((s.D, 3))
        z = s.matvec(x)
        assert _rel(s.matvec(x, fast=True), z) <= 1e-10
        assert _rel(s.matvec(x, fast=True, arith=2), z) <= 1e-10
        assert _rel(s.matvec(x, fast=True, fp32=True), z) <= 2e-6


@pytest.mark.parametrize("pde", [0, 1, 2])
def test_fmm_fp32_lower_orders_within_the_refinement_bound(pde, solver_lib):
    from rskel import geometry as G
    capi = solver_lib
    geo = (G.circle_with_ellipses(16384, 4, np.random.default_rng(2)) if pde == capi.RS_STOKES
           else G.star(16384))
    eps16 = 8e-7 if pde == capi.RS_STOKES else 6e-8
    errs = []
    z = None
    for p in (4, 6, 8, 10, 12, 14, 16):
        s = capi.Solver(geo, pde, 1e-8, fmm_order32=p)
        x = np.random.default_rng(11).standard_normal((s.D, 3))
        if z is None:
            z = s.matvec(x)
        e = _rel(s.matvec(x, fast=True, fp32=True), z)
        assert e <= eps16 * 10.0 ** (0.36 * (16 - p)), (p, e)
        errs.append(e)
        s.close()
    assert errs[0] > errs[3] > errs[6], errs
