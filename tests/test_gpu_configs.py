"""GPU: the multiply connected Stokes configurations at full size.

* 16 holes: outer unit circle plus 16 seeded ellipses (semi-axes in
  [0.05, 0.15]), 131072 points (262144 DOFs), ID tolerance 1e-8, FP32
  factorization + FP64 refinement;
* 64 holes: 64 seeded ellipses (semi-axes in [0.03, 0.06]), 524288 points
  (1048576 DOFs), FP32 factorization with learned sketch sizes (the rank
  model trained on smaller seeded Stokes geometries), refinement that
  switches to GMRES-IR (flexible GMRES preconditioned by the FP32
  factorization) when the stationary iteration stalls.

Data: velocities of Stokeslets inside four holes plus one outside.  Checks:
the reported refinement residual, the same residual recomputed
independently (FP64 multipole product at order 40, plus U alpha from the
oracle's restatement of initialize_U_mat / initialize_Psi_mat), and the
second block Psi mu = alpha.  Tolerances: refine_tol 1e-10; independent
residual <= 2e-10 (the two products differ by their multipole errors);
|Psi mu - alpha| <= 1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(g, geo, rng):
    F = np.zeros(2 * geo.n)
    for c in np.asarray(geo.hole_centers).reshape(-1, 2)[:4]:
        F += g.stokeslet_velocity(geo, c, rng.standard_normal(2))
    return F + g.stokeslet_velocity(geo, (1.7, 0.4), rng.standard_normal(2))


def _check(capi, O, geo, F, s, mu, al):
    st = s.stats()
    assert st["refine_residual"] <= 1e-10, st["refine_residual"]
    U, P = O.border_matrices(geo, 2)
    ev = capi.Solver(geo, capi.RS_STOKES, 1e-8, leaf=64, npp=64, fmm_order=40)
    r = ev.matvec(mu[:, None], fast=True)[:, 0] + U @ al - F
    true = np.linalg.norm(r) / np.linalg.norm(F)
    assert true <= 2e-10, true
    assert np.abs(P @ mu - al).max() <= 1e-12
    ev.close()
    return st, true


def test_stokes_16_ellipses_262144_dofs(solver_lib, oracle_lib):
    from rskel import geometry as g

    capi = solver_lib
    geo = g.circle_with_ellipses(131072, 16, np.random.default_rng(3))
    F = _data(g, geo, np.random.default_rng(4))
    s = capi.Solver(geo, capi.RS_STOKES, 1e-8, leaf=64, npp=64, precision=capi.RS_FP32_REFINE,
                    refine_tol=1e-10, refine_max_iters=10)
    s.factor()
    mu, al = s.solve(F)
    st, true = _check(capi, oracle_lib, geo, F, s, mu, al)
    assert st["refine_iters"] <= 6
    # against the FP64 factorization at ID tolerance 1e-8: that solution
    # carries the ID error amplified by the system (~1e-6 here)
    s64 = capi.Solver(geo, capi.RS_STOKES, 1e-8, leaf=64, npp=64)
    s64.factor()
    mu64, al64 = s64.solve(F)
    assert np.linalg.norm(mu - mu64) / np.linalg.norm(mu64) <= 1e-4


def test_stokes_64_ellipses_1m_dofs_learned_gmres(solver_lib, oracle_lib):
    from rskel import geometry as g

    capi = solver_lib
    # rank model trained on ranks of plain FP32 factorizations of smaller
    # seeded geometries of the same family
    Xs, ys = [], []
    for seed in (10, 11, 12):
        tg = g.circle_with_ellipses(32768, 16, np.random.default_rng(seed), semi=(0.03, 0.08))
        t = capi.Solver(tg, capi.RS_STOKES, 1e-8, leaf=64, npp=64, precision=capi.RS_FP32_REFINE)
        t.factor()
        X, y = t.rank_samples()
        Xs.append(X)
        ys.append(y)
    w, loss = t.rank_train(np.concatenate(Xs), np.concatenate(ys), capi.rank_model_init(0),
                           epochs=1500, lr=3e-3)
    t.close()
    assert loss < 0.01
    geo = g.circle_with_ellipses(524288, 64, np.random.default_rng(3), semi=(0.03, 0.06))
    F = _data(g, geo, np.random.default_rng(4))
    s = capi.Solver(geo, capi.RS_STOKES, 1e-8, leaf=64, npp=64, precision=capi.RS_FP32_REFINE,
                    refine_tol=1e-10, refine_max_iters=10)
    s.set_rank_model(w)
    s.factor()
    mu, al = s.solve(F)
    st, true = _check(capi, oracle_lib, geo, F, s, mu, al)
    assert st["krylov_steps"] > 0
    assert st["rank_predicted"] > 1000 and st["rank_redo"] <= 0.25 * st["rank_predicted"]


def test_gmres_ir_matches_stationary_refinement(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    geo = g.star(65536)
    F = np.stack([g.laplace_point_source(geo, (2.0 * np.cos(a), 2.0 * np.sin(a)))
                  for a in (0.4, 2.5, 4.0)], 1)
    out = []
    for solver in (1, 2):
        s = capi.Solver(geo, capi.RS_LAPLACE, 1e-8, leaf=64, npp=64,
                        precision=capi.RS_FP32_REFINE, refine_tol=1e-10, refine_solver=solver)
        s.factor()
        mu, _ = s.solve(F)
        st = s.stats()
        assert st["refine_residual"] <= 1e-10
        assert (st["krylov_steps"] > 0) == (solver == 2)
        out.append(mu)
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1]) <= 1e-9
