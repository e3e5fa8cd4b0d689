"""GPU: the autotuner (rs_autotune) and the CUDA-graph inverse.

* rs_autotune picks its launch shapes from the candidate sets, and the
  handle then factors and solves to the refinement tolerance.
* With and without the CUDA graph of the factorization's inverse, the
  refined solutions are bit-identical (the graph replays the same
  launches).
* The small levels' ID sketch split over several CTAs per box gives the
  ranks of one CTA per box and the same refined solution.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _star(capi, g, **kw):
    geo = g.star(32768)
    F = np.stack([g.laplace_point_source(geo, (2.0 * np.cos(a), 2.0 * np.sin(a)))
                  for a in (0.3, 1.9)], 1)
    s = capi.Solver(geo, capi.RS_LAPLACE, 1e-8, leaf=64, npp=64, precision=capi.RS_FP32_REFINE,
                    refine_tol=1e-10, **kw)
    return s, F


def test_autotune_picks_candidates_and_solves(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    s, F = _star(capi, g)
    split, wide, elim = s.autotune(reps=2)
    assert split in (1, 32, 128, 256, 512, 1024, 1 << 30) and wide in (1, 2, 4)
    assert elim in (0, 128, 256)
    s.factor()
    mu, _ = s.solve(F)
    assert s.stats()["refine_residual"] <= 1e-10


def test_graph_inverse_is_bit_identical(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    out = []
    for ug in (0, 1):
        s, F = _star(capi, g, use_graphs=ug)
        s.factor()
        mu, _ = s.solve(F)
        mu2, _ = s.solve(F)  # the second solve replays the captured graph
        assert np.array_equal(mu, mu2)
        out.append(mu)
    assert np.array_equal(out[0], out[1])


def test_root_inverse_and_root_lu_agree(solver_lib):
    """FP32 roots of at most 128 DOFs: the explicit inverse (Gauss-Jordan,
    default) and LU with triangular solves give the same refined solution,
    and the same FP32 preconditioner up to FP32 rounding (one refinement
    step at most apart).  Also on a batch, where every tree has its own
    root block."""
    from rskel import geometry as g

    capi = solver_lib
    res = []
    for ri in (1, 0):
        s, F = _star(capi, g, root_inverse=ri, refine_max_iters=12)
        s.factor()
        mu, _ = s.solve(F)
        st = s.stats()
        assert st["num_skel_root"] <= 128
        assert st["refine_residual"] <= 1e-10
        res.append((mu, st["refine_iters"]))
    (m1, i1), (m0, i0) = res
    assert abs(i1 - i0) <= 1
    assert np.linalg.norm(m1 - m0) / np.linalg.norm(m0) <= 1e-9
    rng = np.random.default_rng(12)
    geos = [g.random_star(int(rng.integers(1024, 4096)), rng) for _ in range(6)]
    out = []
    for ri in (1, 0):
        s = capi.Solver(geos[0], capi.RS_LAPLACE, 1e-8, leaf=64, npp=64,
                        precision=capi.RS_FP32_REFINE, refine_tol=1e-10, root_inverse=ri)
        s.set_geometry_batch(geos)
        F = np.concatenate([g.laplace_point_source(q, (2.0, 0.5)) for q in geos])
        s.factor()
        mu, _ = s.solve(F)
        assert s.stats()["refine_residual"] <= 1e-10
        out.append(mu)
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1]) <= 1e-9


def _levels_ranks(s):
    """(level, num_skel) of every compressed box, in node order."""
    out = []
    for i in range(s.num_nodes()):
        info, _, _ = s.node_info(i)
        if info[7]:
            out.append((int(info[0]), int(info[8])))
    return out


def test_row_groups_sketch_matches_one_cta_per_box(solver_lib):
    """The small levels' sketch split over several CTAs per box (id_row_groups)
    sums the same rows of the same signs in another order.  At FP32 ID
    tolerance 1e-4 (far above the sketch's rounding) the ranks of nearly every
    box agree with one CTA per box; at the default 1e-6 (where rounding of
    order 1e-7 |R_00| moves ranks near the threshold) the rank totals agree
    within 1 % and both refined solutions match to 1e-9."""
    from rskel import geometry as g

    capi = solver_lib
    for id_tol in (1e-4, 1e-6):
        sols, ranks = {}, {}
        for rg in (0, -1, 5):
            s, F = _star(capi, g, id_row_groups=rg, fp32_id_tol=id_tol)
            s.factor()
            sols[rg], _ = s.solve(F)
            assert s.stats()["refine_residual"] <= 1e-10
            ranks[rg] = _levels_ranks(s)
            s.close()
        for rg in (-1, 5):
            a, b = ranks[0], ranks[rg]
            assert len(a) == len(b) and [x[0] for x in a] == [x[0] for x in b]
            diff = [abs(x[1] - y[1]) for x, y in zip(a, b)]
            if id_tol == 1e-4:
                assert max(diff) <= 1 and sum(d > 0 for d in diff) <= max(2, len(diff) // 50), rg
            else:
                ka, kb = sum(x[1] for x in a), sum(x[1] for x in b)
                assert abs(ka - kb) <= 0.01 * ka, (rg, ka, kb)
                err = np.linalg.norm(sols[rg] - sols[0]) / np.linalg.norm(sols[0])
                assert err <= 1e-9, (rg, err)
