"""GPU: the autotuner (rs_autotune) and the CUDA-graph inverse.

* rs_autotune picks its launch shapes from the candidate sets, and the
  handle then factors and solves to the refinement tolerance.
* With and without the CUDA graph of the factorization's inverse, the
  refined solutions are bit-identical (the graph replays the same
  launches).
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
    split, wide = s.autotune(reps=2)
    assert split in (1, 32, 128, 256, 512, 1024, 1 << 30) and wide in (1, 2, 4)
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
