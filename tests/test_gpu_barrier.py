"""The bounded grid barrier of the cooperative kernels (the bordered system's
S inverse) gives up and reports instead of waiting forever.

rs_barrier_selftest runs grid barriers over one CTA per SM.  With one CTA
leaving before its first arrival, the other CTAs' waits run out after a
short poll limit (2^14 polls, milliseconds); they raise the error flag and
return, which rs_factor reports as RS_ERR_CUDA "grid barrier timed out".  No
fault or hang is involved: the context stays usable, as the runs after the
timeout show.  The argument checks run without a GPU.
"""
import numpy as np
import pytest

RS_ERR_ARG, RS_ERR_NO_DEVICE = 1, 4


def test_barrier_selftest_checks_arguments(solver_lib):
    import ctypes

    L = solver_lib.lib()
    i, f = ctypes.c_int(0), ctypes.c_float(0)
    r = ctypes.byref
    assert L.rs_barrier_selftest(0, -1, 1 << 16, 0, r(i), r(i), r(i), r(f)) == RS_ERR_ARG
    assert L.rs_barrier_selftest(0, -1, 1 << 16, 65, r(i), r(i), r(i), r(f)) == RS_ERR_ARG
    assert L.rs_barrier_selftest(0, -1, 0, 4, r(i), r(i), r(i), r(f)) == RS_ERR_ARG
    assert L.rs_barrier_selftest(0, -1, (1 << 22) + 1, 4, r(i), r(i), r(i), r(f)) == RS_ERR_ARG
    assert L.rs_barrier_selftest(0, -1, 1 << 16, 4, None, r(i), r(i), r(f)) == RS_ERR_ARG


@pytest.mark.gpu
def test_grid_barrier_timeout_is_reported_and_the_context_survives(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    err, pmin, pmax, _ = capi.barrier_selftest(skip_block=-1, rounds=8)
    assert (err, pmin, pmax) == (0, 8, 8)
    # one CTA never arrives: every wait runs out, none passes a barrier
    err, pmin, pmax, ms = capi.barrier_selftest(skip_block=5, spins=1 << 14, rounds=8)
    assert err == 1 and pmax == 0
    assert ms < 2000.0
    # the context is still usable: barriers and a factor + solve after it
    err, pmin, pmax, _ = capi.barrier_selftest(skip_block=-1, rounds=8)
    assert (err, pmin, pmax) == (0, 8, 8)
    geo = g.unit_circle(1024)
    s = capi.Solver(geo, capi.RS_LAPLACE, 1e-10, leaf=64, npp=64)
    s.factor()
    mu, _ = s.solve(g.laplace_cauchy(geo))
    assert np.all(np.isfinite(mu))
    s.close()
