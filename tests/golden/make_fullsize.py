"""Generates tests/golden/stokes_64_ellipses_1m_oracle.npz: the oracle's
solution of the 64-hole Stokes configuration at ID tolerance 1e-12.

Configuration: Stokes double layer on the unit circle plus 64 seeded
ellipses (rskel.geometry.circle_with_ellipses(524288, 64, default_rng(3),
semi=(0.03, 0.06))), 524288 points, 1048576 DOFs, leaf 64 DOFs, 64 proxy
points.  Right-hand side: velocities of Stokeslets inside the first four
holes plus one at (1.7, 0.4), forces from default_rng(4), as in the GPU
tests.  The oracle (oracle/rs_oracle.c, the CPU restatement of the
reference's factor + multiply_connected_solve) takes about nine minutes on
eight cores, so the solution is cached instead of rerun by the tests.

Stored: mu (1048576) and alpha (192 hole coefficients) with their float64
mantissas rounded to 40 bits (relative rounding <= 2^-41, far below the
1e-8 comparison), which lets the file compress; plus the configuration.

    python tests/golden/make_fullsize.py [threads]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "ie-solver_gb300"), os.path.join(ROOT, "oracle")]

OUT = os.path.join(HERE, "stokes_64_ellipses_1m_oracle.npz")
N_POINTS, HOLES, SEMI, TOL = 524288, 64, (0.03, 0.06), 1e-12


def workload():
    from rskel import geometry as g

    geo = g.circle_with_ellipses(N_POINTS, HOLES, np.random.default_rng(3), semi=SEMI)
    rng = np.random.default_rng(4)
    F = np.zeros(2 * geo.n)
    for c in np.asarray(geo.hole_centers).reshape(-1, 2)[:4]:
        F += g.stokeslet_velocity(geo, c, rng.standard_normal(2))
    F += g.stokeslet_velocity(geo, (1.7, 0.4), rng.standard_normal(2))
    return geo, F


def round40(x):
    """float64 values with the mantissa rounded to nearest at 40 bits."""
    b = np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)
    b = (b + np.uint64(1 << 11)) & ~np.uint64((1 << 12) - 1)
    return b.view(np.float64)


def main():
    import oracle as O

    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    geo, F = workload()
    o = O.OracleSolver(geo, 2, 2, TOL, 64, 64, threads)
    t0 = time.time()
    o.build_tree()
    o.factor()
    mu, alpha = o.solve(F)
    t1 = time.time()
    np.savez_compressed(OUT, mu=round40(np.asarray(mu)[:, 0]), alpha=round40(alpha),
                        n_points=N_POINTS, holes=HOLES, semi=np.array(SEMI), tol=TOL,
                        threads=threads, seconds=t1 - t0)
    print(f"{OUT}: {geo.n} points, factor + solve {t1 - t0:.0f} s on {threads} threads")


if __name__ == "__main__":
    main()
