"""The seeded synthetic workloads against the configurations they stand for
(CPU only): the boundary shapes, node counts, hole placement and the
quadrature the benchmark and the full-size parity tests feed the solver.

* Laplace star r(t) = 1 + 0.3 cos 5t, 65536 nodes: every node on the curve,
  unit outward normals, trapezoidal weights summing to the perimeter, and
  the signed curvature of the parametrised curve.
* Random stars r(t) = 1 + sum_{k=2..8} a_k cos(kt + phi_k), a_k in [0, 0.04].
* Unit circle plus 16 ellipses, semi-axes in [0.05, 0.15], 131072 nodes;
  unit circle plus 64 ellipses, semi-axes in [0.03, 0.06], 524288 nodes:
  the holes' circumscribed circles are disjoint and inside the unit circle,
  hole normals point into the holes (out of the domain), hole curvatures are
  negative, and the node counts add up.

Tolerances: 1e-12 on node positions and unit normals; perimeters by the
trapezoidal rule to 1e-10 relative (spectral for smooth periodic curves).
"""
import math

import numpy as np

from rskel import geometry as g


def _perimeter_quad(r, dr, n=1 << 16):
    t = 2.0 * math.pi * np.arange(n) / n
    return float(np.sum(np.hypot(r(t), dr(t))) * 2.0 * math.pi / n)


def test_star_65536():
    geo = g.star(65536)
    assert geo.n == 65536 and geo.num_holes == 0
    xy = geo.xy()
    th = np.arctan2(xy[:, 1], xy[:, 0])
    r = np.hypot(xy[:, 0], xy[:, 1])
    assert np.abs(r - (1.0 + 0.3 * np.cos(5 * th))).max() < 1e-12
    nv = geo.normals.reshape(-1, 2)
    assert np.abs(np.hypot(nv[:, 0], nv[:, 1]) - 1.0).max() < 1e-12
    assert (np.sum(nv * xy, axis=1) > 0).all()  # outward on a star-shaped curve
    per = _perimeter_quad(lambda t: 1 + 0.3 * np.cos(5 * t), lambda t: -1.5 * np.sin(5 * t))
    assert abs(geo.weights.sum() - per) < 1e-10 * per
    # curvature of r(t): (r^2 + 2 r'^2 - r r'') / (r^2 + r'^2)^(3/2) at the nodes
    t = 2.0 * math.pi * np.arange(geo.n) / geo.n
    rr, d1, d2 = 1 + 0.3 * np.cos(5 * t), -1.5 * np.sin(5 * t), -7.5 * np.cos(5 * t)
    kap = (rr * rr + 2 * d1 * d1 - rr * d2) / (rr * rr + d1 * d1) ** 1.5
    assert np.abs(geo.curvatures - kap).max() < 1e-10


def test_random_stars_stay_within_their_amplitudes():
    rng = np.random.default_rng(4)
    for _ in range(16):
        n = int(rng.integers(1024, 16385))
        geo = g.random_star(n, rng)
        assert geo.n == n
        r = np.hypot(*geo.xy().T)
        assert r.min() >= 1.0 - 7 * 0.04 - 1e-12 and r.max() <= 1.0 + 7 * 0.04 + 1e-12
        assert (geo.weights > 0).all()


def _check_holes(geo, n_total, n_holes, semi):
    assert geo.n == n_total and geo.num_holes == n_holes
    hc = geo.hole_centers.reshape(-1, 2)
    hr = geo.hole_radii
    assert ((hr >= semi[0]) & (hr <= semi[1])).all()
    assert (np.hypot(hc[:, 0], hc[:, 1]) + hr < 0.85 + 1e-12).all()
    d = np.hypot(hc[:, None, 0] - hc[None, :, 0], hc[:, None, 1] - hc[None, :, 1])
    np.fill_diagonal(d, np.inf)
    assert (d >= hr[:, None] + hr[None, :] + 0.02 - 1e-12).all()
    xy = geo.xy()
    nv = geo.normals.reshape(-1, 2)
    outer = geo.num_outer
    assert np.abs(np.hypot(*xy[:outer].T) - 1.0).max() < 1e-12
    # each hole node lies inside its hole's circle, normals into the hole,
    # negative curvature
    inner = xy[outer:]
    dist = np.hypot(inner[:, None, 0] - hc[None, :, 0], inner[:, None, 1] - hc[None, :, 1])
    owner = np.argmin(dist - hr[None, :], axis=1)
    assert (dist[np.arange(len(inner)), owner] <= hr[owner] + 1e-12).all()
    to_c = hc[owner] - inner
    assert (np.sum(nv[outer:] * to_c, axis=1) > 0).all()
    assert (geo.curvatures[outer:] < 0).all() and (geo.curvatures[:outer] > 0).all()


def test_circle_with_16_ellipses_131072():
    geo = g.circle_with_ellipses(131072, 16, np.random.default_rng(3))
    _check_holes(geo, 131072, 16, (0.05, 0.15))


def test_circle_with_64_ellipses_524288():
    geo = g.circle_with_ellipses(524288, 64, np.random.default_rng(3), semi=(0.03, 0.06))
    _check_holes(geo, 524288, 64, (0.03, 0.06))
