"""Seeded boundary generators for the solver's workloads.

Every generator returns a :class:`Geometry`: the four per-node arrays the
solver consumes (points, outward normals, quadrature weights, signed
curvatures), the hole list used by the multiply-connected (bordered) system,
and helpers for boundary data.  The node/array conventions follow the
reference solver's ``Boundary`` class (ie_solver/boundaries/boundary.h:34-65):

* ``points`` and ``normals`` are interleaved ``[x0, y0, x1, y1, ...]``;
* the outer curve comes first, then each hole's nodes in hole order;
* normals point out of the fluid/potential domain (so into each hole) and
  hole curvatures are negative, as in ie_solver/boundaries/annulus.cpp:51-58;
* weights are trapezoidal: |gamma'(t)| * 2*pi / n for a curve with n nodes.

Workloads (all seeded, no external data):

* ``unit_circle(n)`` - unit circle, f = Re(1/(z - z0)), z0 = (2, 0).
* ``star(n, a=0.3, k=5)`` - r(t) = 1 + a cos(k t).
* ``random_star(n, rng)`` - r(t) = 1 + sum_{k=2..8} a_k cos(k t + phi_k),
  a_k ~ U[0, 0.04], phi_k ~ U[0, 2 pi].
* ``circle_with_ellipses(n_total, n_holes, rng)`` - outer unit circle plus
  seeded non-overlapping interior ellipses, semi-axes U[0.05, 0.15].
* ``reference_circle(n)`` / ``reference_annulus(n)`` / ``reference_donut(n)``
  - the reference test shapes (ie_solver/boundaries/circle.cpp:9-34,
  annulus.cpp:9-70, donut.cpp:9-52).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

LAPLACE = 0
LAPLACE_NEUMANN = 1
STOKES = 2


@dataclasses.dataclass
class Geometry:
    points: np.ndarray       # (2n,) interleaved x, y
    normals: np.ndarray      # (2n,) interleaved
    weights: np.ndarray      # (n,)
    curvatures: np.ndarray   # (n,)
    hole_centers: np.ndarray  # (2h,) interleaved
    hole_radii: np.ndarray    # (h,) radius used for hole membership
    num_outer: int = 0

    @property
    def n(self) -> int:
        return self.weights.shape[0]

    @property
    def num_holes(self) -> int:
        return self.hole_radii.shape[0]

    def xy(self) -> np.ndarray:
        return self.points.reshape(-1, 2)


def _param_curve(n, x, y, dx, dy, ddx, ddy, orient=1.0):
    """Nodes, normals, weights and curvature of a closed curve sampled at
    t_i = 2 pi i / n.  ``orient=+1`` gives the outward normal of a
    counter-clockwise curve; ``orient=-1`` flips normal and curvature (holes).
    """
    speed = np.sqrt(dx * dx + dy * dy)
    nx = orient * dy / speed
    ny = -orient * dx / speed
    kappa = orient * (dx * ddy - dy * ddx) / speed ** 3
    w = speed * (2.0 * math.pi / n)
    pts = np.empty(2 * n)
    pts[0::2] = x
    pts[1::2] = y
    nrm = np.empty(2 * n)
    nrm[0::2] = nx
    nrm[1::2] = ny
    return pts, nrm, w, kappa


def _radial(n, r, dr, ddr, cx=0.0, cy=0.0, orient=1.0):
    t = 2.0 * math.pi * np.arange(n) / n
    c, s = np.cos(t), np.sin(t)
    rt, drt, ddrt = r(t), dr(t), ddr(t)
    x = cx + rt * c
    y = cy + rt * s
    dx = drt * c - rt * s
    dy = drt * s + rt * c
    ddx = ddrt * c - 2 * drt * s - rt * c
    ddy = ddrt * s + 2 * drt * c - rt * s
    return _param_curve(n, x, y, dx, dy, ddx, ddy, orient)


def _empty_holes():
    return np.zeros(0), np.zeros(0)


def unit_circle(n: int) -> Geometry:
    t = 2.0 * math.pi * np.arange(n) / n
    pts = np.empty(2 * n)
    pts[0::2] = np.cos(t)
    pts[1::2] = np.sin(t)
    nrm = pts.copy()
    w = np.full(n, 2.0 * math.pi / n)
    kappa = np.ones(n)
    hc, hr = _empty_holes()
    return Geometry(pts, nrm, w, kappa, hc, hr, n)


def star(n: int, a: float = 0.3, k: int = 5) -> Geometry:
    pts, nrm, w, kappa = _radial(
        n,
        lambda t: 1.0 + a * np.cos(k * t),
        lambda t: -a * k * np.sin(k * t),
        lambda t: -a * k * k * np.cos(k * t))
    hc, hr = _empty_holes()
    return Geometry(pts, nrm, w, kappa, hc, hr, n)


def random_star(n: int, rng: np.random.Generator) -> Geometry:
    ks = np.arange(2, 9)
    amp = rng.uniform(0.0, 0.04, size=ks.shape[0])
    phi = rng.uniform(0.0, 2.0 * math.pi, size=ks.shape[0])

    def r(t):
        return 1.0 + sum(a * np.cos(k * t + p) for a, k, p in zip(amp, ks, phi))

    def dr(t):
        return sum(-a * k * np.sin(k * t + p) for a, k, p in zip(amp, ks, phi))

    def ddr(t):
        return sum(-a * k * k * np.cos(k * t + p) for a, k, p in zip(amp, ks, phi))

    pts, nrm, w, kappa = _radial(n, r, dr, ddr)
    hc, hr = _empty_holes()
    return Geometry(pts, nrm, w, kappa, hc, hr, n)


def _ellipse(n, cx, cy, a, b, theta, orient):
    t = 2.0 * math.pi * np.arange(n) / n
    ct, st = math.cos(theta), math.sin(theta)
    ex, ey = a * np.cos(t), b * np.sin(t)
    dex, dey = -a * np.sin(t), b * np.cos(t)
    ddex, ddey = -a * np.cos(t), -b * np.sin(t)
    x = cx + ct * ex - st * ey
    y = cy + st * ex + ct * ey
    dx = ct * dex - st * dey
    dy = st * dex + ct * dey
    ddx = ct * ddex - st * ddey
    ddy = st * ddex + ct * ddey
    return _param_curve(n, x, y, dx, dy, ddx, ddy, orient)


def ellipse(n: int, a: float, b: float, theta: float = 0.0) -> Geometry:
    """Interior of the ellipse with semi-axes a, b rotated by theta, n nodes
    equispaced in the parameter."""
    pts, nrm, w, kappa = _ellipse(n, 0.0, 0.0, a, b, theta, 1.0)
    hc, hr = _empty_holes()
    return Geometry(pts, nrm, w, kappa, hc, hr, n)


def rank_training_curves(count: int, seed: int, n_range=(8192, 65536)):
    """Seeded star and ellipse boundaries for training the rank model:
    random stars r(t) = 1 + sum_{k=2..8} a_k cos(kt + phi_k), stars
    1 + a cos(kt) with a in [0.05, 0.35], k in 3..9, and ellipses with axis
    ratio in [0.3, 1]; n uniform in n_range (multiples of 1024)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = 1024 * int(rng.integers(n_range[0] // 1024, n_range[1] // 1024 + 1))
        kind = i % 3
        if kind == 0:
            out.append(random_star(n, rng))
        elif kind == 1:
            out.append(star(n, a=float(rng.uniform(0.05, 0.35)), k=int(rng.integers(3, 10))))
        else:
            out.append(ellipse(n, 1.0, float(rng.uniform(0.3, 1.0)),
                               float(rng.uniform(0, math.pi))))
    return out


def _ellipse_perimeter(a, b):
    h = ((a - b) / (a + b)) ** 2
    return math.pi * (a + b) * (1 + 3 * h / (10 + math.sqrt(4 - 3 * h)))


def circle_with_ellipses(n_total: int, n_holes: int, rng: np.random.Generator,
                         semi=(0.05, 0.15), margin=0.02, max_r=0.85,
                         node_multiple=8) -> Geometry:
    """Outer unit circle plus ``n_holes`` interior ellipses.

    Hole membership in the bordered system is decided by the circle of radius
    ``hole_radii[h]`` around each centre (ie_solver/linear_solve.cpp:81,95),
    so every ellipse's radius is its semi-major axis and the circumscribed
    circles (plus ``margin``) are kept disjoint and inside r < ``max_r``.
    Node counts are proportional to perimeter, rounded to ``node_multiple``.
    """
    holes = []
    tries = 0
    while len(holes) < n_holes:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place the requested holes")
        a = rng.uniform(*semi)
        b = rng.uniform(*semi)
        a, b = max(a, b), min(a, b)
        rc = math.sqrt(rng.uniform(0.0, 1.0)) * (max_r - a)
        ang = rng.uniform(0.0, 2.0 * math.pi)
        cx, cy = rc * math.cos(ang), rc * math.sin(ang)
        ok = True
        for (hx, hy, ha, _, _) in holes:
            if math.hypot(cx - hx, cy - hy) < a + ha + margin:
                ok = False
                break
        if ok:
            holes.append((cx, cy, a, b, rng.uniform(0.0, math.pi)))
    perims = [2.0 * math.pi] + [_ellipse_perimeter(a, b) for (_, _, a, b, _) in holes]
    total = sum(perims)
    counts = [max(node_multiple, int(round(n_total * p / total / node_multiple)) * node_multiple)
              for p in perims]
    counts[0] += n_total - sum(counts)
    parts = []
    t = 2.0 * math.pi * np.arange(counts[0]) / counts[0]
    pts = np.empty(2 * counts[0])
    pts[0::2] = np.cos(t)
    pts[1::2] = np.sin(t)
    parts.append((pts, pts.copy(), np.full(counts[0], 2.0 * math.pi / counts[0]),
                  np.ones(counts[0])))
    for (cx, cy, a, b, th), cnt in zip(holes, counts[1:]):
        parts.append(_ellipse(cnt, cx, cy, a, b, th, orient=-1.0))
    hc = np.array([v for (cx, cy, _, _, _) in holes for v in (cx, cy)], dtype=np.float64)
    hr = np.array([a for (_, _, a, _, _) in holes], dtype=np.float64)
    return Geometry(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]),
                    np.concatenate([p[2] for p in parts]), np.concatenate([p[3] for p in parts]),
                    hc, hr, counts[0])


def reference_circle(n: int) -> Geometry:
    """ie_solver/boundaries/circle.cpp:9-24: centre (0.5, 0.5), radius 0.25."""
    t = np.arange(n) * 2.0 * math.pi / n
    pts = np.empty(2 * n)
    pts[0::2] = 0.5 + 0.25 * np.cos(t)
    pts[1::2] = 0.5 + 0.25 * np.sin(t)
    nrm = np.empty(2 * n)
    nrm[0::2] = np.cos(t)
    nrm[1::2] = np.sin(t)
    hc, hr = _empty_holes()
    return Geometry(pts, nrm, np.full(n, math.pi / (n * 2)), np.full(n, 4.0), hc, hr, n)


def reference_annulus(n: int) -> Geometry:
    """ie_solver/boundaries/annulus.cpp:9-59: unit circle around (0.5, 0.5)
    with two holes of radius 0.2 at (0.9, 0.5) and (0.1, 0.5), n/5 nodes each."""
    t = np.arange(n) * 2.0 * math.pi / n
    pts = [0.5 + np.cos(t), 0.5 + np.sin(t)]
    xs, ys = [pts[0]], [pts[1]]
    nxs, nys = [np.cos(t)], [np.sin(t)]
    ws = [np.full(n, 2 * math.pi / n)]
    ks = [np.ones(n)]
    hole_nodes = n // 5
    centers = [(0.9, 0.5), (0.1, 0.5)]
    for (cx, cy) in centers:
        th = np.arange(hole_nodes) * 2.0 * math.pi / hole_nodes
        xs.append(cx + 0.2 * np.cos(th))
        ys.append(cy + 0.2 * np.sin(th))
        nxs.append(-np.cos(th))
        nys.append(-np.sin(th))
        ws.append(np.full(hole_nodes, 2 * 0.2 * math.pi / hole_nodes))
        ks.append(np.full(hole_nodes, -1.0 / 0.2))
    x, y = np.concatenate(xs), np.concatenate(ys)
    p = np.empty(2 * x.shape[0])
    p[0::2], p[1::2] = x, y
    nx, ny = np.concatenate(nxs), np.concatenate(nys)
    q = np.empty(2 * x.shape[0])
    q[0::2], q[1::2] = nx, ny
    return Geometry(p, q, np.concatenate(ws), np.concatenate(ks),
                    np.array([0.9, 0.5, 0.1, 0.5]), np.array([0.2, 0.2]), n)


# ---------------------------------------------------------------------------
# Boundary data
# ---------------------------------------------------------------------------

def star_bump(n: int, center: float, height: float = 0.05, width: float = 0.3,
              a: float = 0.3, k: int = 5) -> Geometry:
    """The star r(t) = 1 + a cos(k t) plus a raised-cosine bump of the given
    height on |t - center| < width (angles mod 2 pi).  Nodes outside the bump
    are bit-identical to ``star(n, a, k)``'s, so moving the bump changes the
    boundary locally, as the reference's update experiments do
    (ie_solver_test.cpp:577-612)."""
    def wrap(t):
        return (t - center + math.pi) % (2 * math.pi) - math.pi

    def bump(t):
        u = wrap(t)
        inside = np.abs(u) < width
        return np.where(inside, height * 0.5 * (1 + np.cos(math.pi * u / width)), 0.0)

    def dbump(t):
        u = wrap(t)
        inside = np.abs(u) < width
        return np.where(inside, -height * 0.5 * math.pi / width * np.sin(math.pi * u / width), 0.0)

    def ddbump(t):
        u = wrap(t)
        inside = np.abs(u) < width
        return np.where(inside, -height * 0.5 * (math.pi / width) ** 2 * np.cos(math.pi * u / width),
                        0.0)

    pts, nrm, w, kappa = _radial(
        n,
        lambda t: (1.0 + a * np.cos(k * t)) + bump(t),
        lambda t: (-a * k * np.sin(k * t)) + dbump(t),
        lambda t: (-a * k * k * np.cos(k * t)) + ddbump(t),
    )
    hc, hr = _empty_holes()
    return Geometry(pts, nrm, w, kappa, hc, hr, n)


def reference_donut(n: int) -> Geometry:
    """ie_solver/boundaries/donut.cpp:9-52: unit circle around (0.5, 0.5) with
    one concentric hole of radius 0.5 carrying n/5 nodes."""
    t = np.arange(n) * 2.0 * math.pi / n
    hn = n // 5
    th = np.arange(hn) * 2.0 * math.pi / hn
    x = np.concatenate([0.5 + np.cos(t), 0.5 + 0.5 * np.cos(th)])
    y = np.concatenate([0.5 + np.sin(t), 0.5 + 0.5 * np.sin(th)])
    nx = np.concatenate([np.cos(t), -np.cos(th)])
    ny = np.concatenate([np.sin(t), -np.sin(th)])
    p = np.empty(2 * x.shape[0])
    p[0::2], p[1::2] = x, y
    nr = np.empty(2 * x.shape[0])
    nr[0::2], nr[1::2] = nx, ny
    w = np.concatenate([np.full(n, 2 * math.pi / n), np.full(hn, 2 * 0.5 * math.pi / hn)])
    k = np.concatenate([np.ones(n), np.full(hn, -2.0)])
    return Geometry(p, nr, w, k, np.array([0.5, 0.5]), np.array([0.5]), n)


def donut_neumann_data(geo: Geometry) -> np.ndarray:
    """The donut's DEFAULT Neumann data (donut.cpp:54-61): 1 on the outer
    circle, -1/r_hole on the hole; u = log|x - (0.5, 0.5)| + const solves it."""
    f = np.ones(geo.n)
    f[geo.num_outer:] = -1.0 / geo.hole_radii[0]
    return f


def laplace_point_source(geo: Geometry, src) -> np.ndarray:
    """f(x) = log|x - src| / (2 pi): harmonic inside the domain for an
    exterior source (ie_solver/boundaries/boundary.cpp:49-54 uses (-3, -2))."""
    xy = geo.xy()
    return np.log(np.hypot(xy[:, 0] - src[0], xy[:, 1] - src[1])) / (2.0 * math.pi)


def laplace_cauchy(geo: Geometry, z0=(2.0, 0.0)) -> np.ndarray:
    """f(x) = Re(1 / (z - z0))."""
    xy = geo.xy()
    z = (xy[:, 0] - z0[0]) + 1j * (xy[:, 1] - z0[1])
    return np.real(1.0 / z)


def stokeslet_velocity(geo: Geometry, src, force) -> np.ndarray:
    """Velocity of a 2D Stokeslet at ``src`` with ``force``, interleaved per
    node: u = (1/4pi) (-log r I + r r^T / r^2) F."""
    xy = geo.xy()
    rx = xy[:, 0] - src[0]
    ry = xy[:, 1] - src[1]
    r2 = rx * rx + ry * ry
    lg = -0.5 * np.log(r2)
    dot = (rx * force[0] + ry * force[1]) / r2
    u = np.empty(2 * xy.shape[0])
    u[0::2] = (lg * force[0] + rx * dot) / (4 * math.pi)
    u[1::2] = (lg * force[1] + ry * dot) / (4 * math.pi)
    return u


def tangent_data(geo: Geometry) -> np.ndarray:
    """TANGENT_VEC boundary data (ie_solver/boundaries/boundary.cpp:68-71)."""
    f = np.empty(2 * geo.n)
    f[0::2] = -geo.normals[1::2]
    f[1::2] = geo.normals[0::2]
    return f
