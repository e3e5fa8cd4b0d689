"""Quadtree construction and DOF orderings, bit-exact against the reference.

The golden fixtures (tests/golden/*.npz) hold the reference's own trees
(ie_solver/quadtree/quadtree.cpp:39-432, dumped by oracle/ref_dump.cpp).  The
product builds its tree on the host (no GPU needed), so these run on CPU.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_geometry, load_golden

TREE_FIELDS = ("level_sizes", "node_level", "node_leaf", "node_parent", "node_children",
               "node_corners", "node_side", "nbr_off", "nbr", "orig_off", "orig")


def _pde(d):
    return int(d["meta"][0])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_product_tree_matches_reference(name, solver_lib):
    d = load_golden(name)
    geo = golden_geometry(d)
    pde, sd, leaf, npp = (int(x) for x in d["meta"][:4])
    s = solver_lib.Solver(geo, pde, float(d["tol"][0]), leaf=leaf, npp=npp)
    s.build_tree()
    t = s.tree_dump()
    for f in TREE_FIELDS:
        assert t[f].shape == d[f].shape, f
        assert np.array_equal(t[f], d[f]), f
    mn, mx = s.tree_bounds()
    assert (mn, mx) == tuple(d["tree_minmax"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_tree_matches_reference(name, oracle_lib):
    d = load_golden(name)
    geo = golden_geometry(d)
    pde, sd, leaf, npp = (int(x) for x in d["meta"][:4])
    s = oracle_lib.OracleSolver(geo, pde, sd, float(d["tol"][0]), leaf, npp)
    s.build_tree()
    t = s.tree_dump()
    for f in TREE_FIELDS:
        assert np.array_equal(t[f], d[f]), f


def active_near_from_rules(d):
    """Recomputes every box's active and near lists from the reference's own
    skeletons with the bookkeeping rules (quadtree.cpp:997-1074): a box's
    active list is its children's (skel if compressed else active) in
    children order, leaves use their original box; near is the neighbours' at
    the same or coarser level (original for leaves, active otherwise)."""
    nn = len(d["node_level"])

    def lst(name, i):
        off = d[name + "_off"]
        return d[name][off[i]:off[i + 1]]

    active = {}
    order = sorted(range(nn), key=lambda i: -d["node_level"][i])
    for i in order:
        if d["node_leaf"][i]:
            active[i] = lst("orig", i)
        else:
            parts = []
            for c in d["node_children"][4 * i:4 * i + 4]:
                parts.append(lst("skel", c) if d["node_compressed"][c] else active[c])
            active[i] = np.concatenate(parts)
    near = {}
    for i in range(nn):
        parts = []
        for nb in lst("nbr", i):
            if d["node_level"][nb] > d["node_level"][i]:
                continue
            parts.append(lst("orig", nb) if d["node_leaf"][nb] else active[nb])
        near[i] = np.concatenate(parts) if parts else np.zeros(0, dtype=np.int32)
    return active, near


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_reference_bookkeeping_rules(name):
    """The list rules the product and oracle implement reproduce the
    reference's own active/near lists from its skeletons."""
    d = load_golden(name)
    active, near = active_near_from_rules(d)
    for i in range(len(d["node_level"])):
        off = d["active_off"]
        assert np.array_equal(active[i], d["active"][off[i]:off[i + 1]]), i
        off = d["near_off"]
        assert np.array_equal(near[i], d["near"][off[i]:off[i + 1]]), i
    root_children = d["node_children"][0:4]
    assert np.array_equal(active[0], d["allskel"]) or len(root_children) == 0


def test_tree_edge_cases(solver_lib):
    from rskel import geometry as g

    # a single point (one leaf, one level)
    geo = g.unit_circle(1)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-6, leaf=32, npp=16)
    s.build_tree()
    assert s.stats()["num_levels"] == 1
    # exactly max_leaf_dofs points: no split; one more: split
    for n, lv in ((32, 1), (33, 2)):
        s = solver_lib.Solver(g.unit_circle(n), solver_lib.RS_LAPLACE, 1e-6, leaf=32, npp=16)
        s.build_tree()
        assert s.stats()["num_levels"] >= lv
        if n == 32:
            assert s.stats()["num_levels"] == 1
    # Stokes counts DOFs, not points: 17 points = 34 DOFs > 32 splits
    s = solver_lib.Solver(g.unit_circle(17), solver_lib.RS_STOKES, 1e-6, leaf=32, npp=16)
    s.build_tree()
    assert s.stats()["num_levels"] >= 2


def _cloud(n, rng, kind):
    """Point sets for the tree alone (normals and weights are placeholders):
    a uniform cloud, a cloud on an 8 x 8 lattice of clusters, and a thin
    sliver, each in a seeded random order."""
    from rskel.geometry import Geometry

    if kind == "uniform":
        xy = rng.random((n, 2))
    elif kind == "clusters":
        xy = np.floor(rng.random((n, 2)) * 8) / 8 + 1e-3 * rng.random((n, 2))
    else:
        t = rng.random(n) * 2 * np.pi
        xy = np.stack([3 * np.cos(t), 0.01 * np.sin(t)], axis=1)
    nrm = np.zeros_like(xy)
    nrm[:, 0] = 1.0
    return Geometry(points=xy.ravel().copy(), normals=nrm.ravel().copy(), weights=np.ones(n),
                    curvatures=np.zeros(n), hole_centers=np.zeros(0), hole_radii=np.zeros(0),
                    num_outer=n)


def test_product_tree_matches_oracle_on_varied_geometries(solver_lib, oracle_lib):
    """The product forms the tree by recursive partition of the point indices
    and numbers the boxes in the order insertion would create them; the
    oracle restates the reference's point-by-point insertion.  Trees, level
    lists, leaf lists and neighbour lists agree on curves, holes and point
    clouds, for one and two DOFs per point and several leaf sizes."""
    from rskel import geometry as g

    rng = np.random.default_rng(2024)
    geos = [g.random_star(int(rng.integers(500, 20000)), rng) for _ in range(3)]
    geos += [g.star(12000, 0.3, 7), g.reference_annulus(2048),
             g.circle_with_ellipses(16000, 8, np.random.default_rng(3)),
             g.ellipse(6000, 1.0, 0.05, 0.7)]
    geos += [_cloud(int(rng.integers(200, 9000)), rng, k) for k in ("uniform", "clusters", "sliver")]
    fields = ("level_sizes", "node_level", "node_leaf", "node_parent", "node_children",
              "node_corners", "nbr_off", "nbr", "orig_off", "orig")
    for geo in geos:
        for pde, sd in ((0, 1), (2, 2)):
            for leaf in (16, 33, 64):
                s = solver_lib.Solver(geo, pde, 1e-8, leaf=leaf, npp=64)
                s.build_tree()
                mine = s.tree_dump()
                o = oracle_lib.OracleSolver(geo, pde, sd, 1e-8, leaf, 64, 1)
                o.build_tree()
                ref = o.tree_dump()
                for f in fields:
                    assert np.array_equal(np.asarray(mine[f]), np.asarray(ref[f])), (geo.n, sd, leaf, f)
                s.close()


def test_coincident_points_are_refused(solver_lib):
    """More coincident points than a leaf holds can never be separated (the
    reference's insertion recursion would not end); the build reports an
    argument error instead."""
    from rskel import geometry as g

    geo = g.unit_circle(256)
    geo.points[2 * 10:2 * 60] = np.tile([0.25, 0.5], 50)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-6, leaf=16, npp=16)
    with pytest.raises(solver_lib.RsError) as e:
        s.build_tree()
    assert e.value.code == 1
