"""Host-side QuadTree::perturb (quadtree.cpp:435-801) through rs_perturb on a
tree that has not been factored (no GPU needed): after moving a local bump
along a star-shaped boundary, the updated tree must still be a valid
quadtree of the new points, and it must equal, bit for bit, the tree the
reference's own QuadTree::perturb leaves after the same sequence of
boundaries (tests/golden/perturb_trees.npz, made by the reference built from
its sources through oracle/ref_dump.cpp --perturb; the live reference too
where its build is present).

Compared: level sizes, node order, levels, leaf flags, parents, children,
corners, neighbour lists and the leaves' DOF lists in order.  Interior
boxes' DOF lists are not compared: the reference remaps original_box on
leaves only (quadtree.cpp:585-597), so after a perturbation its interior
lists keep the old numbering, which nothing reads (the factorization builds
interior active lists from the children, quadtree.cpp:1032-1055).
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

STRUCT_KEYS = ("level_sizes", "node_level", "node_leaf", "node_parent", "node_children",
               "node_corners", "nbr_off", "nbr")


def _leaf_lists(d):
    return [d["orig"][d["orig_off"][i]:d["orig_off"][i + 1]].tolist()
            for i in range(len(d["node_level"])) if d["node_leaf"][i]]


def _perturb_cases():
    sys.path.insert(0, os.path.join(GOLDEN))
    import make_golden

    return make_golden.perturb_cases()


def _product_tree(capi, sd, leaf, npp, geos):
    pde = capi.RS_LAPLACE if sd == 1 else capi.RS_STOKES
    s = capi.Solver(geos[0], pde, 1e-8, leaf=leaf, npp=npp)
    s.build_tree()
    for geo in geos[1:]:
        s.set_geometry(geo, perturb=True)
    d = s.tree_dump()
    s.close()
    return d


def _assert_same_tree(d, r, name):
    for k in STRUCT_KEYS:
        assert np.array_equal(d[k], r[k]), (name, k)
    assert _leaf_lists(d) == _leaf_lists(r), name


def test_perturbed_trees_match_the_reference_fixtures(solver_lib):
    ref = np.load(os.path.join(GOLDEN, "perturb_trees.npz"))
    for name, sd, leaf, npp, geos in _perturb_cases():
        r = {k: ref[f"{name}/{k}"] for k in STRUCT_KEYS + ("orig_off", "orig")}
        d = _product_tree(solver_lib, sd, leaf, npp, geos)
        _assert_same_tree(d, r, name)
        # the history matters: a fresh tree of the last boundary differs
        f = solver_lib.Solver(geos[-1], solver_lib.RS_LAPLACE if sd == 1 else solver_lib.RS_STOKES,
                              1e-8, leaf=leaf, npp=npp)
        f.build_tree()
        fd = f.tree_dump()
        f.close()
        assert not (np.array_equal(fd["level_sizes"], d["level_sizes"]) and
                    np.array_equal(fd["nbr"], d["nbr"])), name


def test_perturbed_tree_matches_the_live_reference(solver_lib):
    refio = pytest.importorskip("refio")
    if refio.ref_binary(32, 128) is None:
        pytest.skip("reference build (oracle/_ref) not present")
    from rskel import geometry as G

    rng = np.random.default_rng(21)
    geos = [G.star_bump(3000, center=float(c), height=float(h))
            for c, h in zip(rng.uniform(0, 6.28, 4), rng.uniform(0.05, 0.3, 4))]
    for sd in (1, 2):
        r = refio.run_reference_perturb(geos, sd, 32, 128)
        _assert_same_tree(_product_tree(solver_lib, sd, 32, 128, geos), r, f"live sd{sd}")


def _check_tree(s, geo, leaf):
    d = s.tree_dump()
    nn = len(d["node_level"])
    lev, isleaf, par = d["node_level"], d["node_leaf"], d["node_parent"]
    ch = d["node_children"].reshape(-1, 4)
    cor = d["node_corners"].reshape(-1, 8)
    side = d["node_side"]
    pts = geo.xy()
    seen = np.zeros(geo.n, dtype=int)
    for i in range(nn):
        if not isleaf[i]:
            for c in ch[i]:
                assert c >= 0 and par[c] == i and lev[c] == lev[i] + 1
                assert abs(side[c] - side[i] / 2) <= 1e-15 * side[i]
            continue
        dofs = d["orig"][d["orig_off"][i]:d["orig_off"][i + 1]]
        assert len(dofs) <= leaf or lev[i] == 0
        p = pts[dofs]
        x0, y0 = cor[i, 0], cor[i, 1]
        assert np.all(p[:, 0] >= x0 - 1e-12) and np.all(p[:, 0] <= x0 + side[i] + 1e-12)
        assert np.all(p[:, 1] >= y0 - 1e-12) and np.all(p[:, 1] <= y0 + side[i] + 1e-12)
        seen[dofs] += 1
    assert np.all(seen == 1)  # the leaves partition the points
    assert np.array_equal(d["level_sizes"], np.bincount(lev, minlength=len(d["level_sizes"])))


@pytest.mark.parametrize("height", [0.05, 0.2])
def test_perturbed_tree_is_a_quadtree_of_the_new_points(solver_lib, height):
    from rskel import geometry as G

    leaf = 32
    geo0 = G.star_bump(4096, center=0.0, height=height)
    s = solver_lib.Solver(geo0, solver_lib.RS_LAPLACE, 1e-8, leaf=leaf)
    s.build_tree()
    for c in np.linspace(0.3, 3.0, 5):
        geo = G.star_bump(4096, center=float(c), height=height)
        s.set_geometry(geo, perturb=True)
        _check_tree(s, geo, leaf)


def test_unchanged_boundary_keeps_the_tree(solver_lib):
    from rskel import geometry as G

    geo = G.star_bump(2048, center=1.0)
    s = solver_lib.Solver(geo, solver_lib.RS_LAPLACE, 1e-8, leaf=32)
    s.build_tree()
    before = s.tree_dump()
    s.set_geometry(geo, perturb=True)
    after = s.tree_dump()
    for k in ("node_level", "node_leaf", "node_children", "orig", "nbr"):
        assert np.array_equal(before[k], after[k]), k
