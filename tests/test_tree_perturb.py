"""Host-side QuadTree::perturb (quadtree.cpp:435-801) through rs_perturb on a
tree that has not been factored (no GPU needed): after moving a local bump
along a star-shaped boundary, the updated tree must still be a valid
quadtree of the new points."""
import numpy as np
import pytest


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
