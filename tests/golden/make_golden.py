"""Generates the golden fixtures in tests/golden/ by running the reference
solver itself (built from its own sources by ``make -C oracle ref`` into
oracle/_ref/, driven by oracle/ref_dump.cpp).

Each case stores the reference's quadtree (level order, corners, neighbour
lists, original DOF boxes), its skeleton bookkeeping (active / skel /
redundant / near lists, allskel), its solution mu (and alpha with holes), and
the max-norm backward error against the dense operator that the reference's
own test computes (ie_solver_test.cpp:29-96).  The ID cases store matrices
from real boxes with the reference's ie_Mat::id output (rank, pivots, Z).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "ie-solver_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from rskel import geometry as g  # noqa: E402
import oracle as O  # noqa: E402
import refio  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

TREE_KEYS = ("level_sizes", "node_level", "node_leaf", "node_parent", "node_children",
             "node_corners", "node_side", "nbr_off", "nbr", "orig_off", "orig", "active_off",
             "active", "skel_off", "skel", "red_off", "red", "near_off", "near",
             "node_compressed", "allskel", "tree_minmax")


def cases():
    """(name, geometry, pde, sd, rhs, tol, leaf, npp)."""
    out = []
    geo = g.reference_circle(512)
    out.append(("laplace_circle_512", geo, 0, 1, g.laplace_point_source(geo, (-3.0, -2.0)),
                1e-6, 32, 128))
    out.append(("stokes_circle_512", geo, 2, 2, g.tangent_data(geo), 1e-6, 32, 128))
    geo = g.reference_annulus(512)
    out.append(("laplace_annulus_512", geo, 0, 1, g.laplace_point_source(geo, (-3.0, -2.0)),
                1e-6, 32, 128))
    out.append(("stokes_annulus_512", geo, 2, 2, g.tangent_data(geo), 1e-6, 32, 128))
    geo = g.unit_circle(4096)
    out.append(("laplace_unit_circle_4096", geo, 0, 1, g.laplace_cauchy(geo), 1e-10, 64, 64))
    geo = g.star(8192)
    rng = np.random.default_rng(2)
    th = rng.uniform(0, 2 * np.pi, 2)
    rhs = np.stack([g.laplace_point_source(geo, (2 * np.cos(t), 2 * np.sin(t))) for t in th], 1)
    out.append(("laplace_star_8192_2rhs", geo, 0, 1, rhs, 1e-8, 64, 64))
    geo = g.circle_with_ellipses(4096, 4, np.random.default_rng(3))
    out.append(("stokes_ellipses_4096", geo, 2, 2,
                g.stokeslet_velocity(geo, (1.6, 0.4), (1.0, 0.5)), 1e-8, 64, 64))
    return out


def subset(geo, keep):
    """The boundary with only the nodes where `keep` is true."""
    xy, nv = geo.points.reshape(-1, 2), geo.normals.reshape(-1, 2)
    return g.Geometry(xy[keep].ravel(), nv[keep].ravel(), geo.weights[keep],
                      geo.curvatures[keep], geo.hole_centers, geo.hole_radii, int(keep.sum()))


def perturb_cases():
    """(name, sd, leaf, npp, [boundaries]): QuadTree::initialize_tree on the
    first boundary, then QuadTree::perturb with each later one.  A bump
    moving along a star moves points between leaves (bursting leaves split);
    removing every third node of the bump's arc and putting it back empties
    and refills leaves (sparse subtrees are consolidated, then split again)."""
    out = []
    for height, sd, leaf, npp in ((0.05, 1, 32, 128), (0.2, 1, 32, 128), (0.2, 1, 64, 64),
                                  (0.3, 2, 32, 128)):
        geos = [g.star_bump(4096, center=float(c), height=height)
                for c in [0.0] + list(np.linspace(0.3, 3.0, 5))]
        out.append((f"bump{height:g}_sd{sd}_leaf{leaf}", sd, leaf, npp, geos))
    base = g.star_bump(4096, center=1.0, height=0.2)
    t = np.arange(base.n)
    arc = (t > 400) & (t < 1400)
    thin = subset(base, ~(arc & (t % 3 != 0)))
    out.append(("thin_refill_leaf32", 1, 32, 128, [base, thin, base, thin]))
    return out


def save_geometry(d, geo):
    d["points"] = geo.points
    d["normals"] = geo.normals
    d["weights"] = geo.weights
    d["curvatures"] = geo.curvatures
    d["hole_centers"] = geo.hole_centers
    d["hole_radii"] = geo.hole_radii


def main():
    for name, geo, pde, sd, rhs, tol, leaf, npp in cases():
        res = refio.run_reference(geo, pde, sd, rhs, tol, leaf=leaf, npp=npp, threads=1,
                                  dense_check=True)
        d = {k: res[k] for k in TREE_KEYS}
        d["mu"] = res["mu"]
        if "alpha" in res:
            d["alpha"] = res["alpha"]
        d["dense_residual_max"] = np.array([np.abs(res["dense_residual"]).max()])
        d["meta"] = np.array([pde, sd, leaf, npp, geo.n, geo.num_holes,
                              rhs.shape[1] if rhs.ndim == 2 else 1])
        d["tol"] = np.array([tol])
        d["rhs"] = np.asarray(rhs, dtype=np.float64)
        save_geometry(d, geo)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **d)
        print(name, "nodes", len(d["node_level"]), "residual", d["dense_residual_max"][0])
    # ID fixtures: matrices of real boxes (built by the oracle restatement,
    # whose ID matrices follow kernel.cpp:293-423) with the reference's ID.
    mats, tols, meta = [], [], []
    for name, geo, pde, sd, rhs, tol, leaf, npp in cases()[4:7]:
        s = O.OracleSolver(geo, pde, sd, tol, leaf, npp)
        s.build_tree()
        s.factor()
        picked = 0
        for i in range(s.num_nodes() - 1, 0, -1):
            info, _, _ = s.node_info(i)
            if info[7] and picked < 6:
                A = s.id_matrix(i)
                mats.append(A)
                tols.append(tol)
                meta.append((pde, info[0]))
                picked += 1
    ref = refio.run_reference_id(mats, tols)
    d = {"ranks": ref["ranks"], "perm": ref["perm"], "perm_off": ref["perm_off"], "z": ref["z"],
         "z_off": ref["z_off"], "dims": ref["dims"], "tols": np.array(tols),
         "meta": np.array(meta, dtype=np.int32)}
    for i, A in enumerate(mats):
        d[f"A{i}"] = A
    np.savez_compressed(os.path.join(OUT, "id_cases.npz"), **d)
    print("id cases", len(mats), "ranks", ref["ranks"])
    # perturbed trees: the reference's QuadTree::perturb after each sequence
    d = {}
    for name, sd, leaf, npp, geos in perturb_cases():
        res = refio.run_reference_perturb(geos, sd, leaf, npp)
        for k in ("level_sizes", "node_level", "node_leaf", "node_parent", "node_children",
                  "node_corners", "nbr_off", "nbr", "orig_off", "orig"):
            d[f"{name}/{k}"] = res[k]
        print("perturb", name, "levels", list(res["level_sizes"]))
    np.savez_compressed(os.path.join(OUT, "perturb_trees.npz"), **d)


if __name__ == "__main__":
    main()
