"""Training set and training of the learned skeleton-rank model.

The model (16 -> 64 -> 64 -> 1 multilayer perceptron, include/rskel.h
rs_rank_*) predicts each box's rank fraction k/n from its geometry.  Its
training data are the ranks the plain method itself produces: for every
boundary of a seeded family of random stars, rose curves and ellipses, one
plain FP32 factorization per kernel, whose (features, k/n) pairs
rs_rank_samples returns.  Training is full-batch Adam on the GPU with the
library's own forward and backward kernels (rs_rank_train).

The default family is 2000 boundaries (seed 5) of 1024 to 8192 points, each
factored with the Laplace double layer and with the Stokes double layer
(half as many points, the same number of DOFs), ID tolerance 1e-8, leaf 64
DOFs, 64 proxy points: the two kernels of the configurations the model is
used on.  No boundary of the family is a benchmark or test geometry.
"""
from __future__ import annotations

import time

import numpy as np

from . import capi
from . import geometry as g

FAMILY_SIZE, FAMILY_SEED, FAMILY_POINTS = 2000, 5, (1024, 8192)


def family(count=FAMILY_SIZE, seed=FAMILY_SEED, n_range=FAMILY_POINTS):
    """The seeded training boundaries (random stars, rose curves, ellipses)."""
    return g.rank_training_curves(count, seed, n_range)


def _halved(geo):
    """The same curve with every other node (weights doubled)."""
    return g.Geometry(np.asarray(geo.points).reshape(-1, 2)[::2].ravel(),
                      np.asarray(geo.normals).reshape(-1, 2)[::2].ravel(),
                      2.0 * np.asarray(geo.weights)[::2], np.asarray(geo.curvatures)[::2],
                      geo.hole_centers, geo.hole_radii, geo.n // 2)


def collect(boundaries, pdes=(capi.RS_LAPLACE, capi.RS_STOKES), tol=1e-8, leaf=64, npp=64,
            device=0):
    """(features, k/n) of plain FP32 factorizations of every boundary with each
    kernel in `pdes`; Stokes runs use every other node (same DOF count)."""
    Xs, ys = [], []
    for pde in pdes:
        s = None
        for geo in boundaries:
            gg = _halved(geo) if pde == capi.RS_STOKES else geo
            if s is None:
                s = capi.Solver(gg, pde, tol, leaf=leaf, npp=npp, precision=capi.RS_FP32_REFINE,
                                device=device)
            else:
                s.set_geometry(gg)
            s.factor()
            X, y = s.rank_samples()
            Xs.append(X)
            ys.append(y)
        if s is not None:
            s.close()
    return np.concatenate(Xs), np.concatenate(ys)


def train(X, y, epochs=2000, lr=3e-3, seed=0, device=0):
    """Full-batch Adam on the GPU from the deterministic initial weights;
    returns (weights, final mean squared error)."""
    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8, precision=capi.RS_FP32_REFINE,
                    device=device)
    w, loss = s.rank_train(X, y, capi.rank_model_init(seed), epochs=epochs, lr=lr)
    s.close()
    return w, loss


def train_family(count=FAMILY_SIZE, seed=FAMILY_SEED, n_range=FAMILY_POINTS, epochs=2000,
                 device=0):
    """The model trained on the seeded family; returns (weights, info)."""
    t0 = time.perf_counter()
    X, y = collect(family(count, seed, n_range), device=device)
    t1 = time.perf_counter()
    w, loss = train(X, y, epochs=epochs, device=device)
    info = {"boundaries": count, "seed": seed, "points": list(n_range),
            "kernels": ["laplace", "stokes"], "samples": int(len(y)), "epochs": epochs,
            "final_mse": loss, "collect_s": t1 - t0, "train_s": time.perf_counter() - t1}
    return w, info
