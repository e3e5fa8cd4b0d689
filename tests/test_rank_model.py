"""Learned skeleton ranks: the rank model's hand-written CUDA inference,
gradient and Adam kernels against the oracle's float64 NumPy restatement
(itself pinned by central finite differences) and a PyTorch fp32 autograd
restatement of the same multilayer perceptron, and the FP32 factorization
with predicted sketch sizes against the plain one.

Tolerances: predicted fractions within 2e-6 of the restatements (fp32 sums
in another order); gradients within 1e-4 of max |grad| (the gradient kernel
accumulates with atomics in fp32); Adam steps within 1e-6 of the oracle's;
a factorization with a rank model is refined to the same accuracy bar as
without (1e-8 relative to the FP64 solution), whatever the model predicts.
"""
import numpy as np
import pytest

import rank_model as RM

RS_ERR_ARG = 1


def _torch_mlp(torch, w, X):
    from rskel import capi

    W1, b1, W2, b2, w3, b3 = (torch.tensor(a, dtype=torch.float32, requires_grad=True)
                              for a in capi.rank_unpack(w))
    x = torch.tensor(X, dtype=torch.float32)
    h1 = torch.relu(x @ W1.T + b1)
    h2 = torch.relu(h1 @ W2.T + b2)
    y = torch.sigmoid(h2 @ w3 + b3)
    return y, (W1, b1, W2, b2, w3, b3)


def _features(rng, count):
    X = rng.uniform(0.0, 1.0, (count, 16)).astype(np.float32)
    X[:, 6] = -X[:, 6]  # log box size relative to the root is negative
    return X


def test_init_is_deterministic_and_scaled(solver_lib):
    capi = solver_lib
    a, b, c = capi.rank_model_init(7), capi.rank_model_init(7), capi.rank_model_init(8)
    assert a.size == capi.RANK_WEIGHTS == 5313
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    W1, b1, W2, b2, w3, b3 = capi.rank_unpack(a)
    assert np.abs(W1).max() <= np.sqrt(6 / 16) and np.abs(W2).max() <= np.sqrt(6 / 64)
    assert not b1.any() and not b2.any() and b3[0] == 0.0
    assert W1.std() > 0.2 and W2.std() > 0.1


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = RM.pack([rng.normal(0, s, shape) for s, shape in
                 zip((0.6, 0.1, 0.3, 0.1, 0.3, 0.1), RM.SHAPES)])
    X = rng.uniform(-1, 1, (40, 16))
    t = rng.uniform(0.05, 0.95, 40)
    loss, g = RM.loss_and_gradient(w, X, t)
    assert np.isclose(loss, np.mean((RM.forward(w, X) - t) ** 2))
    idx = np.concatenate([rng.choice(RM.WEIGHTS, 60, replace=False), [RM.WEIGHTS - 1]])
    h = 1e-6
    for i in idx:
        e = np.zeros(RM.WEIGHTS)
        e[i] = h
        fd = (RM.loss_and_gradient(w + e, X, t)[0] - RM.loss_and_gradient(w - e, X, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_oracle_sketch_rows_rule():
    n = np.array([16, 40, 64, 128, 128])
    y = np.array([0.0, 0.5, 1.0, 0.25, 0.9])
    # ceil(1.15 ceil(y n)) + 10, at least 12, at most n + 16
    assert RM.sketch_rows(y, n).tolist() == [12, 33, 80, 47, 144]


def test_rank_entry_points_validate_arguments(solver_lib):
    import ctypes

    capi = solver_lib
    L = capi.lib()
    w = capi.rank_model_init(0)
    X = np.zeros((4, 16), dtype=np.float32)
    y = np.zeros(4, dtype=np.float32)
    f = capi._f
    # checks that come before any device call
    assert L.rs_rank_train(None, f(X), f(y), 4, 10, 1e-3, f(w), None) == RS_ERR_ARG
    assert L.rs_rank_predict(None, f(w), f(X), 4, f(y)) == RS_ERR_ARG
    assert L.rs_rank_gradient(None, f(w), f(X), f(y), 4, f(w), None) == RS_ERR_ARG
    cnt = ctypes.c_int(-1)
    assert L.rs_rank_samples(None, None, None, 0, ctypes.byref(cnt)) == RS_ERR_ARG
    assert L.rs_set_rank_model(None, f(w)) == RS_ERR_ARG


@pytest.mark.gpu
def test_predict_matches_torch(solver_lib):
    torch = pytest.importorskip("torch")
    from rskel import geometry as g

    capi = solver_lib
    rng = np.random.default_rng(3)
    w = capi.rank_model_init(5)
    w[capi.RANK_HIDDEN * 16:capi.RANK_HIDDEN * 17] = rng.normal(0, 0.2, capi.RANK_HIDDEN)  # b1
    w[-1] = 0.3
    X = _features(rng, 1000)
    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8)
    y = s.rank_predict(w, X)
    yt, _ = _torch_mlp(torch, w, X)
    assert np.abs(y - yt.detach().numpy()).max() <= 2e-6
    assert np.abs(y - RM.forward(w, X)).max() <= 2e-6
    assert s.rank_predict(w, X[:0]).size == 0


@pytest.mark.gpu
def test_gradient_matches_torch_autograd(solver_lib):
    torch = pytest.importorskip("torch")
    from rskel import geometry as g

    capi = solver_lib
    rng = np.random.default_rng(4)
    w = capi.rank_model_init(9)
    X = _features(rng, 777)
    t = rng.uniform(0.05, 0.9, 777).astype(np.float32)
    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8)
    grad, loss = s.rank_gradient(w, X, t)
    yt, params = _torch_mlp(torch, w, X)
    lt = ((yt - torch.tensor(t)) ** 2).mean()
    lt.backward()
    gt = np.concatenate([p.grad.numpy().ravel() for p in params])
    assert abs(loss - lt.item()) <= 1e-5 * max(1.0, lt.item())
    assert np.abs(grad - gt).max() <= 1e-4 * np.abs(gt).max()
    lo, go = RM.loss_and_gradient(w, X, t)
    assert abs(loss - lo) <= 1e-5 * max(1.0, lo)
    assert np.abs(grad - go).max() <= 1e-4 * np.abs(go).max()


@pytest.mark.gpu
def test_gradient_and_training_are_reproducible(solver_lib):
    """The gradient sums have a fixed order (no atomics): two calls, and two
    trainings from the same start, give bit-identical results."""
    from rskel import geometry as g

    capi = solver_lib
    rng = np.random.default_rng(8)
    X = _features(rng, 5000)
    t = rng.uniform(0.05, 0.9, 5000).astype(np.float32)
    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8)
    w0 = capi.rank_model_init(3)
    g1, l1 = s.rank_gradient(w0, X, t)
    g2, l2 = s.rank_gradient(w0, X, t)
    assert np.array_equal(g1, g2) and l1 == l2
    wa, la = s.rank_train(X, t, w0, epochs=50, lr=3e-3)
    wb, lb = s.rank_train(X, t, w0, epochs=50, lr=3e-3)
    assert np.array_equal(wa, wb) and la == lb


@pytest.mark.gpu
def test_adam_kernel_matches_oracle(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    rng = np.random.default_rng(6)
    X = _features(rng, 300)
    t = rng.uniform(0.1, 0.8, 300).astype(np.float32)
    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8)
    w0 = capi.rank_model_init(2)
    w3, _ = s.rank_train(X, t, w0, epochs=3, lr=1e-3)
    # the same three full-batch steps in float64
    w, m, v = w0.astype(np.float64), np.zeros(RM.WEIGHTS), np.zeros(RM.WEIGHTS)
    g1 = None
    for step in (1, 2, 3):
        _, gr = RM.loss_and_gradient(w, X, t)
        g1 = gr if g1 is None else g1
        w, m, v = RM.adam_step(w, gr, m, v, step, 1e-3)
    # Adam moves a weight by about lr per step whatever its gradient's size:
    # compare the moves where the gradient's sign is well determined (FP32
    # sums in another order may flip the sign of a gradient near zero), and
    # bound the rest
    sure = np.abs(g1) > 1e-3 * np.abs(g1).max()
    assert sure.sum() > 1000
    assert np.abs((w3 - w0) - (w - w0))[sure].max() <= 2e-5
    assert np.abs(w3 - w0).max() <= 3.03e-3


@pytest.mark.gpu
def test_training_lowers_the_loss(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    rng = np.random.default_rng(5)
    X = _features(rng, 2048)
    # a smooth rank-fraction-like target of the features
    t = (0.15 + 0.5 * X[:, 0] * (1 - 0.5 * X[:, 7]) + 0.2 * X[:, 10] ** 2).astype(np.float32)
    t = np.clip(t, 0.02, 0.98)
    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8)
    w0 = capi.rank_model_init(1)
    _, l0 = s.rank_gradient(w0, X, t)
    w1, l1 = s.rank_train(X, t, w0, epochs=400, lr=3e-3)
    _, l1b = s.rank_gradient(w1, X, t)
    assert l1 < 0.1 * l0 and l1b < 0.1 * l0
    assert np.abs(s.rank_predict(w1, X) - t).mean() < 0.05


def _mixed(capi, geo, **kw):
    return capi.Solver(geo, capi.RS_LAPLACE, 1e-8, leaf=64, npp=64,
                       precision=capi.RS_FP32_REFINE, refine_tol=1e-11, refine_max_iters=8,
                       fp32_id_tol=1e-6, **kw)


def _rhs(geo):
    from rskel import geometry as g

    return np.stack([g.laplace_point_source(geo, (2.5 * np.cos(a), 2.5 * np.sin(a)))
                     for a in (0.3, 2.0)], axis=1)


@pytest.mark.gpu
def test_learned_sketch_sizes_keep_the_solution(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    # training samples: plain mixed-precision factorizations of other curves
    Xs, ys = [], []
    rng = np.random.default_rng(12)
    for geo in (g.random_star(16384, rng), g.random_star(32768, rng), g.star(16384, a=0.2, k=7)):
        s = _mixed(capi, geo)
        s.factor()
        X, y = s.rank_samples()
        assert len(y) > 100 and np.all((y > 0) & (y <= 1))
        assert X.shape == (len(y), 16) and np.isfinite(X).all()
        Xs.append(X)
        ys.append(y)
        s.close()
    X, y = np.concatenate(Xs), np.concatenate(ys)
    t = _mixed(capi, g.star(32768))
    w, loss = t.rank_train(X, y, capi.rank_model_init(0), epochs=1500, lr=3e-3)
    assert loss < 0.01
    # plain and learned factorizations of a new curve
    F = _rhs(g.star(32768))
    t.factor()
    mu0, _ = t.solve(F)
    st0 = t.stats()
    assert st0["rank_predicted"] == 0
    t.set_rank_model(w)
    t.factor()
    mu1, _ = t.solve(F)
    st1 = t.stats()
    assert st1["rank_predicted"] > 100
    assert st1["rank_redo"] <= 0.25 * st1["rank_predicted"]
    # what the model gains: shorter sketches, less ID work
    assert st1["sketch_rows"] <= 0.85 * st0["sketch_rows"], (st1["sketch_rows"], st0["sketch_rows"])
    assert st1["id_flops"] <= 0.85 * st0["id_flops"]
    s64 = capi.Solver(g.star(32768), capi.RS_LAPLACE, 1e-8, leaf=64, npp=64)
    s64.factor()
    mu64, _ = s64.solve(F)
    rel = np.linalg.norm(mu1 - mu64) / np.linalg.norm(mu64)
    rel0 = np.linalg.norm(mu0 - mu64) / np.linalg.norm(mu64)
    assert rel <= 1e-8 and rel0 <= 1e-8, (rel, rel0)
    assert st1["refine_residual"] <= 1e-11
    # switching the model off gives the plain factorization back
    t.set_rank_model(None)
    t.factor()
    assert t.stats()["rank_predicted"] == 0


@pytest.mark.gpu
def test_too_small_predictions_fall_back_to_the_full_sketch(solver_lib):
    from rskel import geometry as g

    capi = solver_lib
    geo = g.star(32768)
    F = _rhs(geo)
    s = _mixed(capi, geo)
    s.factor()
    mu0, _ = s.solve(F)
    _, y0 = s.rank_samples()
    X0, _ = s.rank_samples()
    s0_rows = s.stats()["sketch_rows"]
    # plain ranks of the boxes whose sketch is predicted: at most 128 DOFs
    # (feature 0 is n / 128), on levels of at least one ID box per SM (152 on
    # a GB300; feature 5 is level / 16)
    n0 = np.rint(X0[:, 0] * 128.0)
    lv = np.rint(X0[:, 5] * 16.0).astype(int)
    big = np.bincount(lv)[lv] >= 152
    k0 = np.rint(y0 * n0)[(n0 <= 128) & big]
    # every prediction ~0: 12-row sketches
    w = np.zeros(capi.RANK_WEIGHTS, dtype=np.float32)
    w[-1] = -30.0
    for judge in (0.0, 4.0):
        t = _mixed(capi, geo, rank_judge=judge)
        t.set_rank_model(w)
        t.factor()
        mu1, _ = t.solve(F)
        st = t.stats()
        _, y1 = t.rank_samples()
        assert st["rank_predicted"] > 100
        if judge == 0.0:
            # without the residual judge a box needs 8 rows to spare: every box
            # of rank above 4 is redone
            assert st["rank_redo"] >= 0.9 * st["rank_predicted"]
            assert st["rank_redo_judge"] == 0
        else:
            # with it, a box whose 12 rows settled its rank (k <= 11) and whose
            # test rows confirm the residual is kept; every box of plain rank
            # 12 or more is redone (boxes lists may differ by a few per cent)
            assert st["rank_redo"] >= 0.98 * np.count_nonzero(k0 >= 12)
            assert st["rank_redo"] < st["rank_predicted"]
        assert st["sketch_rows"] > 0.5 * s0_rows
        # redone boxes get the plain factorization's ranks (boxes not redone may
        # pick other skeletons, which can change later levels' box lists)
        assert abs(len(y1) - len(y0)) <= 0.02 * len(y0)
        assert abs(float(np.mean(y1)) - float(np.mean(y0))) <= 0.02
        assert np.linalg.norm(mu1 - mu0) / np.linalg.norm(mu0) <= 1e-9
        t.close()
