"""rs_id_noalloc, the ID entry point that allocates no device memory (its
scratch tile is a fixed file-scope device array), against rs_id_batched on
the same matrices.

This file is collected last so that its GPU test also runs after every other
GPU test of the session (the static scratch then holds whatever the earlier
calls left in it).  The largest documented sizes run first (m = 2048 with
n = 222 and m = 1024 with n = 478 fill the 524288-double array to within
2 %), so every later, smaller call starts on a scratch array holding a
full-size tile's values, which it must overwrite before reading.

Tolerances: equal rank and pivot order on matrices with a clear
singular-value gap; |Z - Z_batched| <= 1e-9 max(1, |Z|) (the two paths order
the same FP64 operations differently); ID reconstruction error within
100 tol |A|, as for rs_id_batched against the reference's ID matrices.  On
those matrices the rank may differ by one: rs_id_batched folds the rows
into an n x n triangle by Householder reflections before the pivoted QR,
while this entry point runs the pivoted QR on the whole m x n tile, so the
two compute |R_ii| with different roundings, and the reference's matrices
have singular values that decay smoothly through the threshold tol |R_00|.
"""
import os

import numpy as np
import pytest

RS_ERR_ARG, RS_ERR_CAPACITY = 1, 5


def _gapped(rng, m, n, k):
    U = np.linalg.qr(rng.standard_normal((m, k)))[0]
    V = np.linalg.qr(rng.standard_normal((n, k)))[0]
    return (U * np.logspace(0, -4, k)) @ V.T + 1e-14 * rng.standard_normal((m, n))


def _noalloc(capi, torch, A, tol):
    m, n = A.shape
    dA = torch.from_numpy(np.ascontiguousarray(A.ravel(order="F"))).cuda()
    rank = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    Z = torch.full((n * n // 4 + 1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = capi.lib().rs_id_noalloc(m, n, dA.data_ptr(), tol, rank.data_ptr(), perm.data_ptr(),
                                  Z.data_ptr(), stream)
    assert rc == 0, rc
    torch.cuda.current_stream().synchronize()
    k = int(rank.item())
    z = Z[: k * (n - k)].cpu().numpy().reshape((k, n - k), order="F") if k else None
    return k, perm.cpu().numpy(), z


def test_noalloc_rejects_bad_sizes(solver_lib):
    from rskel import capi

    L = capi.lib()
    # argument and capacity checks come before any device call
    assert L.rs_id_noalloc(0, 10, 1, 1e-8, 1, 1, 1, None) == RS_ERR_ARG
    assert L.rs_id_noalloc(10, 10, None, 1e-8, 1, 1, 1, None) == RS_ERR_ARG
    assert L.rs_id_noalloc(10, 10, 1, 0.0, 1, 1, 1, None) == RS_ERR_ARG
    assert L.rs_id_noalloc(2048, 223, 1, 1e-8, 1, 1, 1, None) == RS_ERR_CAPACITY
    assert L.rs_id_noalloc(1024, 479, 1, 1e-8, 1, 1, 1, None) == RS_ERR_CAPACITY
    assert L.rs_id_noalloc(100000, 8, 1, 1e-8, 1, 1, 1, None) == RS_ERR_CAPACITY


@pytest.mark.gpu
def test_noalloc_matches_batched_two_calls_in_a_row(solver_lib):
    torch = pytest.importorskip("torch")
    from rskel import capi
    from rskel import geometry as g

    s = capi.Solver(g.unit_circle(64), capi.RS_LAPLACE, 1e-8)
    rng = np.random.default_rng(11)
    tol = 1e-8
    # the two largest documented sizes, then two calls in a row, the second
    # smaller than the first, then the first again
    full = [_gapped(rng, 2048, 222, 60), _gapped(rng, 1024, 478, 60)]
    cases = [_gapped(rng, 640, 200, 40), _gapped(rng, 150, 48, 12)]
    first = None
    for A in full + cases + [cases[0]]:
        k, perm, Z = _noalloc(capi, torch, A, tol)
        (kb, pb, zb), = capi.id_batched(s, [A], tol)
        assert k == kb and np.array_equal(perm, pb), (k, kb)
        assert np.abs(Z - zb).max() <= 1e-9 * max(1.0, np.abs(zb).max())
        err = np.linalg.norm(A[:, perm[k:]] - A[:, perm[:k]] @ Z, 2)
        assert err <= 100 * tol * np.linalg.norm(A, 2)
        if A is cases[0]:
            if first is None:
                first = (k, perm, Z)
            else:  # the repeated call gives the same result bit for bit
                assert first[0] == k and np.array_equal(first[1], perm)
                assert np.array_equal(first[2], Z)
    # the reference's own ID matrices (rank within one of rs_id_batched's)
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "id_cases.npz"))
    for i in range(len(d["ranks"])):
        A, tl = d[f"A{i}"], float(d["tols"][i])
        k, perm, Z = _noalloc(capi, torch, A, tl)
        (kb, pb, zb), = capi.id_batched(s, [A], tl)
        assert abs(k - kb) <= 1 and sorted(perm.tolist()) == list(range(A.shape[1]))
        if k:
            err = np.linalg.norm(A[:, perm[k:]] - A[:, perm[:k]] @ Z, 2)
            assert err <= 100 * tl * np.linalg.norm(A, 2)
