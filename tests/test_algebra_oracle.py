"""The CPU oracle of the low-rank algebra and the hierarchical Cholesky
(oracle/algebra.py) pinned by dense known answers: no test file of the
reference covers this code, so every operation is checked against the same
operation on dense matrices, and the Cholesky factor against LAPACK's dense
Cholesky of the assembled matrix."""
import numpy as np
import pytest

from oracle import algebra as A


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def rand_lr(rng, m, n, r, decay=0.5):
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    return A.LR(U, decay ** np.arange(r), V)


def test_getrank_known_answers():
    assert A.getrank(np.array([3.0, 2.0, 1.0])) == 3
    assert A.getrank(np.array([1.0, 1e-17])) == 1          # tol = 2 eps(1)
    assert A.getrank(np.array([1.0, 5e-16])) == 2          # 5e-16 > 4.44e-16
    assert A.getrank(np.array([])) == 0
    assert A.getrank(np.array([0.0, 0.0])) == 0


def test_lowrank_operations_match_dense():
    rng = np.random.default_rng(1)
    L1, L2 = rand_lr(rng, 70, 50, 6), rand_lr(rng, 70, 50, 9)
    D1, D2 = A.lr_dense(L1), A.lr_dense(L2)
    assert rel(A.lr_dense(A.lr_add(L1, L2)), D1 + D2) < 1e-13
    assert rel(A.lr_dense(A.lr_sub(L1, L2)), D1 - D2) < 1e-13
    assert A.lr_add(L1, L1).s.size == 6                      # rank of 2 L1
    Z = A.lr_sub(L1, L1)
    assert np.linalg.norm(A.lr_dense(Z)) < 1e-14 * np.linalg.norm(D1)
    L3 = rand_lr(rng, 50, 40, 5)
    assert rel(A.lr_dense(A.lr_mul(L1, L3)), D1 @ A.lr_dense(L3)) < 1e-13
    L4 = rand_lr(rng, 70, 30, 4)
    assert rel(A.lr_dense(A.lr_adjmul(L1, L4)), D1.T @ A.lr_dense(L4)) < 1e-13
    M = rng.standard_normal((20, 70))
    assert rel(A.lr_dense(A.dense_lr_mul(M, L1)), M @ D1) < 1e-13
    N = rng.standard_normal((50, 15))
    assert rel(A.lr_dense(A.lr_dense_mul(L1, N)), D1 @ N) < 1e-13
    S = A.svdtrunc(D1 + D2)
    assert S.s.size == 15 and rel(A.lr_dense(S), D1 + D2) < 1e-13


@pytest.mark.parametrize("dense_below", [0, 128])
def test_tree_sums_match_dense(dense_below):
    T, D = A.spd_hodlr(256, 32, dense_below=dense_below, seed=2)
    rng = np.random.default_rng(3)
    L = rand_lr(rng, 256, 256, 5)
    DT = A.todense(T)
    for sh, sl, first in ((1.0, 1.0, False), (1.0, -1.0, False), (1.0, 1.0, True), (-1.0, 1.0, True)):
        G = A.h_lr(T, L, sh, sl, first)
        # unassigned blocks stay unassigned: compare on the assigned (upper) part
        mask = A.todense(A.h_h(T, T, 1.0)) != 0
        assert rel(A.todense(G)[mask], (sh * DT + sl * A.lr_dense(L))[mask]) < 1e-13
    assert rel(A.todense(A.h_h(T, T, 1.0)), 2 * DT) < 1e-14
    assert np.linalg.norm(A.todense(A.h_h(T, T, -1.0))) < 1e-13 * np.linalg.norm(DT)


@pytest.mark.parametrize("kernel,dense_below", [("gauss", 0), ("gauss", 128), ("exp", 0)])
def test_cholesky_matches_dense_lapack(kernel, dense_below):
    T, D = A.spd_hodlr(512, 32, kernel=kernel, dense_below=dense_below, seed=4)
    R = A.cholesky(T)
    Rd = A.todense(R)
    assert np.allclose(np.tril(Rd, -1), 0)
    assert rel(Rd.T @ Rd, D) < 1e-12
    assert rel(Rd, np.linalg.cholesky(D).T) < 1e-9
    b = np.random.default_rng(5).standard_normal(512)
    x = A.solvetransposed(R, b)
    assert rel(Rd.T @ x, b) < 1e-10


def test_exponential_kernel_keeps_rank_one():
    # exp(-|x - y|) has rank-1 off-diagonal blocks, and so do its Cholesky factor's
    T, _ = A.spd_hodlr(256, 32, kernel="exp", rank_tol=1e-13, seed=6)
    R = A.cholesky(T)

    def ranks(b):
        if isinstance(b, A.HB):
            return ranks(b.blocks[0][0]) + [len(b.blocks[0][1].s)] + ranks(b.blocks[1][1])
        return []
    assert max(ranks(T)) == 1
    assert max(ranks(R)) <= 2


def test_cholesky_rejects_indefinite():
    T, D = A.spd_hodlr(128, 32, seed=7)
    T.blocks[1][1].blocks[1][1][0, 0] = -1.0
    with pytest.raises(np.linalg.LinAlgError):
        A.cholesky(T)


def test_package_getrank_matches_oracle():
    import hierarchicalmatrices as hm
    rng = np.random.default_rng(8)
    for s in (np.array([3.0, 2.0, 1.0]), np.array([1.0, 1e-17]), np.array([1.0, 5e-16]), np.array([]),
              np.array([0.0, 0.0]), np.sort(rng.uniform(0, 1, 40))[::-1] * 10.0 ** -np.arange(40)):
        assert hm.getrank(s) == A.getrank(s)
    s32 = np.array([1.0, 5e-7, 1e-8], dtype=np.float32)          # eps(1f0) = 1.19e-7: tol = 3.6e-7
    assert hm.getrank(s32) == 2
