"""CPU oracle of the low-rank algebra and the hierarchical Cholesky (test
infrastructure only: tests import it as the checker, the product never does).

A numpy restatement of HierarchicalMatrices.jl v0.2.2, step by step, with
numpy's LAPACK QR and SVD standing in for Julia's qr! and svd! (the same
LAPACK routines):

  getrank                    src/LowRankMatrix.jl:70-80
  svdtrunc                   src/LowRankMatrix.jl:82-86
  lr_add / lr_sub            src/LowRankMatrix.jl:95-111
  lr_mul / lr_adjmul         src/LowRankMatrix.jl:113-126
  dense_lr_mul / lr_dense_mul  src/LowRankMatrix.jl:128-142
  h_lr (H +/- L, L +/- H)    src/algebra.jl:394-524
  h_h (G +/- H)              src/hierarchical.jl:174-231
  cholesky                   src/cholesky.jl:12-92
  solvetransposed            src/cholesky.jl:97-228

Trees are ``HB(blocks)`` with ``blocks`` a list of lists of entries that are
``LR`` (U, s, V), 2-D ndarrays, nested ``HB`` or None (unassigned); sizes
follow src/hierarchical.jl:33-47 (rows from the last block column, columns
from the first block row).

No test file of the reference covers this code; the oracle is pinned by
dense known answers instead (tests/test_algebra_oracle.py): every operation
against the same operation on the dense matrices, and the Cholesky factor
against LAPACK's dense Cholesky (R'R = A, R = chol(A)).
"""
from collections import namedtuple

import numpy as np
import scipy.linalg

LR = namedtuple("LR", "U s V")


class HB:
    def __init__(self, blocks):
        self.blocks = blocks

    @property
    def M(self):
        return len(self.blocks)

    @property
    def N(self):
        return len(self.blocks[0])


def shape(b):
    if b is None:
        return (0, 0)
    if isinstance(b, LR):
        return (b.U.shape[0], b.V.shape[0])
    if isinstance(b, HB):
        return (sum(shape(b.blocks[m][b.N - 1])[0] for m in range(b.M)),
                sum(shape(b.blocks[0][n])[1] for n in range(b.N)))
    return b.shape


def getrank(s):
    """src/LowRankMatrix.jl:70-80."""
    r = len(s)
    if r == 0:
        return 0
    tol = r * np.spacing(abs(s[0]))
    while r >= 1:
        if s[r - 1] > tol:
            return r
        r -= 1
    return r


def _trunc(U, S, Vt):
    r = getrank(S)
    return LR(U[:, :r], S[:r], Vt.T[:, :r])


def svdtrunc(A):
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    return _trunc(U, S, Vt)


def _sum(L1, L2, sign):
    QU, RU = np.linalg.qr(np.hstack([L1.U, L2.U]))
    QV, RV = np.linalg.qr(np.hstack([L1.V, L2.V]))
    W, S, Zt = np.linalg.svd(RU @ np.diag(np.concatenate([L1.s, sign * L2.s])) @ RV.T, full_matrices=False)
    r = getrank(S)
    return LR((QU @ W)[:, :r], S[:r], (QV @ Zt.T)[:, :r])


def lr_add(L1, L2):
    return _sum(L1, L2, 1.0)


def lr_sub(L1, L2):
    return _sum(L1, L2, -1.0)


def lr_mul(L1, L2):
    W, S, Zt = np.linalg.svd(np.diag(L1.s) @ L1.V.T @ L2.U @ np.diag(L2.s), full_matrices=False)
    r = getrank(S)
    return LR((L1.U @ W)[:, :r], S[:r], (L2.V @ Zt.T)[:, :r])


def lr_adjmul(L1, L2):
    W, S, Zt = np.linalg.svd(np.diag(L1.s) @ L1.U.T @ L2.U @ np.diag(L2.s), full_matrices=False)
    r = getrank(S)
    return LR((L1.V @ W)[:, :r], S[:r], (L2.V @ Zt.T)[:, :r])


def dense_lr_mul(A, L):
    Q, R = np.linalg.qr(A @ L.U)
    W, S, Zt = np.linalg.svd(R @ np.diag(L.s), full_matrices=False)
    r = getrank(S)
    return LR((Q @ W)[:, :r], S[:r], (L.V @ Zt.T)[:, :r])


def lr_dense_mul(L, A):
    Q, R = np.linalg.qr(A.T @ L.V)
    W, S, Zt = np.linalg.svd(np.diag(L.s) @ R.T, full_matrices=False)
    r = getrank(S)
    return LR((L.U @ W)[:, :r], S[:r], (Q @ Zt.T)[:, :r])


def lr_dense(L):
    """L as a dense matrix, summing k = r:-1:1 as getindex does (src/LowRankMatrix.jl:50-58)."""
    out = np.zeros((L.U.shape[0], L.V.shape[0]), dtype=L.U.dtype)
    for k in range(len(L.s) - 1, -1, -1):
        out += np.outer(L.U[:, k] * L.s[k], L.V[:, k])
    return out


def todense(b):
    if b is None:
        raise ValueError("unassigned block")
    if isinstance(b, LR):
        return lr_dense(b)
    if isinstance(b, HB):
        m, n = shape(b)
        D = np.zeros((m, n))
        p = 0
        for i in range(b.M):
            q = 0
            for j in range(b.N):
                blk = b.blocks[i][j]
                if blk is not None:
                    bm, bn = shape(blk)
                    D[p:p + bm, q:q + bn] = todense(blk)
                q += shape(b.blocks[0][j])[1]
            p += shape(b.blocks[i][b.N - 1])[0]
        return D
    return np.array(b, dtype=np.float64)


def h_lr(H, L, sign_h, sign_l, lr_first):
    """sign_h H + sign_l L blockwise (src/algebra.jl:394-524); lr_first puts
    L[pr, qr] first (L +/- H)."""
    G = [[None] * H.N for _ in range(H.M)]
    p = 0
    for m in range(H.M):
        q = 0
        for n in range(H.N):
            b = H.blocks[m][n]
            if b is not None:
                bm, bn = shape(b)
                Ls = LR(L.U[p:p + bm], L.s, L.V[q:q + bn])
                if isinstance(b, HB):
                    G[m][n] = h_lr(b, Ls, sign_h, sign_l, lr_first)
                elif isinstance(b, LR):
                    if lr_first:
                        G[m][n] = _sum(Ls, b, sign_h)
                    else:
                        G[m][n] = _sum(b, Ls, sign_l)
                else:
                    G[m][n] = sign_h * b + sign_l * lr_dense(Ls)
            q += shape(H.blocks[0][n])[1]
        p += shape(H.blocks[m][H.N - 1])[0]
    return HB(G)


def h_h(G, H, sign):
    """G + H or G - H for equal block types (src/hierarchical.jl:174-231)."""
    F = [[None] * H.N for _ in range(H.M)]
    for m in range(H.M):
        for n in range(H.N):
            a, b = G.blocks[m][n], H.blocks[m][n]
            if a is None or b is None or type(a) is not type(b):
                continue
            if isinstance(b, HB):
                F[m][n] = h_h(a, b, sign)
            elif isinstance(b, LR):
                F[m][n] = _sum(a, b, sign)
            else:
                F[m][n] = a + sign * b
    return HB(F)


def cholesky(A):
    """src/cholesky.jl:12-92; a dense block is factored by LAPACK from its upper
    triangle (cholesky(Symmetric(A)).U)."""
    if not isinstance(A, HB):
        U = np.triu(A)
        return np.linalg.cholesky(U + np.triu(A, 1).T).T
    assert A.M == 2 and A.N == 2
    A11, A12, A22 = A.blocks[0][0], A.blocks[0][1], A.blocks[1][1]
    R11 = cholesky(A11)
    R12 = solvetransposed(R11, A12)
    if isinstance(R12, LR):
        S = lr_adjmul(R12, R12)
        A22m = h_lr(A22, S, 1.0, -1.0, False) if isinstance(A22, HB) else A22 - lr_dense(S)
    else:
        S = R12.T @ R12
        A22m = (todense(A22) if isinstance(A22, HB) else A22) - S
    R22 = cholesky(A22m)
    return HB([[R11, R12], [None, R22]])


def _solve_vec(R, b):
    if not isinstance(R, HB):
        return scipy.linalg.solve_triangular(R, b, trans="T", lower=False)
    n = shape(R)[1]
    s = shape(R.blocks[0][0])[1]
    x1 = _solve_vec(R.blocks[0][0], b[:s])
    R12 = R.blocks[0][1]
    t = R12.V @ (R12.s * (R12.U.T @ x1)) if isinstance(R12, LR) else R12.T @ x1
    x2 = _solve_vec(R.blocks[1][1], b[s:n] - t)
    return np.concatenate([x1, x2])


def solvetransposed(R, B):
    """src/cholesky.jl:97-228, column by column as the reference does."""
    if isinstance(B, LR):
        Uh = np.zeros_like(B.U)
        for j in range(B.U.shape[1]):
            Uh[:, j] = _solve_vec(R, B.U[:, j])
        return LR(Uh, B.s, B.V)
    B = np.asarray(B, dtype=np.float64)
    if B.ndim == 1:
        return _solve_vec(R, B)
    out = np.zeros_like(B)
    for j in range(B.shape[1]):
        out[:, j] = _solve_vec(R, B[:, j])
    return out


# ------------------------------------------------------------------ test matrices

def spd_hodlr(n, leaf, kernel="gauss", shift=1e-2, rank_tol=1e-15, dense_below=0, seed=0):
    """A symmetric positive definite matrix K + shift I on sorted points of
    [0, 1] as a 2 x 2 recursive tree: dense diagonal leaves of at most ``leaf``
    rows, upper off-diagonal blocks as truncated SVDs (singular values above
    rank_tol * the largest) or dense for blocks of at most ``dense_below``
    rows, the lower block unassigned as src/cholesky.jl reads only the upper
    blocks.  Returns (tree, dense symmetric matrix of the tree)."""
    rng = np.random.default_rng(seed)
    x = np.sort(rng.uniform(0.0, 1.0, n))
    d = x[:, None] - x[None, :]
    if kernel == "gauss":
        K = np.exp(-d * d / (2 * 0.15 ** 2))
    elif kernel == "exp":
        K = np.exp(-np.abs(d))
    else:
        raise ValueError(kernel)
    K = K + shift * np.eye(n)

    def build(i0, i1):
        if i1 - i0 <= leaf:
            return K[i0:i1, i0:i1].copy()
        mid = (i0 + i1) // 2
        B = K[i0:mid, mid:i1]
        if i1 - i0 <= dense_below:
            A12 = B.copy()
        else:
            U, S, Vt = np.linalg.svd(B, full_matrices=False)
            r = int(np.sum(S > rank_tol * S[0]))
            A12 = LR(U[:, :r].copy(), S[:r].copy(), Vt[:r].T.copy())
        return HB([[build(i0, mid), A12], [None, build(mid, i1)]])

    T = build(0, n)
    D = todense(T)
    D = np.triu(D) + np.triu(D, 1).T
    return T, D
