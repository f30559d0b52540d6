"""Pins the CPU oracle: the reference's own tests (test/runtests.jl), its
example check against dense products (examples/Kernel.jl:73-78), the tree
counts of the interleaved grid, and the committed golden fixtures."""
import glob
import os
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_blockrank_even():
    # test/runtests.jl:5-7: BLOCKRANK(T) is even for every float type
    for T in (np.float16, np.float32, np.float64):
        assert O.blockrank(np.finfo(T).eps) % 2 == 0
    assert O.blockrank(np.finfo(np.float64).eps) == 20
    assert O.blockrank(np.finfo(np.float32).eps) == 10


def test_chebyshev_nodes_and_weights():
    # src/BarycentricMatrix.jl:92-136 against the closed forms
    for n in (2, 5, 10, 20):
        k = np.arange(1, n + 1)
        x = O.chebyshevpoints(n, 1)
        np.testing.assert_allclose(x, np.cos((2 * k - 1) * np.pi / (2 * n)), atol=2e-16)
        w = O.chebyshevbarycentricweights(n, 1)
        np.testing.assert_allclose(np.abs(w), np.sin((2 * k - 1) * np.pi / (2 * n)), atol=2e-16)
        assert np.all(np.sign(w[1::2]) < 0) and np.all(np.sign(w[0::2]) > 0)
        x2 = O.chebyshevpoints(n, 2)
        np.testing.assert_allclose(x2, np.cos((k - 1) * np.pi / (n - 1)) if n > 1 else x2, atol=2e-16)


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_dense_block_known_answers(T):
    # test/runtests.jl:15-33, same cases, FP64 oracle on the values of T
    rng = np.random.default_rng(0)
    A = rng.random((10, 5)).astype(T).astype(np.float64)
    x = rng.random(40).astype(T).astype(np.float64)
    eps = np.finfo(T).eps

    y = np.zeros(40)
    O.dense_mul(y, A, x, 1, 1)
    assert np.linalg.norm(y[0:10] - A @ x[0:5]) <= eps * np.linalg.norm(A @ x[0:5])
    y[:] = 0
    O.dense_mul(y, A, x, 5, 5, 2, 2)
    assert np.linalg.norm(y[4:23:2] - A @ x[4:14:2]) <= eps * np.linalg.norm(A @ x[4:14:2])
    y[:] = 0
    O.dense_mul(y, A, x, 1, 5, 2, 1, trans=True)
    assert np.linalg.norm(y[0:5] - A.T @ x[4:23:2]) <= eps * np.linalg.norm(A.T @ x[4:23:2])
    y[:] = 0
    O.dense_mul(y, A, x, 6, 3, 1, 3, trans=True)
    assert np.linalg.norm(y[5:18:3] - A.T @ x[2:12]) <= eps * np.linalg.norm(A.T @ x[2:12])


def test_dense_block_exact_rational():
    # test/runtests.jl:35-52 use BigFloat and require exact equality; the
    # generic restatement on Fractions must equal the exact product.
    rng = np.random.default_rng(0)
    A = [[Fraction(float(v)) for v in row] for row in rng.random((10, 5))]
    x = [Fraction(float(v)) for v in rng.random(40)]

    def Ax(rows, cols):
        return [sum(A[i][j] * x[c] for j, c in enumerate(cols)) for i in rows]

    def ATx(cols):
        return [sum(A[j][i] * x[c] for j, c in enumerate(cols)) for i in range(5)]

    y = [Fraction(0)] * 40
    O.dense_mul_generic(y, A, x, 1, 1)
    assert y[0:10] == Ax(range(10), range(0, 5))
    y = [Fraction(0)] * 40
    O.dense_mul_generic(y, A, x, 5, 5, 2, 2)
    assert y[4:23:2] == Ax(range(10), range(4, 14, 2))
    y = [Fraction(0)] * 40
    O.dense_mul_t_generic(y, A, x, 1, 5, 2, 1)
    assert y[0:5] == ATx(range(4, 23, 2))
    y = [Fraction(0)] * 40
    O.dense_mul_t_generic(y, A, x, 6, 3, 1, 3)
    assert y[5:18:3] == ATx(range(2, 12))


def test_lowrank_block_matches_numpy():
    rng = np.random.default_rng(3)
    U, V = rng.standard_normal((7, 3)), rng.standard_normal((9, 3))
    s = rng.random(3)
    x = rng.standard_normal(30)
    y = np.zeros(30)
    O.lowrank_mul(y, U, s, V, x, 2, 4, 2, 3)
    L = U @ np.diag(s) @ V.T
    np.testing.assert_allclose(y[1:1 + 3 * 7:3], L @ x[3:3 + 2 * 9:2], rtol=1e-13, atol=1e-13)
    y[:] = 0
    O.lowrank_mul(y, U, s, V, x, 1, 1, adjoint=True)
    np.testing.assert_allclose(y[0:9], L.T @ x[0:7], rtol=1e-13, atol=1e-13)


def test_indsplit_semantics():
    x = np.array([0.9, 0.75, 0.5, 0.5, 0.25, 0.1])
    # points >= midpoint (ties included) go to the first half
    assert O.indsplit(x, 0, 6, 1.0, 0.0) == ((0, 4), (4, 2))
    assert O.indsplit(x, 2, 4, 0.5, 0.0) == ((2, 3), (5, 1))
    # an empty range still reads its first element: below the midpoint both
    # halves stay empty; at or above it the reference's scan makes the first
    # half a one-element range (UnitRange first:first)
    assert O.indsplit(x, 4, 0, 1.0, 0.0) == ((4, 0), (4, 0))
    assert O.indsplit(x, 3, 0, 0.5, 0.0) == ((3, 1), (4, 0))
    with pytest.raises(IndexError):
        O.indsplit(x, 6, 0, 1.0, 0.0)


def test_grid_tree_counts():
    x, y = O.grid_points(2048)
    H = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    st = H.stats()
    assert (st["bary"], st["dense"], st["depth"]) == (156, 94, 4)
    meta, _ = H.leaves()
    assert np.all(meta[meta[:, 0] == O.TAG_DENSE][:, 2] == 64)


@pytest.mark.parametrize("kernel", [O.CAUCHY, O.COULOMB, O.COULOMB_PRIME, O.LOG])
@pytest.mark.parametrize("family", ["chebyshev", "quadratic"])
def test_oracle_matches_dense(kernel, family):
    # examples/Kernel.jl:58-110 prints ||K b - KF b|| / ||K b||; the oracle
    # must reproduce the dense product to near machine precision.
    x, y, box = O.example_points(family, 1000)
    b = np.random.default_rng(2).standard_normal(1000)
    u = O.OracleKernelMatrix(kernel, x, y, *box) @ b
    ud = O.kernel_dense(kernel, x, y) @ b
    assert np.linalg.norm(u - ud) / np.linalg.norm(ud) < 1e-13


def test_oracle_parallel_is_bitwise_serial():
    x, y = O.grid_points(4096)
    H = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0, nthreads=4)
    b = np.random.default_rng(5).standard_normal(4096)
    u1 = np.zeros(4096)
    u4 = np.zeros(4096)
    H.mul(u1, b, nthreads=1)
    H.mul(u4, b, nthreads=4)
    assert np.array_equal(u1, u4)


def test_dense_rows_compensated():
    x, y = O.grid_points(2048)
    b = np.random.default_rng(4).standard_normal(2048)
    rows = np.arange(0, 2048, 17)
    got = O.dense_rows(O.CAUCHY, x, y, b, rows)
    ref = O.kernel_dense(O.CAUCHY, x[rows], y) @ b
    np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-9)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_golden(path):
    d = np.load(path)
    name = os.path.basename(path)
    kernel = {"cauchy": O.CAUCHY, "coulomb": O.COULOMB, "coulombprime": O.COULOMB_PRIME,
              "log": O.LOG}[name[:-4].split("_")[1]]
    H = O.OracleKernelMatrix(kernel, d["x"], d["y"], *d["box"])
    st = H.stats()
    assert [st["bary"], st["dense"], st["depth"], st["stored_values"]] == d["stats"].tolist()
    u = H @ d["b"]
    np.testing.assert_allclose(u, d["u"], rtol=1e-14, atol=1e-14 * np.abs(d["u"]).max())
    assert np.linalg.norm(u - d["u_dense"]) / np.linalg.norm(d["u_dense"]) < 1e-13


def test_hier_walk_matches_dense():
    # src/HierarchicalMatrix.jl:24-52: generic block walk with strides
    rng = np.random.default_rng(9)
    H = O.PyHier(2, 2)
    H.blocks[0][0] = rng.standard_normal((3, 4))
    H.blocks[0][1] = O.PyLowRank(rng.standard_normal((3, 2)), rng.random(2), rng.standard_normal((5, 2)))
    inner = O.PyHier(2, 2)
    inner.blocks[0][0] = rng.standard_normal((2, 2))
    inner.blocks[0][1] = rng.standard_normal((2, 2))
    inner.blocks[1][0] = rng.standard_normal((2, 2))
    inner.blocks[1][1] = O.PyLowRank(rng.standard_normal((2, 1)), rng.random(1), rng.standard_normal((2, 1)))
    H.blocks[1][0] = inner
    H.blocks[1][1] = rng.standard_normal((4, 5))
    assert H.shape == (7, 9)

    def dense(b):
        if isinstance(b, O.PyHier):
            return np.block([[dense(c) for c in row] for row in b.blocks])
        if isinstance(b, O.PyLowRank):
            return b.U @ np.diag(b.sigma) @ b.V.T
        return b
    D = dense(H)
    x = rng.standard_normal(40)
    y = np.zeros(40)
    O.hier_mul(y, H, x, 3, 2, 2, 3)
    np.testing.assert_allclose(y[2:2 + 3 * 7:3], D @ x[1:1 + 2 * 9:2], rtol=1e-12, atol=1e-12)
