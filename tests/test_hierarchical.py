"""The @hierarchical type generator and user-assembled HierarchicalMatrix on
the host side (no GPU): block tags, sizes, element access and the block-walk
offsets, against the oracle's restatement (src/hierarchical.jl,
src/HierarchicalMatrix.jl) and dense products."""
import numpy as np
import pytest

import hierarchicalmatrices as hm
from oracle import oracle as O


def random_tree(rng):
    H = hm.HierarchicalMatrix(2, 2)
    P = O.PyHier(2, 2)
    A = rng.standard_normal((3, 4))
    H[hm.Block(1), hm.Block(1)] = A
    P.blocks[0][0] = A
    U, s, V = rng.standard_normal((3, 2)), rng.random(2), rng.standard_normal((5, 2))
    H[hm.Block(1), hm.Block(2)] = hm.LowRankMatrix(U, s, V)
    P.blocks[0][1] = O.PyLowRank(U, s, V)
    inner = hm.HierarchicalMatrix(2, 2)
    pin = O.PyHier(2, 2)
    for (i, j) in ((0, 0), (0, 1), (1, 0)):
        B = rng.standard_normal((2, 2))
        inner[hm.Block(i + 1), hm.Block(j + 1)] = B
        pin.blocks[i][j] = B
    U2, s2, V2 = rng.standard_normal((2, 1)), rng.random(1), rng.standard_normal((2, 1))
    inner[hm.Block(2), hm.Block(2)] = hm.LowRankMatrix(U2, s2, V2)
    pin.blocks[1][1] = O.PyLowRank(U2, s2, V2)
    H[hm.Block(2), hm.Block(1)] = inner
    P.blocks[1][0] = pin
    D = rng.standard_normal((4, 5))
    H[hm.Block(2), hm.Block(2)] = D
    P.blocks[1][1] = D
    return H, P


def dense_of(P):
    if isinstance(P, O.PyHier):
        return np.block([[dense_of(c) for c in row] for row in P.blocks])
    if isinstance(P, O.PyLowRank):
        return P.U @ np.diag(P.sigma) @ P.V.T
    return P


def test_tags_sizes_and_elements():
    H, P = random_tree(np.random.default_rng(0))
    assert H.assigned.tolist() == [[3, 2], [1, 3]]        # 1 self, 2 LowRankMatrix, 3 Matrix
    assert H.blocksize() == (2, 2)
    assert H.shape == P.shape == (7, 9)
    assert H.blocksize(1, 2, 2) == 5 and H.blocksize(2, 1, 1) == 4
    D = dense_of(P)
    for i in range(1, 8):
        for j in range(1, 10):
            assert H[i, j] == pytest.approx(D[i - 1, j - 1], abs=1e-14)


def test_leaf_offsets_follow_block_walk():
    H, _ = random_tree(np.random.default_rng(1))
    offs = [(p, q) for _, p, q in H.leaves()]
    assert offs == [(0, 0), (0, 4), (3, 0), (3, 2), (5, 0), (5, 2), (3, 4)]


def test_parametric_member_store():
    # test/runtests.jl:13 and :54-56: a parametric member type gets a store
    # named after its outer type holding (outer, inner) pairs
    T = hm.hierarchical("UpperTriangularHierarchicalMatrix", "Matrix", ("UpperTriangular", "LowRankMatrix"),
                        "Diagonal")
    H = T(2, 2)
    assert hasattr(H, "UpperTriangularblocks") and hasattr(H, "Matrixblocks") and hasattr(H, "Diagonalblocks")
    assert T.block_types[1] == ("UpperTriangular", "LowRankMatrix")
    L = hm.LowRankMatrix(np.eye(2), np.ones(2), np.eye(2))
    H[hm.Block(1), hm.Block(2)] = ("UpperTriangular", L)
    assert H.assigned[0, 1] == 3


def test_unassigned_and_foreign_blocks():
    H = hm.HierarchicalMatrix(2, 2)
    H[hm.Block(1), hm.Block(1)] = "not a block"              # ignored, as the generated setindex! does
    assert H.assigned[0, 0] == 0 and H.blocksize(1, 1, 1) == 0


def test_cached_shape_follows_block_assignments():
    """size(H) is cached between block assignments (it is read many times by
    the algebra's walks); assigning a block anywhere, also inside a child,
    makes the parent report the new size (src/hierarchical.jl:33-47)."""
    rng = np.random.default_rng(3)
    inner = hm.HierarchicalMatrix(2, 2)
    for i, j in ((1, 1), (1, 2), (2, 1), (2, 2)):
        inner[hm.Block(i), hm.Block(j)] = rng.standard_normal((2, 3))
    H = hm.HierarchicalMatrix(2, 2)
    H[hm.Block(1), hm.Block(1)] = inner
    H[hm.Block(1), hm.Block(2)] = rng.standard_normal((4, 5))
    H[hm.Block(2), hm.Block(1)] = rng.standard_normal((1, 6))
    H[hm.Block(2), hm.Block(2)] = rng.standard_normal((1, 5))
    assert H.shape == (5, 11)
    assert H.shape == (5, 11)                       # served from the cache
    inner[hm.Block(2), hm.Block(1)] = rng.standard_normal((7, 3))     # a child's block changes
    H[hm.Block(1), hm.Block(2)] = rng.standard_normal((9, 5))         # rows come from block column 2
    assert inner.shape == (4, 6)
    assert H.shape == (10, 11)
    inner[hm.Block(1), hm.Block(1)] = rng.standard_normal((2, 10))    # widens block row 1 of the child
    assert H.shape == (10, 18)                      # the parent sees the child's change
