"""Low-rank algebra, H +/- L, H +/- H, hierarchicalcholesky and solvetransposed
on the GPU (hm_lr_svd, hm_gemm_batched, hm_axpby_batched, hm_potrf_batched,
hm_solve_transposed) against the CPU oracle (oracle/algebra.py, pinned by
dense known answers).

Truncated SVDs are unique only up to the singular vectors' signs, so results
are compared as the matrices they represent (relative Frobenius error), with
ranks compared where the spectrum is far from the getrank threshold.
Tolerances: 1e-12 in FP64 and 2e-5 in FP32 for the block operations; the
Cholesky factor's own bounds (CHOL) separate forward from backward error."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import algebra as G  # noqa: E402
from oracle import algebra as A  # noqa: E402

TOL = {torch.float64: 1e-12, torch.float32: 2e-5}
DT = [torch.float64, torch.float32]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def dev(a, dt):
    return torch.tensor(np.ascontiguousarray(np.asarray(a).T), dtype=dt, device="cuda").t() if np.ndim(a) == 2 \
        else torch.tensor(np.asarray(a), dtype=dt, device="cuda")


def host(t):
    return t.detach().double().cpu().numpy()


def lr_dev(L, dt):
    return hm.LowRankMatrix(dev(L.U, dt), dev(L.s, dt), dev(L.V, dt))


def lr_host(L):
    return A.LR(host(L.U), host(L.sigma), host(L.V))


def tree_dev(T, dt):
    if isinstance(T, A.LR):
        return lr_dev(T, dt)
    if not isinstance(T, A.HB):
        return dev(T, dt)
    H = hm.HierarchicalMatrix(T.M, T.N, dtype=np.float64 if dt == torch.float64 else np.float32)
    for m in range(T.M):
        for n in range(T.N):
            if T.blocks[m][n] is not None:
                H[hm.Block(m + 1), hm.Block(n + 1)] = tree_dev(T.blocks[m][n], dt)
    return H


def tree_host(H):
    if isinstance(H, hm.LowRankMatrix):
        return lr_host(H)
    if isinstance(H, torch.Tensor):
        return host(H)
    M, N = H.blocksize()
    return A.HB([[None if H.block(m, n) is None else tree_host(H.block(m, n)) for n in range(N)] for m in range(M)])


def rand_lr(rng, m, n, r, decay=0.5):
    U, _ = np.linalg.qr(rng.standard_normal((m, r)))
    V, _ = np.linalg.qr(rng.standard_normal((n, r)))
    return A.LR(U, decay ** np.arange(r), V)


def check_svd_form(L, dt):
    """Descending non-negative singular values and orthonormal factors (to
    about q eps: rotations accumulate rounding in proportion to the width)."""
    s = host(L.sigma)
    assert np.all(np.diff(s) <= 0) and np.all(s >= 0)
    tol = 1e-12 if dt == torch.float64 else 4 * max(len(s), 20) * 1.19e-7
    for F in (host(L.U), host(L.V)):
        assert np.abs(F.T @ F - np.eye(F.shape[1])).max() < tol


@pytest.mark.parametrize("dt", DT)
def test_lowrank_operations(dt):
    rng = np.random.default_rng(11)
    L1, L2 = rand_lr(rng, 300, 200, 6), rand_lr(rng, 300, 200, 9)
    g1, g2 = lr_dev(L1, dt), lr_dev(L2, dt)
    cases = [
        (G.lr_add(g1, g2), A.lr_add(L1, L2)),
        (G.lr_sub(g1, g2), A.lr_sub(L1, L2)),
        (G.lr_add(g1, g1), A.lr_add(L1, L1)),
    ]
    L3 = rand_lr(rng, 200, 150, 5)
    cases.append((G.lr_mul(g1, lr_dev(L3, dt)), A.lr_mul(L1, L3)))
    L4 = rand_lr(rng, 300, 120, 4)
    cases.append((G.times(hm.adjoint(g1), lr_dev(L4, dt)), A.lr_adjmul(L1, L4)))
    M = rng.standard_normal((90, 300))
    cases.append((G.times(dev(M, dt), g1), A.dense_lr_mul(M, L1)))
    N = rng.standard_normal((200, 70))
    cases.append((G.times(g1, dev(N, dt)), A.lr_dense_mul(L1, N)))
    d1, d2 = rng.uniform(0.5, 2.0, 300), rng.uniform(0.5, 2.0, 200)
    cases.append((G.times(G.Diagonal(dev(d1, dt)), g1), A.dense_lr_mul(np.diag(d1), L1)))
    cases.append((G.times(g1, G.Diagonal(dev(d2, dt))), A.lr_dense_mul(L1, np.diag(d2))))
    for got, ref in cases:
        check_svd_form(got, dt)
        assert got.rank() == len(ref.s)
        assert rel(A.lr_dense(lr_host(got)), A.lr_dense(ref)) <= TOL[dt]
    # a 120 x 120 core: global-memory Jacobi in FP64 (shared memory in FP32)
    L5, L6 = rand_lr(rng, 400, 300, 60, 0.9), rand_lr(rng, 400, 300, 60, 0.9)
    got, ref = G.lr_add(lr_dev(L5, dt), lr_dev(L6, dt)), A.lr_add(L5, L6)
    check_svd_form(got, dt)
    assert got.rank() == len(ref.s) == 120
    assert rel(A.lr_dense(lr_host(got)), A.lr_dense(ref)) <= TOL[dt]
    Z = G.lr_sub(g1, g1)                        # rank-deficient: ranks may differ, the matrix is ~0
    assert np.linalg.norm(A.lr_dense(lr_host(Z))) <= TOL[dt] * np.linalg.norm(A.lr_dense(L1))
    S = G.times(2.5, g1)
    assert rel(host(S.sigma), 2.5 * L1.s) <= TOL[dt]


@pytest.mark.parametrize("dt", DT)
@pytest.mark.parametrize("m,n", [(400, 40), (40, 400), (96, 96), (7, 3)])
def test_svdtrunc(dt, m, n):
    rng = np.random.default_rng(m + n)
    k = min(m, n, 12)
    B = rng.standard_normal((m, k)) @ np.diag(0.7 ** np.arange(k)) @ rng.standard_normal((k, n))
    got, ref = G.svdtrunc(dev(B, dt)), A.svdtrunc(B)
    check_svd_form(got, dt)
    if dt == torch.float64:
        assert got.rank() == len(ref.s) == k
    assert rel(A.lr_dense(lr_host(got)), B) <= TOL[dt] * 10


@pytest.mark.parametrize("dt", DT)
@pytest.mark.parametrize("dense_below", [0, 128])
def test_tree_sums(dt, dense_below):
    T, _ = A.spd_hodlr(512, 32, dense_below=dense_below, seed=12)
    rng = np.random.default_rng(13)
    L = rand_lr(rng, 512, 512, 5)
    H, g = tree_dev(T, dt), lr_dev(L, dt)
    for got, ref in ((G.add(H, g), A.h_lr(T, L, 1.0, 1.0, False)),
                     (G.sub(H, g), A.h_lr(T, L, 1.0, -1.0, False)),
                     (G.add(g, H), A.h_lr(T, L, 1.0, 1.0, True)),
                     (G.sub(g, H), A.h_lr(T, L, -1.0, 1.0, True))):
        assert (got.assigned == H.assigned).all()
        assert rel(A.todense(tree_host(got)), A.todense(ref)) <= TOL[dt]
    assert rel(A.todense(tree_host(G.add(H, H))), A.todense(A.h_h(T, T, 1.0))) <= TOL[dt]
    D = A.todense(T)
    assert np.linalg.norm(A.todense(tree_host(G.sub(H, H)))) <= TOL[dt] * np.linalg.norm(D)
    assert rel(host(G.todense(H)), D) <= TOL[dt]


# Cholesky tolerances: the factor's forward error grows with the condition
# number (about 4e4 here), the backward errors (R'R - A, R'x - b) do not.
CHOL = {torch.float64: dict(fwd=1e-10, bwd=1e-12, solve=1e-9),
        torch.float32: dict(fwd=1e-2, bwd=1e-4, solve=5e-3)}


@pytest.mark.parametrize("dt", DT)
@pytest.mark.parametrize("kernel,dense_below", [("gauss", 0), ("gauss", 128), ("exp", 0)])
def test_hierarchical_cholesky(dt, kernel, dense_below):
    T, D = A.spd_hodlr(1024, 64, kernel=kernel, dense_below=dense_below, seed=14)
    R = G.hierarchicalcholesky(tree_dev(T, dt))
    Rd = A.todense(tree_host(R))
    Ro = A.todense(A.cholesky(T))
    tol = CHOL[dt]
    assert np.allclose(np.tril(Rd, -1), 0)
    assert rel(Rd, Ro) <= tol["fwd"]
    assert rel(Rd.T @ Rd, D) <= tol["bwd"]
    # solvetransposed on the factor: vector, matrix and low-rank right-hand sides
    rng = np.random.default_rng(15)
    b = rng.standard_normal(1024)
    x = host(G.solvetransposed(R, dev(b, dt)))
    assert rel(Rd.T @ x, b) <= tol["solve"]
    if dt == torch.float64:
        assert rel(x, A.solvetransposed(A.cholesky(T), b)) <= tol["fwd"]
    B = rng.standard_normal((1024, 5))
    X = host(G.solvetransposed(R, dev(B, dt)))
    assert rel(Rd.T @ X, B) <= tol["solve"]
    L = rand_lr(rng, 1024, 64, 3)
    XL = G.solvetransposed(R, lr_dev(L, dt))
    assert rel(Rd.T @ host(XL.U), L.U) <= tol["solve"]
    assert np.array_equal(host(XL.V), host(lr_dev(L, dt).V))


@pytest.mark.parametrize("dt", DT)
@pytest.mark.parametrize("n,leaf", [(1024, 64), (2000, 50), (4096, 128)])
def test_native_cholesky_matches_recursion(dt, n, leaf):
    """hm_hchol_factor (the recursion of src/cholesky.jl:12-92 run natively,
    R12'R12 passed whole into the A22 updates) against the block-by-block
    recursion and the oracle, on uneven and deeper trees."""
    T, D = A.spd_hodlr(n, leaf, kernel="gauss", seed=n)
    Td = tree_dev(T, dt)
    Rn = G.hierarchicalcholesky(Td)
    Rp = G.hierarchicalcholesky(Td, native=False)
    Rdn, Rdp = A.todense(tree_host(Rn)), A.todense(tree_host(Rp))
    tol = CHOL[dt]
    assert np.allclose(np.tril(Rdn, -1), 0)
    assert rel(Rdn, Rdp) <= tol["fwd"]
    assert rel(Rdn.T @ Rdn, D) <= tol["bwd"]
    if dt == torch.float64:
        assert rel(Rdn, A.todense(A.cholesky(T))) <= tol["fwd"]
    # the leaves carry their inverses, which solvetransposed applies
    leaves = [b for b, _, _ in Rn.leaves() if G._is_dense(b)]
    nmax = 112 if dt == torch.float64 else 159        # leaves whose inverse hm_trtri_batched makes
    assert all(getattr(b, "_hm_inverse", None) is not None for b in leaves if b.shape[0] <= nmax)
    b = np.random.default_rng(n + 1).standard_normal(n)
    x = host(G.solvetransposed(Rn, dev(b, dt)))
    assert rel(Rdn.T @ x, b) <= tol["solve"]
    # the factor's memory lives as long as its tensors do
    U = [blk for blk, _, _ in Rn.leaves() if isinstance(blk, hm.LowRankMatrix)][0].U
    del Rn
    import gc
    gc.collect()
    torch.cuda.synchronize()
    assert torch.isfinite(U).all()


def test_native_cholesky_edge_cases():
    """hm_hchol_factor on trees the driver handles by its other paths: leaves
    of 200 rows (beyond the fused leaf kernel: the batched Cholesky kernel and
    substitution by R in the solves, no inverse) and blocks of rank 0 (R12 of
    rank 0, no update), against the oracle's factor."""
    dt = torch.float64
    T, D = A.spd_hodlr(1600, 200, kernel="gauss", seed=31)
    R = G.hierarchicalcholesky(tree_dev(T, dt))
    Rd = A.todense(tree_host(R))
    assert rel(Rd, A.todense(A.cholesky(T))) <= CHOL[dt]["fwd"]
    assert rel(Rd.T @ Rd, D) <= CHOL[dt]["bwd"]
    # rank 0: a block-diagonal SPD matrix whose upper blocks are empty LowRankMatrix
    T, D = A.spd_hodlr(512, 64, kernel="gauss", seed=32)

    def zero_blocks(B):
        if isinstance(B, A.HB):
            B.blocks[0][1] = A.LR(np.zeros((B.blocks[0][1].U.shape[0], 0)), np.zeros(0),
                                  np.zeros((B.blocks[0][1].V.shape[0], 0)))
            zero_blocks(B.blocks[0][0])
            zero_blocks(B.blocks[1][1])
    zero_blocks(T)
    D = A.todense(T)
    D = np.triu(D) + np.triu(D, 1).T
    R = G.hierarchicalcholesky(tree_dev(T, dt))
    Rd = A.todense(tree_host(R))
    assert rel(Rd.T @ Rd, D) <= CHOL[dt]["bwd"]
    assert rel(Rd, A.todense(A.cholesky(T))) <= CHOL[dt]["fwd"]
    assert all(b.U.shape[1] == 0 for b, _, _ in R.leaves() if isinstance(b, hm.LowRankMatrix))


def test_native_cholesky_releases_memory():
    """The factor's memory (held by its tensors) and the driver's temporary
    arenas, streams and staging buffers are all released: device memory
    returns to its level after repeated factorisations once the factors are
    dropped, also after a factorisation that fails."""
    import gc
    dt = torch.float64
    T, _ = A.spd_hodlr(2048, 64, kernel="gauss", seed=33)
    Td = tree_dev(T, dt)
    Tb, _ = A.spd_hodlr(512, 64, seed=34)
    Tb.blocks[0][0].blocks[0][0].blocks[0][0][0, 0] = -1.0
    Tbd = tree_dev(Tb, dt)                          # torch's own allocations before the baseline
    R = G.hierarchicalcholesky(Td)                  # warm-up: modules, attributes
    del R
    gc.collect()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        R = G.hierarchicalcholesky(Td)
        assert R.blocksize() == (2, 2)
        del R
    with pytest.raises(np.linalg.LinAlgError):
        G.hierarchicalcholesky(Tbd)
    gc.collect()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


@pytest.mark.parametrize("dt", DT)
def test_solve_ops_agree(dt):
    """hm_solve_transposed with a diagonal leaf given four ways: R (HM_SOLVE_TRSM),
    R^{-1} (HM_SOLVE_INV), R^T (HM_SOLVE_LTRSM, staged in shared memory up to 64
    rows, read from global memory above) and against numpy's R^{-T} b; the
    low-rank update between two leaves as in src/cholesky.jl:142-228."""
    import ctypes
    from hierarchicalmatrices import _lib
    rng = np.random.default_rng(23)
    tol = 1e-12 if dt == torch.float64 else 2e-5
    for n1, n2 in ((40, 64), (100, 70)):
        R1 = np.triu(rng.standard_normal((n1, n1))) + 4 * np.eye(n1)
        R2 = np.triu(rng.standard_normal((n2, n2))) + 4 * np.eye(n2)
        U, sg, V = rng.standard_normal((n1, 3)), rng.random(3), rng.standard_normal((n2, 3))
        b = rng.standard_normal((n1 + n2, 2))
        x1 = np.linalg.solve(R1.T, b[:n1])
        x2 = np.linalg.solve(R2.T, b[n1:] - V @ (sg[:, None] * (U.T @ x1)))
        ref = np.vstack([x1, x2])
        keep = [dev(m, dt) for m in (R1, R2, np.linalg.inv(R1), np.linalg.inv(R2), R1.T.copy(), R2.T.copy(), U, sg, V)]
        d = dict(zip(("R1", "R2", "W1", "W2", "L1", "L2", "U", "s", "V"), keep))
        for kind, a1, a2 in ((_lib.HM_SOLVE_TRSM, "R1", "R2"), (_lib.HM_SOLVE_INV, "W1", "W2"),
                             (_lib.HM_SOLVE_LTRSM, "L1", "L2")):
            ops = (_lib.SolveOp * 3)()
            ops[0].kind, ops[0].o1, ops[0].n1, ops[0].A, ops[0].ld = kind, 0, n1, d[a1].data_ptr(), n1
            ops[1].kind, ops[1].r, ops[1].o1, ops[1].n1, ops[1].o2, ops[1].n2 = _lib.HM_SOLVE_LR, 3, 0, n1, n1, n2
            ops[1].A, ops[1].ld, ops[1].s, ops[1].B, ops[1].ld2 = d["U"].data_ptr(), n1, d["s"].data_ptr(), d["V"].data_ptr(), n2
            ops[2].kind, ops[2].o1, ops[2].n1, ops[2].A, ops[2].ld = kind, n1, n2, d[a2].data_ptr(), n2
            X = dev(b, dt)
            _lib.check(_lib.lib.hm_solve_transposed(_lib.HM_F64 if dt == torch.float64 else _lib.HM_F32, 3, ops,
                                                     ctypes.c_void_p(X.data_ptr()), X.stride(1), 2, None))
            torch.cuda.synchronize()
            assert rel(host(X), ref) <= tol, (kind, n1)


@pytest.mark.parametrize("dt", DT)
def test_trtri_batched(dt):
    """hm_trtri_batched: W = R^{-1} of upper triangular blocks (the inverses
    solvetransposed applies to small diagonal leaves) against numpy's inverse."""
    import ctypes
    from hierarchicalmatrices import _lib
    rng = np.random.default_rng(17)
    nmax = 112 if dt == torch.float64 else 159
    sizes = [1, 17, 64, 96, nmax]
    Rs = [np.triu(rng.standard_normal((n, n))) + 4 * np.eye(n) for n in sizes]
    Rd = [dev(R, dt) for R in Rs]
    Wd = [torch.full((n, n), float("nan"), dtype=dt, device="cuda").t() for n in sizes]
    arr = (_lib.TrtriProblem * len(sizes))()
    for i, n in enumerate(sizes):
        arr[i].n, arr[i].R, arr[i].ldr = n, Rd[i].data_ptr(), Rd[i].stride(1)
        arr[i].W, arr[i].ldw = Wd[i].data_ptr(), Wd[i].stride(1)
    dti = _lib.HM_F64 if dt == torch.float64 else _lib.HM_F32
    _lib.check(_lib.lib.hm_trtri_batched(dti, len(sizes), arr, None))
    torch.cuda.synchronize()
    tol = 1e-13 if dt == torch.float64 else 2e-6
    for R, W in zip(Rs, Wd):
        Wh = host(W)
        assert np.all(np.tril(Wh, -1) == 0)
        assert rel(Wh, np.linalg.inv(R)) <= tol * np.linalg.cond(R)
    big = nmax + 1
    Rb = dev(np.eye(big), dt)
    Wb = torch.empty((big, big), dtype=dt, device="cuda")
    pb = (_lib.TrtriProblem * 1)()
    pb[0].n, pb[0].R, pb[0].ldr, pb[0].W, pb[0].ldw = big, Rb.data_ptr(), big, Wb.data_ptr(), big
    assert _lib.lib.hm_trtri_batched(dti, 1, pb, None) == _lib.HM_ERR_UNSUPPORTED


def test_cholesky_errors():
    T, _ = A.spd_hodlr(128, 32, seed=16)
    T.blocks[1][1].blocks[1][1][0, 0] = -1.0          # the last 32 x 32 diagonal leaf
    with pytest.raises(np.linalg.LinAlgError):
        G.hierarchicalcholesky(tree_dev(T, torch.float64))
    # the first leaf fails: the rest of the factorisation runs on its NaNs and
    # the pivot check at the end still names the first failure
    T, _ = A.spd_hodlr(128, 32, seed=16)
    T.blocks[0][0].blocks[0][0][0, 0] = -1.0
    with pytest.raises(np.linalg.LinAlgError, match="pivot 1"):
        G.hierarchicalcholesky(tree_dev(T, torch.float64))
    H3 = hm.HierarchicalMatrix(3, 3)
    with pytest.raises(AssertionError):
        G.hierarchicalcholesky(H3)
    with pytest.raises(np.linalg.LinAlgError):
        G.hierarchicalcholesky(dev(-np.eye(4), torch.float64))
