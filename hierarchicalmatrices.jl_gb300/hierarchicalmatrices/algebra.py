"""Low-rank arithmetic, H +/- L, H +/- H and the hierarchical Cholesky on the GPU.

Mirrors, with the reference's operand order and truncation rule:
  * ``getrank``, ``svdtrunc``, ``lrzeros``           src/LowRankMatrix.jl:70-93
  * ``L1 + L2``, ``L1 - L2``                         src/LowRankMatrix.jl:95-111
  * ``L1 * L2``, ``L1' * L2``                        src/LowRankMatrix.jl:113-126
  * ``A * L``, ``L * A``, ``D * L``, ``L * D``       src/LowRankMatrix.jl:128-158
  * ``B * L``, ``L * B``, ``L / B`` (B a number)     src/LowRankMatrix.jl:160-171
  * ``H + L``, ``L + H``, ``H - L``, ``L - H``       src/algebra.jl:394-524
  * ``G + H``, ``G - H`` (same block structure)      src/hierarchical.jl:174-231
  * ``hierarchicalcholesky``                         src/cholesky.jl:12-92
  * ``solvetransposed``                              src/cholesky.jl:97-228

Every block's arithmetic runs in libhmgpu.so (hm_lr_svd: Householder QR and a
Jacobi SVD per block; hm_gemm_batched, hm_axpby_batched, hm_potrf_batched,
hm_solve_transposed); this module walks the block trees in the reference's
order and batches all blocks of one operation into one call.  Matrices are
column-major CUDA tensors (FP64 or FP32); a LowRankMatrix holds U (m x r),
sigma (r) and V (n x r) on the device.  Results of the truncated SVDs differ
from LAPACK's by the choice of singular vectors (signs, rotations within
repeated singular values) and by rounding; the matrices they represent agree
to rounding, and ranks agree wherever the spectrum is separated from the
getrank threshold.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .hierarchical import _EPOCH, AbstractHierarchical, Adjoint, LowRankMatrix, _colmajor, _is_dense


class Diagonal:
    """LinearAlgebra.Diagonal(d) for the products of src/LowRankMatrix.jl:144-158."""

    def __init__(self, d):
        self.diag = d
        self.shape = (int(d.shape[0]), int(d.shape[0]))


# ------------------------------------------------------------------ helpers

def _torch():
    import torch
    return torch


def _stream():
    from .kernelmatrix import _stream_ptr
    return _stream_ptr(None)


def _dt(t):
    torch = _torch()
    if t.dtype == torch.float64:
        return _lib.HM_F64
    if t.dtype == torch.float32:
        return _lib.HM_F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def _dev(a, dtype=None):
    """A column-major CUDA tensor (stride(0) == 1) of a matrix or a vector."""
    torch = _torch()
    if not isinstance(a, torch.Tensor):
        a = torch.as_tensor(np.asarray(a), device="cuda")
    if dtype is not None and a.dtype != dtype:
        a = a.to(dtype)
    if not a.is_cuda:
        a = a.cuda()
    if a.dim() == 1:
        return a.contiguous()
    return _colmajor(a)


def _ld(t):
    return max(int(t.stride(1)) if t.dim() == 2 else int(t.shape[0]), int(t.shape[0]), 1)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else None


def _empty(m, n, dtype):
    torch = _torch()
    return torch.empty((n, m), dtype=dtype, device="cuda").t()


def _lr_dev(L, dtype=None):
    """(U, sigma, V) of a LowRankMatrix as column-major CUDA tensors of one dtype."""
    dtype = dtype or (L.U.dtype if hasattr(L.U, "dtype") and not isinstance(L.U, np.ndarray) else None)
    U = _dev(L.U, dtype)
    return U, _dev(L.sigma, U.dtype), _dev(L.V, U.dtype)


def getrank(sigma):
    """getrank(sigma) (src/LowRankMatrix.jl:70-80): the largest r with
    sigma[r] > length(sigma) * eps(sigma[1]) (1-based), 0 for no values."""
    s = np.asarray(sigma.detach().cpu() if hasattr(sigma, "detach") else sigma)
    r = len(s)
    if r == 0:
        return 0
    tol = r * np.spacing(np.abs(s[0]).astype(s.dtype))
    while r >= 1:
        if s[r - 1] > tol:
            return r
        r -= 1
    return r


# ------------------------------------------------------------------ batched calls

class _SvdBatch:
    """Truncated SVDs X = P M Q^T of many blocks, run as one hm_lr_svd call."""

    def __init__(self, dtype):
        self.dtype = dtype
        self.specs = []

    def add(self, m, n, P=(), Q=(), s=(), sign2=1.0, qr_left=True, qr_right=True, Xm=None, Ym=None, identity_q=False):
        """P, Q: lists of one or two (tensor, columns) parts; s: the matching
        diagonal parts (or (s1, s2) of the Xm^T Ym core).  Returns the slot
        whose LowRankMatrix ``run`` fills in."""
        self.specs.append(dict(m=m, n=n, P=list(P), Q=list(Q), s=list(s), sign2=sign2, qr_left=qr_left,
                               qr_right=qr_right, Xm=Xm, Ym=Ym, identity_q=identity_q))
        return len(self.specs) - 1

    def run(self):
        """One hm_lr_svd call for every problem with a non-empty core; the
        others (no columns, or an empty inner dimension) have rank 0."""
        torch = _torch()
        res = [None] * len(self.specs)
        live, outs, keep = [], [], []
        for i, sp in enumerate(self.specs):
            P, Q = sp["P"], sp["Q"]
            a = sum(c for _, c in P)
            b = sp["n"] if sp["identity_q"] else sum(c for _, c in Q)
            ka = min(sp["m"], a) if sp["qr_left"] else a
            kb = min(sp["n"], b) if sp["qr_right"] else b
            q = min(ka, kb)
            if q == 0 or (sp["Xm"] is not None and sp["Xm"].shape[0] == 0):
                res[i] = LowRankMatrix(_empty(sp["m"], 0, self.dtype), torch.empty(0, dtype=self.dtype, device="cuda"),
                                       _empty(sp["n"], 0, self.dtype))
                continue
            live.append(i)
            outs.append((_empty(sp["m"], q, self.dtype), torch.empty(q, dtype=self.dtype, device="cuda"),
                         _empty(sp["n"], q, self.dtype)))
        if not live:
            return res
        arr = (_lib.LrProblem * len(live))()
        for k, i in enumerate(live):
            sp, pb = self.specs[i], arr[k]
            P, Q, s = sp["P"], sp["Q"], sp["s"]
            pb.m, pb.n = sp["m"], sp["n"]
            pb.qr_left, pb.qr_right = int(sp["qr_left"]), int(sp["qr_right"])
            for j, (t, c) in enumerate(P):
                if j == 0:
                    pb.P1, pb.ldp1, pb.a1 = _ptr(t), _ld(t), c
                else:
                    pb.P2, pb.ldp2, pb.a2 = _ptr(t), _ld(t), c
            if sp["identity_q"]:
                pb.b1 = sp["n"]                      # Q1 = NULL: the identity
            else:
                for j, (t, c) in enumerate(Q):
                    if j == 0:
                        pb.Q1, pb.ldq1, pb.b1 = _ptr(t), _ld(t), c
                    else:
                        pb.Q2, pb.ldq2, pb.b2 = _ptr(t), _ld(t), c
            if len(s) > 0:
                pb.s1 = _ptr(s[0])
            if len(s) > 1:
                pb.s2 = _ptr(s[1])
            pb.sign2 = float(sp["sign2"])
            if sp["Xm"] is not None:
                X, Y = sp["Xm"], sp["Ym"]
                pb.Xm, pb.Ym, pb.t, pb.ldx, pb.ldy = _ptr(X), _ptr(Y), int(X.shape[0]), _ld(X), _ld(Y)
            U, sv, V = outs[k]
            pb.U, pb.s, pb.V = _ptr(U), _ptr(sv), _ptr(V)
            keep.append((P, Q, s, sp["Xm"], sp["Ym"]))
        ranks = (ctypes.c_int32 * len(live))()
        dt = _lib.HM_F64 if self.dtype == torch.float64 else _lib.HM_F32
        check(lib.hm_lr_svd(dt, len(live), arr, ranks, _stream()))
        for k, i in enumerate(live):
            U, sv, V = outs[k]
            r = int(ranks[k])
            res[i] = LowRankMatrix(U[:, :r], sv[:r], V[:, :r])
        del keep
        return res


def _gemm(dtype, probs):
    """probs: dicts with m, n, k, P, transp, Q, transq, s, alpha, beta, C, D."""
    if not probs:
        return
    arr = (_lib.GemmProblem * len(probs))()
    for i, g in enumerate(probs):
        pb = arr[i]
        pb.m, pb.n, pb.k = g["m"], g["n"], g["k"]
        if g["k"] > 0:
            pb.P, pb.ldp, pb.transp = _ptr(g["P"]), _ld(g["P"]), int(g.get("transp", 0))
            pb.Q, pb.ldq, pb.transq = _ptr(g["Q"]), _ld(g["Q"]), int(g.get("transq", 0))
            pb.s = _ptr(g.get("s"))
        pb.alpha, pb.beta = float(g.get("alpha", 1.0)), float(g.get("beta", 0.0))
        C = g.get("C")
        if C is not None:
            pb.C, pb.ldc = _ptr(C), _ld(C)
        pb.D, pb.ldd = _ptr(g["D"]), _ld(g["D"])
    check(lib.hm_gemm_batched(_lib.HM_F64 if dtype == _torch().float64 else _lib.HM_F32, len(probs), arr, _stream()))


def _axpby(dtype, probs):
    """probs: dicts with A, alpha, B, beta, dr, dc, D (all m x n)."""
    probs = [g for g in probs if g["D"].numel() > 0]
    if not probs:
        return
    arr = (_lib.AxpbyProblem * len(probs))()
    for i, g in enumerate(probs):
        pb = arr[i]
        D = g["D"]
        pb.m = int(D.shape[0])
        pb.n = int(D.shape[1]) if D.dim() == 2 else 1
        pb.A, pb.lda = _ptr(g["A"]), _ld(g["A"])
        if g.get("B") is not None:
            pb.B, pb.ldb = _ptr(g["B"]), _ld(g["B"])
        pb.dr, pb.dc = _ptr(g.get("dr")), _ptr(g.get("dc"))
        pb.alpha, pb.beta = float(g.get("alpha", 1.0)), float(g.get("beta", 0.0))
        pb.D, pb.ldd = _ptr(D), _ld(D)
    check(lib.hm_axpby_batched(_lib.HM_F64 if dtype == _torch().float64 else _lib.HM_F32, len(probs), arr, _stream()))


def _copy(A):
    D = _empty(A.shape[0], A.shape[1], A.dtype) if A.dim() == 2 else _torch().empty_like(A)
    _axpby(A.dtype, [dict(A=A, D=D)])
    return D


# ------------------------------------------------------------------ LowRankMatrix algebra

def lrzeros(dtype, m, n):
    """lrzeros(T, m, n) (src/LowRankMatrix.jl:88-93): the m x n rank-0 matrix."""
    torch = _torch()
    tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
    return LowRankMatrix(_empty(m, 0, tdt), torch.empty(0, dtype=tdt, device="cuda"), _empty(n, 0, tdt))


def svdtrunc(A):
    """svdtrunc(A) (src/LowRankMatrix.jl:82-86): the SVD of a dense matrix
    truncated by getrank (min(size(A)) <= 4096)."""
    A = _dev(A)
    m, n = A.shape
    if n > m:
        L = svdtrunc(_dev(A.t().contiguous()))          # svd(A') = V S U'
        return LowRankMatrix(L.V, L.sigma, L.U)
    torch = _torch()
    ones = torch.ones(n, dtype=A.dtype, device="cuda")
    b = _SvdBatch(A.dtype)
    b.add(m, n, P=[(A, n)], s=[ones], qr_left=True, qr_right=False, identity_q=True)
    return b.run()[0]


def _lr_sum(L1, L2, sign):
    if L1.shape != L2.shape:
        raise ValueError(f"DimensionMismatch: {L1.shape} and {L2.shape}")
    U1, s1, V1 = _lr_dev(L1)
    U2, s2, V2 = _lr_dev(L2, U1.dtype)
    b = _SvdBatch(U1.dtype)
    b.add(L1.shape[0], L1.shape[1], P=[(U1, U1.shape[1]), (U2, U2.shape[1])],
          Q=[(V1, V1.shape[1]), (V2, V2.shape[1])], s=[s1, s2], sign2=sign)
    return b.run()[0]


def lr_add(L1, L2):
    """L1 + L2 (src/LowRankMatrix.jl:95-102)."""
    return _lr_sum(L1, L2, 1.0)


def lr_sub(L1, L2):
    """L1 - L2 (src/LowRankMatrix.jl:104-111)."""
    return _lr_sum(L1, L2, -1.0)


def _lr_core_product(P, Q, X, Y, s1, s2, m, n):
    b = _SvdBatch(P.dtype)
    b.add(m, n, P=[(P, P.shape[1])], Q=[(Q, Q.shape[1])], s=[s1, s2], qr_left=False, qr_right=False, Xm=X, Ym=Y)
    return b.run()[0]


def lr_mul(L1, L2):
    """L1 * L2 (src/LowRankMatrix.jl:113-118): svd(Sigma1 V1'U2 Sigma2), U1 W, V2 Z."""
    if L1.shape[1] != L2.shape[0]:
        raise ValueError(f"DimensionMismatch: {L1.shape} * {L2.shape}")
    U1, s1, V1 = _lr_dev(L1)
    U2, s2, V2 = _lr_dev(L2, U1.dtype)
    return _lr_core_product(U1, V2, V1, U2, s1, s2, L1.shape[0], L2.shape[1])


def lr_adjmul(L1, L2):
    """L1' * L2 (src/LowRankMatrix.jl:120-126): svd(Sigma1 U1'U2 Sigma2), V1 W, V2 Z."""
    if L1.shape[0] != L2.shape[0]:
        raise ValueError(f"DimensionMismatch: {L1.shape}' * {L2.shape}")
    U1, s1, V1 = _lr_dev(L1)
    U2, s2, V2 = _lr_dev(L2, U1.dtype)
    return _lr_core_product(V1, V2, U1, U2, s1, s2, L1.shape[1], L2.shape[1])


def dense_lr_mul(A, L):
    """A * L (src/LowRankMatrix.jl:128-134): qr(A L.U), svd(R Sigma); D * L for a
    Diagonal D (:144-150)."""
    U, s, V = _lr_dev(L)
    r = U.shape[1]
    if isinstance(A, Diagonal):
        d = _dev(A.diag, U.dtype)
        AU = _empty(U.shape[0], r, U.dtype)
        _axpby(U.dtype, [dict(A=U, dr=d, D=AU)])
        m = U.shape[0]
    else:
        A = _dev(A, U.dtype)
        if A.shape[1] != U.shape[0]:
            raise ValueError(f"DimensionMismatch: {tuple(A.shape)} * {L.shape}")
        m = A.shape[0]
        AU = _empty(m, r, U.dtype)
        _gemm(U.dtype, [dict(m=m, n=r, k=A.shape[1], P=A, Q=U, transq=1, D=AU)])
    b = _SvdBatch(U.dtype)
    b.add(m, L.shape[1], P=[(AU, r)], Q=[(V, r)], s=[s], qr_left=True, qr_right=False)
    return b.run()[0]


def lr_dense_mul(L, A):
    """L * A (src/LowRankMatrix.jl:136-142): qr(A' L.V), svd(Sigma R'); L * D for
    a Diagonal D (:152-158)."""
    U, s, V = _lr_dev(L)
    r = U.shape[1]
    if isinstance(A, Diagonal):
        d = _dev(A.diag, U.dtype)
        AtV = _empty(V.shape[0], r, U.dtype)
        _axpby(U.dtype, [dict(A=V, dr=d, D=AtV)])
        n = V.shape[0]
    else:
        A = _dev(A, U.dtype)
        if A.shape[0] != V.shape[0]:
            raise ValueError(f"DimensionMismatch: {L.shape} * {tuple(A.shape)}")
        n = A.shape[1]
        AtV = _empty(n, r, U.dtype)
        _gemm(U.dtype, [dict(m=n, n=r, k=A.shape[0], P=A, transp=1, Q=V, transq=1, D=AtV)])
    b = _SvdBatch(U.dtype)
    b.add(L.shape[0], n, P=[(U, r)], Q=[(AtV, r)], s=[s], qr_left=False, qr_right=True)
    return b.run()[0]


def lr_scale(L, B):
    """B * L, L * B (src/LowRankMatrix.jl:160-161, 163-168): sigma scaled by B."""
    U, s, V = _lr_dev(L)
    out = _torch().empty_like(s)
    if s.numel():
        _axpby(s.dtype, [dict(A=s.reshape(-1, 1), alpha=float(B), D=out.reshape(-1, 1))])
    return LowRankMatrix(U, out, V)


def times(A, B):
    """The reference's ``*`` between LowRankMatrix, Adjoint(LowRankMatrix),
    dense matrices, Diagonal and numbers."""
    if isinstance(A, Adjoint) and isinstance(A.parent, LowRankMatrix) and isinstance(B, LowRankMatrix):
        return lr_adjmul(A.parent, B)
    if isinstance(A, LowRankMatrix):
        if isinstance(B, LowRankMatrix):
            return lr_mul(A, B)
        if isinstance(B, (int, float, np.floating)):
            return lr_scale(A, B)
        if isinstance(B, Diagonal) or _is_dense(B):
            return lr_dense_mul(A, B)
    if isinstance(B, LowRankMatrix):
        if isinstance(A, (int, float, np.floating)):
            return lr_scale(B, A)
        if isinstance(A, Diagonal) or _is_dense(A):
            return dense_lr_mul(A, B)
    raise TypeError(f"no method * for {type(A).__name__} and {type(B).__name__}")


# ------------------------------------------------------------------ H +/- L, H +/- H

def _sub_lr(L, pr, qr):
    """L[pr, qr] (src/LowRankMatrix.jl:60-62) as device views."""
    U, s, V = L
    return U[pr[0]:pr[1]], s, V[qr[0]:qr[1]]


class _Walk:
    """One blockwise operation over a tree: collects the dense and low-rank
    block problems, runs each kind as one batched call, then fills the
    result tree."""

    def __init__(self, dtype):
        self.dtype = dtype
        self.svd = _SvdBatch(dtype)
        self.gemm = []
        self.axpby = []
        self.fill = []          # (tree, m, n, kind, payload)

    def finish(self):
        _gemm(self.dtype, self.gemm)
        _axpby(self.dtype, self.axpby)
        res = self.svd.run()
        for G, m, n, kind, payload in self.fill:
            block = res[payload] if kind == "svd" else payload
            G[_block(m + 1), _block(n + 1)] = block


def _block(k):
    from .hierarchical import Block
    return Block(k)


def _hl_walk(H, L, sign_h, sign_l, lr_first, W):
    """G = sign_h H + sign_l L[...] blockwise (src/algebra.jl:394-524), with the
    low-rank part L = (U, s, V) first in the QR stacks when lr_first (L +/- H)."""
    M, N = H.blocksize()
    G = type(H)(M, N, dtype=H.dtype)
    p = 0
    for m in range(M):
        q = 0
        for n in range(N):
            tag = H.assigned[m, n]
            if tag != 0:
                pr = (p, p + H.blocksize(m + 1, n + 1, 1))
                qr = (q, q + H.blocksize(m + 1, n + 1, 2))
                b = H.block(m, n)
                Us, ss, Vs = _sub_lr(L, pr, qr)
                if isinstance(b, AbstractHierarchical):
                    G[_block(m + 1), _block(n + 1)] = _hl_walk(b, (Us, ss, Vs), sign_h, sign_l, lr_first, W)
                elif isinstance(b, LowRankMatrix):
                    Ub, sb, Vb = _lr_dev(b, W.dtype)
                    r, rb = Us.shape[1], Ub.shape[1]
                    if lr_first:          # L[pr, qr] +/- B
                        slot = W.svd.add(pr[1] - pr[0], qr[1] - qr[0], P=[(Us, r), (Ub, rb)], Q=[(Vs, r), (Vb, rb)],
                                         s=[ss, sb], sign2=sign_h)
                    else:                 # B +/- L[pr, qr]
                        slot = W.svd.add(pr[1] - pr[0], qr[1] - qr[0], P=[(Ub, rb), (Us, r)], Q=[(Vb, rb), (Vs, r)],
                                         s=[sb, ss], sign2=sign_l)
                    W.fill.append((G, m, n, "svd", slot))
                elif _is_dense(b):
                    Db = _dev(b, W.dtype)
                    out = _empty(Db.shape[0], Db.shape[1], W.dtype)
                    W.gemm.append(dict(m=Db.shape[0], n=Db.shape[1], k=Us.shape[1], P=Us, Q=Vs, s=ss,
                                       alpha=sign_l, beta=sign_h, C=Db, D=out))
                    W.fill.append((G, m, n, "dense", out))
                else:
                    raise TypeError(f"no method +/- for {type(b).__name__} and LowRankMatrix")
            q += H.blocksize(1, n + 1, 2)
        p += H.blocksize(m + 1, N, 1)
    return G


def h_lr(H, L, sign_h=1.0, sign_l=1.0, lr_first=False):
    """sign_h H + sign_l L for a hierarchical H and a LowRankMatrix L."""
    if tuple(H.shape) != tuple(L.shape):
        raise ValueError(f"DimensionMismatch: {H.shape} and {L.shape}")
    dtype = _dev(L.U).dtype
    W = _Walk(dtype)
    G = _hl_walk(H, _lr_dev(L, dtype), sign_h, sign_l, lr_first, W)
    W.finish()
    return G


def _hh_walk(G, H, sign, W):
    M, N = H.blocksize()
    F = type(H)(M, N, dtype=H.dtype)
    for m in range(M):
        for n in range(N):
            tg, th = G.assigned[m, n], H.assigned[m, n]
            if tg != th or th == 0:
                continue          # the reference assigns only blocks of equal type
            a, b = G.block(m, n), H.block(m, n)
            if isinstance(b, AbstractHierarchical):
                F[_block(m + 1), _block(n + 1)] = _hh_walk(a, b, sign, W)
            elif isinstance(b, LowRankMatrix):
                U1, s1, V1 = _lr_dev(a, W.dtype)
                U2, s2, V2 = _lr_dev(b, W.dtype)
                if a.shape != b.shape:
                    raise ValueError(f"DimensionMismatch: {a.shape} and {b.shape}")
                slot = W.svd.add(a.shape[0], a.shape[1], P=[(U1, U1.shape[1]), (U2, U2.shape[1])],
                                 Q=[(V1, V1.shape[1]), (V2, V2.shape[1])], s=[s1, s2], sign2=sign)
                W.fill.append((F, m, n, "svd", slot))
            elif _is_dense(b):
                A, B = _dev(a, W.dtype), _dev(b, W.dtype)
                if tuple(A.shape) != tuple(B.shape):
                    raise ValueError(f"DimensionMismatch: {tuple(A.shape)} and {tuple(B.shape)}")
                out = _empty(A.shape[0], A.shape[1], W.dtype)
                W.axpby.append(dict(A=A, B=B, alpha=1.0, beta=sign, D=out))
                W.fill.append((F, m, n, "dense", out))
            else:
                raise TypeError(f"no method +/- for {type(b).__name__}")
    return F


def h_h(G, H, sign=1.0):
    """G + H (sign 1) or G - H (sign -1) blockwise (src/hierarchical.jl:174-231)."""
    W = _Walk(_tree_dtype(H))
    F = _hh_walk(G, H, sign, W)
    W.finish()
    return F


def _tree_dtype(H):
    torch = _torch()
    for b, _, _ in H.leaves():
        if isinstance(b, LowRankMatrix) and isinstance(b.U, torch.Tensor):
            return b.U.dtype
        if isinstance(b, torch.Tensor):
            return b.dtype
    return torch.float64 if H.dtype == np.float64 else torch.float32


def add(A, B):
    """The reference's ``+`` for LowRankMatrix and hierarchical operands."""
    if isinstance(A, LowRankMatrix) and isinstance(B, LowRankMatrix):
        return lr_add(A, B)
    if isinstance(A, AbstractHierarchical) and isinstance(B, LowRankMatrix):
        return h_lr(A, B, 1.0, 1.0, False)
    if isinstance(A, LowRankMatrix) and isinstance(B, AbstractHierarchical):
        return h_lr(B, A, 1.0, 1.0, True)
    if isinstance(A, AbstractHierarchical) and isinstance(B, AbstractHierarchical):
        return h_h(A, B, 1.0)
    raise TypeError(f"no method + for {type(A).__name__} and {type(B).__name__}")


def sub(A, B):
    """The reference's ``-`` for LowRankMatrix and hierarchical operands."""
    if isinstance(A, LowRankMatrix) and isinstance(B, LowRankMatrix):
        return lr_sub(A, B)
    if isinstance(A, AbstractHierarchical) and isinstance(B, LowRankMatrix):
        return h_lr(A, B, 1.0, -1.0, False)
    if isinstance(A, LowRankMatrix) and isinstance(B, AbstractHierarchical):
        return h_lr(B, A, -1.0, 1.0, True)
    if isinstance(A, AbstractHierarchical) and isinstance(B, AbstractHierarchical):
        return h_h(A, B, -1.0)
    raise TypeError(f"no method - for {type(A).__name__} and {type(B).__name__}")


# ------------------------------------------------------------------ dense views of trees

def todense(H, dtype=None):
    """The dense matrix of a hierarchical (or low-rank) matrix on the device:
    what Julia's generic AbstractMatrix arithmetic materialises for H - Matrix."""
    torch = _torch()
    if isinstance(H, LowRankMatrix):
        U, s, V = _lr_dev(H, dtype)
        D = _empty(H.shape[0], H.shape[1], U.dtype)
        _gemm(U.dtype, [dict(m=H.shape[0], n=H.shape[1], k=U.shape[1], P=U, Q=V, s=s, D=D)])
        return D
    dtype = dtype or _tree_dtype(H)
    m, n = H.shape
    D = torch.zeros((n, m), dtype=dtype, device="cuda").t()
    gem, axp = [], []
    for b, p, q in H.leaves():
        sh = b.shape
        view = D[p:p + sh[0], q:q + sh[1]]
        if isinstance(b, LowRankMatrix):
            U, s, V = _lr_dev(b, dtype)
            gem.append(dict(m=sh[0], n=sh[1], k=U.shape[1], P=U, Q=V, s=s, D=view))
        elif _is_dense(b):
            axp.append(dict(A=_dev(b, dtype), D=view))
        else:
            raise TypeError(f"no dense form for {type(b).__name__}")
    _gemm(dtype, [g for g in gem if g["k"] > 0])
    _axpby(dtype, axp)
    return D


# ------------------------------------------------------------------ Cholesky and the solve

def _potrf(A, infos=None):
    """hierarchicalcholesky(A::Matrix) = Matrix(cholesky(Symmetric(A)).U).
    With ``infos`` (a list) the factorisation is queued without waiting and
    its device info word appended; the caller checks the words later."""
    A = _dev(A)
    n = A.shape[0]
    if A.dim() != 2 or A.shape[1] != n:
        raise ValueError(f"DimensionMismatch: Cholesky of a {tuple(A.shape)} matrix")
    R = _empty(n, n, A.dtype)
    arr = (_lib.PotrfProblem * 1)()
    arr[0].n, arr[0].A, arr[0].lda, arr[0].R, arr[0].ldr = n, _ptr(A), _ld(A), _ptr(R), _ld(R)
    if infos is not None:
        word = _torch().zeros(1, dtype=_torch().int32, device=A.device)
        check(lib.hm_potrf_batched_async(_dt(A), 1, arr, ctypes.c_void_p(word.data_ptr()), _stream()))
        infos.append(word)
        return R
    info = (ctypes.c_int32 * 1)()
    st = lib.hm_potrf_batched(_dt(A), 1, arr, info, _stream())
    if st == _lib.HM_ERR_NOT_POSDEF:
        raise np.linalg.LinAlgError(f"PosDefException: matrix is not positive definite; "
                                    f"Cholesky factorization failed at pivot {info[0]}")
    check(st)
    return R


_TAGS_DIAG = (1, 3)      # HierarchicalMatrix or Matrix on the diagonal
_TAGS_OFF = (2, 3)       # LowRankMatrix or Matrix above it


def _check_2x2(A):
    if A.blocksize() != (2, 2):
        raise AssertionError("blocksize(A) == (2, 2)")
    t = (int(A.assigned[0, 0]), int(A.assigned[0, 1]), int(A.assigned[1, 1]))
    if t[0] not in _TAGS_DIAG or t[1] not in _TAGS_OFF or t[2] not in _TAGS_DIAG:
        raise TypeError(f"no method for block types {t} (src/cholesky.jl covers diagonal "
                        "HierarchicalMatrix/Matrix and LowRankMatrix/Matrix above)")
    return t


def hierarchicalcholesky(A, native=True):
    """hierarchicalcholesky(A) (src/cholesky.jl:12-92): the upper factor R with
    R'R = A of a symmetric positive definite 2 x 2 hierarchical matrix (or a
    dense matrix), in the reference's block order:
    R11 = chol(A11); R12 = R11^{-T} A12; R22 = chol(A22 - R12'R12).
    A HODLR tree (every upper off-diagonal block a LowRankMatrix, diagonal
    blocks hierarchical or dense) is factored by one hm_hchol_factor call,
    which runs this recursion natively; other trees (dense off-diagonal
    blocks), or native=False, take the recursion here, one batched call per
    block operation.  The dense diagonal leaves are factored without waiting;
    their pivot checks are read once at the end, and the first failing leaf
    (in the reference's order) raises the PosDefException the reference would
    raise."""
    if _is_dense(A) or not isinstance(A, AbstractHierarchical):
        return _hchol(A, None)
    if native:
        dtype = _tree_dtype(A)
        try:
            nodes = _hodlr_nodes(A, dtype)
        except _NotHodlr:
            nodes = None
        if nodes is not None:
            return _hchol_native(nodes, dtype)
    infos = []
    R = _hchol(A, infos)
    if infos:
        words = _torch().cat(infos).cpu().numpy()
        bad = np.flatnonzero(words)
        if bad.size:
            raise np.linalg.LinAlgError(f"PosDefException: matrix is not positive definite; "
                                        f"Cholesky factorization failed at pivot {int(words[bad[0]])}")
    return R


class _NotHodlr(Exception):
    pass


def _hodlr_nodes(A, dtype):
    """The node list of hm_hchol_factor (pre-order, the root first), each
    node a dict with the tree object and its device blocks; raises _NotHodlr
    for trees the native driver does not take."""
    nodes = []

    def rec(B):
        if _is_dense(B):
            D = _dev(B, dtype)
            if D.dim() != 2 or D.shape[0] != D.shape[1] or D.shape[0] == 0:
                raise _NotHodlr
            nodes.append(dict(obj=B, n=int(D.shape[0]), n1=0, left=-1, right=-1, D=D))
            return len(nodes) - 1
        if not isinstance(B, AbstractHierarchical) or B.blocksize() != (2, 2):
            raise _NotHodlr
        t = (int(B.assigned[0, 0]), int(B.assigned[0, 1]), int(B.assigned[1, 1]))
        if t[0] not in _TAGS_DIAG or t[1] != 2 or t[2] not in _TAGS_DIAG:
            raise _NotHodlr
        i = len(nodes)
        nodes.append(None)
        left, right = rec(B.block(0, 0)), rec(B.block(1, 1))
        U, sg, V = _lr_dev(B.block(0, 1), dtype)
        n1, n2 = nodes[left]["n"], nodes[right]["n"]
        if U.shape[0] != n1 or V.shape[0] != n2 or U.shape[1] != V.shape[1] or sg.shape[0] != U.shape[1]:
            raise _NotHodlr
        nodes[i] = dict(obj=B, n=n1 + n2, n1=n1, left=left, right=right, U=U, s=sg, V=V)
        return i

    rec(A)
    return nodes


class _HcholOwner:
    """The memory of one hm_hchol_factor result; the factor's tensors are
    views of it and keep this object alive, so it is freed with the last."""

    def __init__(self, ctx):
        self.ctx = ctx

    def __del__(self):
        if self.ctx and lib is not None:
            lib.hm_hchol_free(self.ctx)
            self.ctx = None


class _DeviceSpan:
    """__cuda_array_interface__ of a column-major block owned by _HcholOwner."""

    def __init__(self, owner, ptr, shape, strides, typestr):
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": shape, "strides": strides, "typestr": typestr,
                                         "data": (ptr, False), "version": 2}


def _owned(owner, ptr, m, n, ld, dtype):
    torch = _torch()
    if m == 0 or n == 0 or not ptr:
        return torch.empty(m, dtype=dtype, device="cuda") if n is None else _empty(m, n, dtype)
    es = 8 if dtype == torch.float64 else 4
    ts = "<f8" if es == 8 else "<f4"
    if n is None:
        span = _DeviceSpan(owner, ptr, (m,), (es,), ts)
    else:
        span = _DeviceSpan(owner, ptr, (m, n), (es, es * ld), ts)
    return torch.as_tensor(span, device="cuda")


def _hchol_native(nodes, dtype):
    """hm_hchol_factor on the node list; the factor as a tree of the input's
    types whose blocks are views of the call's result memory (each dense
    leaf carries its inverse as ``_hm_inverse`` for solvetransposed)."""
    torch = _torch()
    arr = (_lib.HcholNode * len(nodes))()
    for i, nd in enumerate(nodes):
        pb = arr[i]
        pb.n, pb.n1, pb.left, pb.right = nd["n"], nd["n1"], nd["left"], nd["right"]
        if nd["left"] < 0:
            pb.D, pb.ldd = _ptr(nd["D"]), _ld(nd["D"])
        else:
            U, sg, V = nd["U"], nd["s"], nd["V"]
            pb.r = int(U.shape[1])
            pb.U, pb.ldu, pb.s, pb.V, pb.ldv = _ptr(U), _ld(U), _ptr(sg), _ptr(V), _ld(V)
    ctx = ctypes.c_void_p()
    fail = (ctypes.c_int32 * 2)()
    dt = _lib.HM_F64 if dtype == torch.float64 else _lib.HM_F32
    st = lib.hm_hchol_factor(dt, len(nodes), arr, 0, ctypes.byref(ctx), fail, _stream())
    if st == _lib.HM_ERR_NOT_POSDEF:
        raise np.linalg.LinAlgError(f"PosDefException: matrix is not positive definite; "
                                    f"Cholesky factorization failed at pivot {int(fail[1])}")
    check(st)
    owner = _HcholOwner(ctx.value)
    outs = []
    for i in range(len(nodes)):
        o = _lib.HcholOut()
        check(lib.hm_hchol_result(ctx, i, ctypes.byref(o)))
        outs.append(o)

    def build(i):
        nd, o = nodes[i], outs[i]
        if nd["left"] < 0:
            n = nd["n"]
            R = _owned(owner, o.R, n, n, o.ldr, dtype)
            if o.W:
                R._hm_inverse = _owned(owner, o.W, n, n, o.ldw, dtype)
            return R
        n1, n2, r = nd["n1"], nd["n"] - nd["n1"], int(o.r)
        R = type(nd["obj"])(2, 2, dtype=nd["obj"].dtype)
        R[_block(1), _block(1)] = build(nd["left"])
        R[_block(1), _block(2)] = LowRankMatrix(_owned(owner, o.U, n1, r, o.ldu, dtype),
                                                 _owned(owner, o.s, r, None, 0, dtype),
                                                 _owned(owner, o.V, n2, r, o.ldv, dtype))
        R[_block(2), _block(2)] = build(nd["right"])
        return R

    return build(0)


def _hchol(A, infos):
    if _is_dense(A):
        return _potrf(A, infos)
    if not isinstance(A, AbstractHierarchical):
        raise TypeError(f"no method hierarchicalcholesky for {type(A).__name__}")
    _check_2x2(A)
    R = type(A)(2, 2, dtype=A.dtype)
    A11, A12, A22 = A.block(0, 0), A.block(0, 1), A.block(1, 1)
    R11 = _hchol(A11, infos)
    R[_block(1), _block(1)] = R11
    R12 = solvetransposed(R11, A12)
    R[_block(1), _block(2)] = R12
    if isinstance(R12, LowRankMatrix):
        S = lr_adjmul(R12, R12)
        if isinstance(A22, AbstractHierarchical):
            A22m = h_lr(A22, S, 1.0, -1.0, False)
        else:
            D = _dev(A22)
            U, s, V = _lr_dev(S, D.dtype)
            A22m = _empty(D.shape[0], D.shape[1], D.dtype)
            _gemm(D.dtype, [dict(m=D.shape[0], n=D.shape[1], k=U.shape[1], P=U, Q=V, s=s, alpha=-1.0, beta=1.0,
                                 C=D, D=A22m)])
    else:
        M = R12
        D = todense(A22) if isinstance(A22, AbstractHierarchical) else _dev(A22)
        A22m = _empty(D.shape[0], D.shape[1], D.dtype)
        _gemm(D.dtype, [dict(m=D.shape[0], n=D.shape[1], k=M.shape[0], P=M, transp=1, Q=M, transq=1,
                             alpha=-1.0, beta=1.0, C=D, D=A22m)])
    R[_block(2), _block(2)] = _hchol(A22m, infos)
    return R


def _schedule(R, off, ops, keep):
    """The forward-substitution schedule of R^{-T} in the order of the
    reference's recursion (src/cholesky.jl:142-228).  A hierarchical R keeps
    its own schedule (offsets from its first row) until the next block
    assignment, so a factor's schedule is built from its halves' schedules."""
    if isinstance(R, AbstractHierarchical):
        c = getattr(R, "_solve_sched", None)
        if c is None or c[0] != _EPOCH[0]:
            own_ops, own_keep = [], []
            _schedule_build(R, 0, own_ops, own_keep)
            _invert_leaves(own_ops, own_keep)
            c = (_EPOCH[0], own_ops, own_keep)
            R._solve_sched = c
        for o in c[1]:
            if off:
                o = dict(o)
                o["o1"] += off
                if "o2" in o:
                    o["o2"] += off
            ops.append(o)
        keep.extend(c[2])
        return R.shape[1]
    return _schedule_build(R, off, ops, keep)


_INV_MAX = 96      # diagonal leaves up to this size are applied through their inverse


def _invert_leaves(ops, keep):
    """Replace the triangular solves of small diagonal leaves by products with
    their inverses (HM_SOLVE_INV), the inverses made by one batched call: a
    leaf's serial forward substitution on one warp is slow at GB300's FP64
    rate, its inverse's product runs on every warp of the CTA."""
    todo = [o for o in ops if o["kind"] == _lib.HM_SOLVE_TRSM and 0 < o["n1"] <= _INV_MAX]
    for o in todo:                                # leaves of a native factor come with their inverse
        W = getattr(o["A"], "_hm_inverse", None)
        if W is not None:
            keep.append(W)
            o["kind"], o["A"], o["ld"] = _lib.HM_SOLVE_INV, W, _ld(W)
    todo = [o for o in todo if o["kind"] == _lib.HM_SOLVE_TRSM]
    if not todo or any(o["A"].dtype != todo[0]["A"].dtype for o in todo):
        return                                    # nothing to do, or mixed storage: keep the substitutions
    dtype = todo[0]["A"].dtype
    arr = (_lib.TrtriProblem * len(todo))()
    inv = []
    for i, o in enumerate(todo):
        W = _empty(o["n1"], o["n1"], dtype)
        inv.append(W)
        pb = arr[i]
        pb.n, pb.R, pb.ldr, pb.W, pb.ldw = o["n1"], _ptr(o["A"]), o["ld"], _ptr(W), _ld(W)
    check(lib.hm_trtri_batched(_dt(todo[0]["A"]), len(todo), arr, _stream()))
    keep.extend(inv)
    for o, W in zip(todo, inv):
        o["kind"], o["A"], o["ld"] = _lib.HM_SOLVE_INV, W, _ld(W)


def _schedule_build(R, off, ops, keep):
    if _is_dense(R):
        Rd = _dev(R)
        n = Rd.shape[0]
        keep.append(Rd)
        ops.append(dict(kind=_lib.HM_SOLVE_TRSM, o1=off, n1=n, A=Rd, ld=_ld(Rd)))
        return n
    if not isinstance(R, AbstractHierarchical):
        raise TypeError(f"no method solvetransposed for {type(R).__name__}")
    _check_2x2(R)
    R11, R12, R22 = R.block(0, 0), R.block(0, 1), R.block(1, 1)
    s = _schedule(R11, off, ops, keep)
    n2 = R.shape[1] - s
    if isinstance(R12, LowRankMatrix):
        U, sg, V = _lr_dev(R12)
        keep.extend((U, sg, V))
        ops.append(dict(kind=_lib.HM_SOLVE_LR, r=U.shape[1], o1=off, n1=s, o2=off + s, n2=n2, A=U, ld=_ld(U),
                        s=sg, B=V, ld2=_ld(V)))
    else:
        M = _dev(R12)
        keep.append(M)
        ops.append(dict(kind=_lib.HM_SOLVE_DENSE, o1=off, n1=s, o2=off + s, n2=n2, A=M, ld=_ld(M)))
    _schedule(R22, off + s, ops, keep)
    return R.shape[1]


def _solve_inplace(R, X):
    ops, keep = [], []
    _schedule(R, 0, ops, keep)
    arr = (_lib.SolveOp * len(ops))()
    for i, o in enumerate(ops):
        pb = arr[i]
        pb.kind, pb.r = o["kind"], o.get("r", 0)
        pb.o1, pb.n1, pb.o2, pb.n2 = o["o1"], o["n1"], o.get("o2", 0), o.get("n2", 0)
        pb.ld, pb.ld2 = o["ld"], o.get("ld2", 0)
        pb.A, pb.s, pb.B = _ptr(o["A"]), _ptr(o.get("s")), _ptr(o.get("B"))
        if pb.A is None:                         # an empty block: nothing to read
            pb.A = ctypes.c_void_p(X.data_ptr())
    ncols = 1 if X.dim() == 1 else X.shape[1]
    ldb = X.shape[0] if X.dim() == 1 else _ld(X)
    check(lib.hm_solve_transposed(_dt(X), len(ops), arr, ctypes.c_void_p(X.data_ptr()), ldb, ncols, _stream()))
    del keep
    return X


def solvetransposed(R, B):
    """solvetransposed(R, B) = R^{-T} B (src/cholesky.jl:97-228) for an upper
    triangular R (dense or the hierarchical factor of hierarchicalcholesky)
    and B a vector, a dense matrix or a LowRankMatrix (whose U is solved)."""
    n = R.shape[0] if _is_dense(R) else R.shape[1]
    if isinstance(B, LowRankMatrix):
        U, s, V = _lr_dev(B)
        if U.shape[0] != n:
            raise ValueError(f"DimensionMismatch: R is {n} x {n}, U has {U.shape[0]} rows")
        X = _copy(U)
        if X.shape[1] > 0:
            _solve_inplace(R, X)
        return LowRankMatrix(X, s, V)
    Bd = _dev(B)
    if Bd.shape[0] != n:
        raise ValueError(f"DimensionMismatch: R is {n} x {n}, B has {Bd.shape[0]} rows")
    X = _copy(Bd) if Bd.dim() == 2 else _copy(Bd.reshape(-1, 1)).reshape(-1)
    if X.numel() > 0:
        _solve_inplace(R, X)
    return X
