"""Block types and user-assembled hierarchical matrices on the GPU.

Mirrors the reference's generic layer:
  * ``Block(K)``                               src/block.jl:8-10
  * ``hierarchical(name, *types)``             the @hierarchical macro, src/hierarchical.jl:4-232
  * ``HierarchicalMatrix``                     src/HierarchicalMatrix.jl:1 (LowRankMatrix, Matrix blocks)
  * ``LowRankMatrix(U, sigma, V)``             src/LowRankMatrix.jl:28-43
  * ``BarycentricMatrix2D(f, a, b, c, d, x, y, ir, jr)``   src/BarycentricMatrix.jl:236-297
  * ``mul_(y, A, x, istart, jstart, INCX, INCY)`` for dense, transposed, low-rank
    (and adjoint), barycentric and hierarchical blocks   src/algebra.jl:37-277,
    src/HierarchicalMatrix.jl:24-52

Products run on the GPU through libhmgpu.so: device vectors are torch CUDA
tensors; a HierarchicalMatrix is flattened to its leaf blocks (with the
reference's block-walk offsets) and uploaded once, on its first product.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib

_vp = ctypes.c_void_p
_pi64 = ctypes.POINTER(ctypes.c_int64)


class Block:
    """Block(K): index of a block row or column (src/block.jl:8-10)."""

    def __init__(self, K):
        self.K = int(K)

    def __eq__(self, other):
        return isinstance(other, Block) and self.K == other.K

    def __hash__(self):
        return hash(("Block", self.K))

    def __repr__(self):
        return f"Block({self.K})"


def _np64(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy().astype(np.float64)
    except ImportError:
        pass
    return np.asarray(a, dtype=np.float64)


class LowRankMatrix:
    """A = U diag(sigma) V^T (src/LowRankMatrix.jl:28-43); U is m x r, V n x r."""

    def __init__(self, U, sigma, V):
        self.U, self.sigma, self.V = U, sigma, V
        self.shape = (int(U.shape[0]), int(V.shape[0]))

    def rank(self):
        return int(self.sigma.shape[0])

    def dense(self):
        U, s, V = _np64(self.U), _np64(self.sigma), _np64(self.V)
        return (U * s) @ V.T

    def norm(self):
        """norm(L) = first(sigma) (src/LowRankMatrix.jl:46)."""
        return float(_np64(self.sigma[:1])[0])

    def cond(self):
        """cond(L) (src/LowRankMatrix.jl:47): Inf below full rank, else sigma_1 / sigma_r."""
        s = _np64(self.sigma)
        return float("inf") if len(s) < min(self.shape) else float(s[0] / s[-1])

    def getindex(self, i, j):
        """L[i, j], 1-based, summed over k = r:-1:1 (src/LowRankMatrix.jl:50-58)."""
        U, s, V = _np64(self.U[i - 1]), _np64(self.sigma), _np64(self.V[j - 1])
        ret = 0.0
        for k in range(len(s) - 1, -1, -1):
            ret += U[k] * s[k] * V[k]
        return ret

    def __getitem__(self, key):
        """L[ir, jr] for 0-based slices: LowRankMatrix(U[ir, :], sigma, V[jr, :])
        (src/LowRankMatrix.jl:60-62)."""
        ir, jr = key
        if isinstance(ir, slice) and isinstance(jr, slice):
            return LowRankMatrix(self.U[ir], self.sigma, self.V[jr])
        return self.getindex(int(ir) + 1, int(jr) + 1)

    # the reference's arithmetic (src/LowRankMatrix.jl:95-171, src/algebra.jl:394-524)
    def __add__(self, other):
        from . import algebra
        return algebra.add(self, other)

    def __sub__(self, other):
        from . import algebra
        return algebra.sub(self, other)

    def __mul__(self, other):
        from . import algebra
        return algebra.times(self, other)

    def __rmul__(self, other):
        from . import algebra
        return algebra.times(other, self)

    def __matmul__(self, other):
        from . import algebra
        return algebra.times(self, other)

    def __truediv__(self, B):
        from . import algebra
        return algebra.lr_scale(self, 1.0 / float(B))


class BarycentricMatrix2D:
    """The barycentric block of the kernel f on boxes [a, b] x [c, d] for the
    points x[ir], y[jr] (src/BarycentricMatrix.jl:236-297): U F V^T with U, V
    the Lagrange bases at first-kind Chebyshev nodes and F the kernel at the
    nodes.  Factors are computed on the GPU in FP64 and stored as ``dtype``
    device tensors."""

    def __init__(self, f, a, b, c, d, x, y, ir, jr, *, rank=20, dtype=np.float64, device="cuda"):
        import torch
        from .kernelmatrix import _kernel_id
        xs = np.ascontiguousarray(_np64(x)[ir.start:ir.stop])
        ys = np.ascontiguousarray(_np64(y)[jr.start:jr.stop])
        tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32
        self.U = torch.empty((rank, len(xs)), dtype=tdt, device=device).t()    # column-major m x r
        self.V = torch.empty((rank, len(ys)), dtype=tdt, device=device).t()
        self.F = torch.empty((rank, rank), dtype=tdt, device=device).t()
        check(lib.hm_bary_factors(_kernel_id(f), rank, float(a), float(b), float(c), float(d), _lib.f64_ptr(xs),
                                  len(xs), _lib.f64_ptr(ys), len(ys),
                                  _lib.HM_F64 if tdt == torch.float64 else _lib.HM_F32,
                                  self.U.data_ptr(), self.F.data_ptr(), self.V.data_ptr(), None))
        self.ir, self.jr = ir, jr
        self.shape = (len(xs), len(ys))

    def rank(self):
        return int(self.F.shape[0])

    def dense(self):
        U, F, V = _np64(self.U), _np64(self.F), _np64(self.V)
        return U @ F @ V.T


class EvenBarycentricMatrix:
    """EvenBarycentricMatrix(T, f, a, b, c, d) (src/BarycentricMatrix.jl:5-45):
    the block of rows a:b and columns c:d (integers) of a kernel f(T, x, j)
    that couples only rows and columns of matching parity, interpolated in
    the row variable at BLOCKRANK(T) first-kind Chebyshev nodes of [a, b].
    W (n x (b-a+1)) and F ((d-c+1) x n) are formed on the host in FP64 with
    the reference's formulas (F calls the user's f) and stored on the device,
    split by row and column parity, as ``dtype``; mul_ runs its products on
    the GPU (two stride-2 low-rank products, src/algebra.jl:168-239)."""

    @staticmethod
    def factors(f, a, b, c, d, n, T=np.float64):
        """(W, F) in FP64 by src/BarycentricMatrix.jl:17-45: w_i = sum_k
        lambda_k / (2i - a - b - (b - a) x_k), W[k, i] = lambda_k / ((2i - a - b -
        (b - a) x_k) w_i), F[j, k] = f(T, (a + b)/2 + (b - a) x_k / 2, j)."""
        x, lam = _lib.chebyshev(n)
        i = np.arange(a, b + 1, dtype=np.float64)
        den = (2.0 * i[None, :] - a - b) - (b - a) * x[:, None]            # n x m
        w = np.zeros(i.size)
        for k in range(n):                                                  # the reference's order over k
            w += lam[k] * (1.0 / den[k])
        W = lam[:, None] * (1.0 / (den * w[None, :]))
        F = np.empty((d - c + 1, n))
        for k in range(n):
            node = (a + b) / 2 + (b - a) * x[k] / 2
            for jj in range(d - c + 1):
                F[jj, k] = f(T, node, c + jj)
        return W, F

    def __init__(self, f, a, b, c, d, *, dtype=np.float64, rank=None, device="cuda"):
        import torch
        from .kernelmatrix import BLOCKRANK
        T = np.dtype(dtype).type
        n = int(rank) if rank else BLOCKRANK(T)
        a, b, c, d = int(a), int(b), int(c), int(d)
        W, F = self.factors(f, a, b, c, d, n, T)
        self.W, self.F = W, F
        self.a, self.b, self.c, self.d, self.n = a, b, c, d, n
        self.shape = (b - a + 1, d - c + 1)
        tdt = torch.float64 if np.dtype(dtype) == np.float64 else torch.float32

        def dev(M):                                          # column-major device copy
            return torch.tensor(np.ascontiguousarray(M.T), dtype=tdt, device=device).t()
        # parity p (0-based row/column index parity) factors: U_p = W[:, p::2]^T, V_p = F[p::2, :]
        self.U = [dev(W[:, p::2].T) for p in (0, 1)]
        self.V = [dev(F[p::2, :]) for p in (0, 1)]
        self.ones = torch.ones(n, dtype=tdt, device=device)

    def rank(self):
        return self.n

    def dense(self, istart=1, jstart=1):
        """The operator mul_ applies at these offsets (entries couple when
        i + j + istart + jstart is even, 1-based i, j)."""
        m, p = self.shape
        M = (self.F @ self.W).T                                              # m x p, before the parity mask
        ii, jj = np.meshgrid(np.arange(1, m + 1), np.arange(1, p + 1), indexing="ij")
        return np.where((ii + jj + istart + jstart) % 2 == 0, M, 0.0)


class Transpose:
    """transpose(A) for a dense block (src/algebra.jl:50-65)."""

    def __init__(self, A):
        self.parent = A
        self.shape = (A.shape[1], A.shape[0])


class Adjoint:
    """adjoint(L) for a LowRankMatrix or a real dense block (src/algebra.jl:67-82, 133-159)."""

    def __init__(self, A):
        self.parent = A
        self.shape = (A.shape[1], A.shape[0])

    def __mul__(self, other):
        """L1' * L2 (src/LowRankMatrix.jl:120-126)."""
        from . import algebra
        return algebra.times(self, other)

    __matmul__ = __mul__


def transpose(A):
    return Transpose(A)


def adjoint(A):
    return Adjoint(A)


# --------------------------------------------------------------------- @hierarchical

# Incremented by every block assignment of every hierarchical matrix: a cached
# shape or solve schedule is valid while the epoch it was made in is current.
_EPOCH = [0]


class AbstractHierarchical:
    """Base of the classes made by ``hierarchical``: an M x N grid of blocks,
    each of one of the declared types or of the class itself, with the
    ``assigned`` tags of src/hierarchical.jl:49-52 (1 = the class itself,
    l = the (l-1)-th declared type, 0 = empty)."""

    _types = ()
    _store_names = ()

    def __init__(self, M, N, dtype=np.float64):
        self.M, self.N = int(M), int(N)
        self.dtype = np.dtype(dtype)
        self.assigned = np.zeros((self.M, self.N), dtype=np.int64)
        for name in self._store_names:
            setattr(self, name, [[None] * self.N for _ in range(self.M)])
        self._handle = None
        self._handle_dtype = None

    def _tag_of(self, A):
        if isinstance(A, type(self)):
            return 1
        for l, T in enumerate(self._types):
            if _isa(A, T):
                return l + 2
        return 0

    def __setitem__(self, key, A):
        bm, bn = key
        if not (isinstance(bm, Block) and isinstance(bn, Block)):
            raise TypeError("index blocks with H[Block(m), Block(n)] (1-based)")
        m, n = bm.K - 1, bn.K - 1
        tag = self._tag_of(A)
        if tag == 0:
            return        # the reference ignores blocks of other types (src/hierarchical.jl:149-172)
        getattr(self, self._store_names[tag - 1])[m][n] = A
        self.assigned[m, n] = tag
        _EPOCH[0] += 1
        self._invalidate()

    def __getitem__(self, key):
        bm, bn = key
        if isinstance(bm, Block) and isinstance(bn, Block):
            m, n = bm.K - 1, bn.K - 1
            tag = self.assigned[m, n]
            return None if tag == 0 else getattr(self, self._store_names[tag - 1])[m][n]
        return self.getindex(int(bm), int(bn))

    def _invalidate(self):
        if self._handle is not None:
            lib.hm_free(self._handle)
        self._handle = None

    # blockwise sums (src/algebra.jl:394-524, src/hierarchical.jl:174-231)
    def __add__(self, other):
        from . import algebra
        return algebra.add(self, other)

    def __sub__(self, other):
        from . import algebra
        return algebra.sub(self, other)

    def block(self, m, n):
        tag = self.assigned[m, n]
        return None if tag == 0 else getattr(self, self._store_names[tag - 1])[m][n]

    def blocksize(self, m=None, n=None, k=None):
        """blocksize(H) = (M, N); blocksize(H, m, n, k) (1-based) = size of block (m, n) along k."""
        if m is None:
            return (self.M, self.N)
        b = self.block(m - 1, n - 1)
        return 0 if b is None else int(_shape(b)[k - 1])

    @property
    def shape(self):
        # rows from block column N, columns from block row 1 (src/hierarchical.jl:33-47);
        # cached until the next block assignment anywhere
        c = getattr(self, "_shape_cache", None)
        if c is not None and c[0] == _EPOCH[0]:
            return c[1]
        sh = (sum(self.blocksize(m, self.N, 1) for m in range(1, self.M + 1)),
              sum(self.blocksize(1, n, 2) for n in range(1, self.N + 1)))
        self._shape_cache = (_EPOCH[0], sh)
        return sh

    def size(self, dim=None):
        return self.shape if dim is None else self.shape[dim - 1]

    def getindex(self, i, j):
        """Element (i, j), 1-based (src/hierarchical.jl:120-147); CPU."""
        m = 1
        while m <= self.M:
            r = self.blocksize(m, self.N, 1)
            if i > r:
                i -= r
                m += 1
            else:
                break
        n = 1
        while n <= self.N:
            s = self.blocksize(1, n, 2)
            if j > s:
                j -= s
                n += 1
            else:
                break
        b = self.block(m - 1, n - 1)
        if b is None:
            return 0.0
        if isinstance(b, AbstractHierarchical):
            return b.getindex(i, j)
        return float(_dense(b)[i - 1, j - 1])

    # -- flattening and the GPU product ---------------------------------------
    def leaves(self, row0=0, col0=0):
        """Leaf blocks with the offsets of the reference's block walk
        (src/HierarchicalMatrix.jl:24-52): (block, row0, col0)."""
        out = []
        p = 0
        for m in range(self.M):
            q = 0
            for n in range(self.N):
                b = self.block(m, n)
                if isinstance(b, AbstractHierarchical):
                    out.extend(b.leaves(row0 + p, col0 + q))
                elif b is not None:
                    out.append((b, row0 + p, col0 + q))
                q += self.blocksize(1, n + 1, 2)
            p += self.blocksize(m + 1, self.N, 1)
        return out

    def handle(self, dtype=None):
        dtype = np.dtype(dtype or self.dtype)
        if self._handle is not None and self._handle_dtype == dtype:
            return self._handle
        self._invalidate()
        kinds, r0, rr, c0, cc, rk, offs, vals = [], [], [], [], [], [], [], []
        off = 0
        for b, p, q in self.leaves():
            if isinstance(b, LowRankMatrix):
                U, s, V = _np64(b.U), _np64(b.sigma), _np64(b.V)
                data = np.concatenate([U.ravel(order="F"), s.ravel(), V.ravel(order="F")])
                kind, rank = 1, len(s)
            elif isinstance(b, BarycentricMatrix2D):
                U, F, V = _np64(b.U), _np64(b.F), _np64(b.V)
                data = np.concatenate([U.ravel(order="F"), F.ravel(order="F"), V.ravel(order="F")])
                kind, rank = 2, F.shape[0]
            else:
                data = _dense(b).ravel(order="F")
                kind, rank = 0, 0
            sh = _shape(b)
            kinds.append(kind); r0.append(p); rr.append(sh[0]); c0.append(q); cc.append(sh[1]); rk.append(rank)
            offs.append(off); vals.append(data); off += len(data)
        values = np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1))
        arr = lambda v, t=np.int64: np.ascontiguousarray(np.array(v, dtype=t))   # noqa: E731
        kinds_a, r0a, rra, c0a, cca, rka, offa = arr(kinds, np.int32), arr(r0), arr(rr), arr(c0), arr(cc), arr(rk), arr(offs)
        m, n = self.shape
        h = _vp()
        check(lib.hm_hier_build(_lib.HM_F64 if dtype == np.float64 else _lib.HM_F32, m, n, len(kinds),
                                kinds_a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), r0a.ctypes.data_as(_pi64),
                                rra.ctypes.data_as(_pi64), c0a.ctypes.data_as(_pi64), cca.ctypes.data_as(_pi64),
                                rka.ctypes.data_as(_pi64), _lib.f64_ptr(values), offa.ctypes.data_as(_pi64), None,
                                ctypes.byref(h)))
        self._handle, self._handle_dtype = h, dtype
        return h

    def mul(self, y, x, istart=1, jstart=1, incx=1, incy=1, *, stream=None):
        """mul!(y, H, x, istart, jstart, INCX, INCY) on device vectors (accumulates)."""
        from .kernelmatrix import _stream_ptr
        h = self.handle(_np_dtype(y))
        check(lib.hm_mul_strided(h, x.data_ptr(), x.numel(), jstart, incx, y.data_ptr(), y.numel(), istart, incy,
                                 _stream_ptr(stream)))
        return y

    def __matmul__(self, x):
        import torch
        from .kernelmatrix import _stream_ptr
        h = self.handle(_np_dtype(x))
        if x.dim() == 1:
            y = torch.zeros(self.shape[0], dtype=x.dtype, device=x.device)
            return self.mul(y, x.contiguous())
        X = x if x.stride(0) == 1 else x.t().contiguous().t()
        Y = torch.zeros((x.shape[1], self.shape[0]), dtype=x.dtype, device=x.device).t()
        check(lib.hm_mul(h, X.data_ptr(), max(X.stride(1), self.shape[1]), Y.data_ptr(), max(Y.stride(1), self.shape[0]),
                         x.shape[1], 1, _stream_ptr(None)))
        return Y

    def __del__(self):
        try:
            self._invalidate()
        except Exception:
            pass


def _np_dtype(t):
    import torch
    return np.float64 if t.dtype == torch.float64 else np.float32


def _shape(b):
    if isinstance(b, AbstractHierarchical):
        return b.shape
    return tuple(int(v) for v in b.shape)


def _dense(b):
    if isinstance(b, (LowRankMatrix, BarycentricMatrix2D)):
        return b.dense()
    return _np64(b)


_TYPE_NAMES = {"LowRankMatrix": LowRankMatrix, "BarycentricMatrix2D": BarycentricMatrix2D, "Matrix": None}


def _isa(A, T):
    if isinstance(T, tuple):              # parametric member, e.g. ("UpperTriangular", "LowRankMatrix")
        return isinstance(A, tuple) and len(A) == 2 and A[0] == T[0] and _isa(A[1], T[1])
    if T is None or T == "Matrix":
        return _is_dense(A)
    if isinstance(T, str):
        T = _TYPE_NAMES.get(T, T)
        if isinstance(T, str):
            return type(A).__name__ == T
    return isinstance(A, T)


def _is_dense(A):
    if isinstance(A, np.ndarray):
        return A.ndim == 2
    try:
        import torch
        return isinstance(A, torch.Tensor) and A.dim() == 2
    except ImportError:
        return False


def hierarchical(name, *types):
    """The @hierarchical macro (src/hierarchical.jl:4-232): a class named
    ``name`` whose blocks are itself or one of ``types`` (a class, a type name
    such as "Matrix" or "LowRankMatrix", or a parametric pair such as
    ("UpperTriangular", "LowRankMatrix")).  Block stores are named
    ``<Type>blocks`` like the generated Julia fields."""

    def store(T):
        if isinstance(T, tuple):
            return f"{T[0]}blocks"
        return f"{T if isinstance(T, str) else T.__name__}blocks"

    stores = (f"{name}blocks",) + tuple(store(T) for T in types)
    cls = type(name, (AbstractHierarchical,), {"_types": tuple(types), "_store_names": stores,
                                                "block_types": tuple(types)})
    return cls


HierarchicalMatrix = hierarchical("HierarchicalMatrix", LowRankMatrix, "Matrix")


# --------------------------------------------------------------------- mul!

def _strided_args(t):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dim() != 1 or not t.is_contiguous():
        raise TypeError("vectors must be contiguous 1-D CUDA tensors")
    return t.data_ptr(), t.numel()


def mul_(y, A, x, istart=1, jstart=1, incx=1, incy=1, *, stream=None):
    """mul!(y, A, x, istart, jstart[, INCX, INCY]): y[istart + (i-1) INCY] += (A x)[i]
    with x read at x[jstart + (j-1) INCX] (1-based, as in src/algebra.jl:26-30).
    Accumulates into y.  A: dense CUDA matrix, Transpose/Adjoint of one,
    LowRankMatrix (or its Adjoint), BarycentricMatrix2D, a hierarchical matrix
    or a KernelMatrix."""
    import torch
    from .kernelmatrix import KernelMatrix, _stream_ptr
    sp = _stream_ptr(stream)
    if isinstance(A, AbstractHierarchical):
        return A.mul(y, x, istart, jstart, incx, incy, stream=stream)
    if isinstance(A, KernelMatrix):
        if istart == jstart == incx == incy == 1 and y.numel() == A.shape[0] and x.numel() == A.shape[1]:
            return A.mul(y, x, accumulate=True, stream=stream)
        return A.mul_strided(y, x, istart, jstart, incx, incy, stream=stream)
    yp, ly = _strided_args(y)
    xp, lx = _strided_args(x)
    dt = _lib.HM_F64 if y.dtype == torch.float64 else _lib.HM_F32
    trans = isinstance(A, (Transpose, Adjoint))
    B = A.parent if trans else A
    if isinstance(B, LowRankMatrix):
        U, s, V = B.U, B.sigma, B.V
        m, n, r = U.shape[0], V.shape[0], s.shape[0]
        check(lib.hm_lowrank_mul(1 if trans else 0, dt, _colmajor(U).data_ptr(), s.contiguous().data_ptr(), 1,
                                 _colmajor(V).data_ptr(), m, n, r, xp, lx, jstart, incx, yp, ly, istart, incy, sp))
        return y
    if isinstance(B, EvenBarycentricMatrix):
        if trans:
            raise TypeError("the reference defines no transposed EvenBarycentricMatrix product")
        m, p = B.shape
        ishift, jshift = istart - 1, jstart - 1
        for pi in (0, 1):                              # 0-based row parity
            pj = pi if (ishift + jshift) % 2 == 0 else 1 - pi
            mu, nv = B.U[pi].shape[0], B.V[pj].shape[0]
            if mu == 0 or nv == 0:
                continue
            check(lib.hm_lowrank_mul(0, dt, B.U[pi].data_ptr(), B.ones.data_ptr(), 1, B.V[pj].data_ptr(),
                                     mu, nv, B.n, xp, lx, jstart + pj * incx, 2 * incx, yp, ly,
                                     istart + pi * incy, 2 * incy, sp))
        return y
    if isinstance(B, BarycentricMatrix2D):
        m, n = B.shape
        check(lib.hm_lowrank_mul(1 if trans else 0, dt, _colmajor(B.U).data_ptr(), _colmajor(B.F).data_ptr(), 0,
                                 _colmajor(B.V).data_ptr(), m, n, B.rank(), xp, lx, jstart, incx, yp, ly, istart,
                                 incy, sp))
        return y
    M = _colmajor(B)
    check(lib.hm_dense_mul(1 if trans else 0, dt, M.data_ptr(), M.shape[0], M.shape[1], max(M.stride(1), M.shape[0]),
                           xp, lx, jstart, incx, yp, ly, istart, incy, sp))
    return y


def _colmajor(t):
    """A column-major (stride(0) == 1) view or copy of a 2-D CUDA tensor."""
    if t.dim() == 1:
        return t.contiguous()
    if t.stride(0) == 1 and t.stride(1) >= t.shape[0]:
        return t
    return t.t().contiguous().t()
