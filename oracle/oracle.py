"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates HierarchicalMatrices.jl v0.2.2 on the CPU (see
hm_oracle.c for the file:line of each reference function).  Only tests,
``__graft_entry__.smoke`` and the CPU-baseline leg of ``bench.py`` import this
module; the product never does.

Besides the C library this module holds a small pure-Python restatement of the
generic ``HierarchicalMatrix`` block walk (src/HierarchicalMatrix.jl:24-52) for
user-assembled trees, used on small cases only.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

CAUCHY, COULOMB, COULOMB_PRIME, LOG = 0, 1, 2, 3
TAG_KMAT, TAG_BARY, TAG_DENSE = 1, 2, 3

_d = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64
_pi64 = ctypes.POINTER(ctypes.c_int64)


def build():
    """Compile hm_oracle.c into oracle/_build/liboracle.so."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "hm_oracle.c"))
        ):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.or_blockrank.restype = ctypes.c_int
        L.or_blockrank.argtypes = [ctypes.c_double]
        L.or_chebyshevpoints.argtypes = [ctypes.c_int, ctypes.c_int, _d]
        L.or_chebyshevweights.argtypes = [ctypes.c_int, ctypes.c_int, _d]
        L.or_kernel_eval.restype = ctypes.c_double
        L.or_kernel_eval.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.or_indsplit_api.restype = ctypes.c_int
        L.or_indsplit_api.argtypes = [_d, _i64, _i64, _i64, ctypes.c_double, ctypes.c_double, _pi64]
        L.or_kernelmatrix.restype = ctypes.c_int
        L.or_kernelmatrix.argtypes = [ctypes.c_int, _d, _i64, _d, _i64, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, _i64, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_void_p)]
        L.or_free.argtypes = [ctypes.c_void_p]
        L.or_kernelmatrix_mul.restype = ctypes.c_int
        L.or_kernelmatrix_mul.argtypes = [ctypes.c_void_p, _d, _i64, _d, _i64, ctypes.c_int]
        L.or_kernelmatrix_size.argtypes = [ctypes.c_void_p, _pi64]
        L.or_kernelmatrix_stats.argtypes = [ctypes.c_void_p, _pi64]
        L.or_kernelmatrix_leaves.restype = _i64
        L.or_kernelmatrix_leaves.argtypes = [ctypes.c_void_p, _i64, _pi64, _d]
        L.or_kernelmatrix_block_data.restype = ctypes.c_int
        L.or_kernelmatrix_block_data.argtypes = [ctypes.c_void_p, _i64, ctypes.c_int, _d]
        for name in ("or_dense_mul", "or_dense_mul_t"):
            f = getattr(L, name)
            f.argtypes = [_d, _d, _i64, _i64, _d, _i64, _i64, _i64, _i64]
        for name in ("or_lowrank_mul", "or_lowrank_mul_t"):
            f = getattr(L, name)
            f.argtypes = [_d, _d, _d, _d, _i64, _i64, _i64, _d, _i64, _i64, _i64, _i64]
        L.or_dense_rows.argtypes = [ctypes.c_int, _d, _d, _i64, _d, _pi64, _i64, _d, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_d)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def blockrank(eps):
    return lib().or_blockrank(float(eps))


def chebyshevpoints(n, kind=1):
    out = np.zeros(n)
    lib().or_chebyshevpoints(n, kind, _ptr(out))
    return out


def chebyshevbarycentricweights(n, kind=1):
    out = np.zeros(n)
    lib().or_chebyshevweights(n, kind, _ptr(out))
    return out


def kernel_eval(kernel, x, y):
    return lib().or_kernel_eval(kernel, float(x), float(y))


def indsplit(x, start, length, a, b):
    """Returns ((s1, l1), (s2, l2)) with 0-based starts; raises IndexError like
    the reference's BoundsError."""
    x = _f64(x)
    out = np.zeros(4, dtype=np.int64)
    st = lib().or_indsplit_api(_ptr(x), len(x), start, length, a, b, out.ctypes.data_as(_pi64))
    if st == 1:
        raise IndexError("indsplit read past the end of the point list")
    return (int(out[0]), int(out[1])), (int(out[2]), int(out[3]))


class OracleKernelMatrix:
    """The reference's KernelMatrix built and multiplied on the CPU."""

    def __init__(self, kernel, x, y, a, b, c, d, rank=20, blocksize=None, nthreads=1):
        self.x = _f64(x)
        self.y = _f64(y)
        if blocksize is None:
            blocksize = 4 * rank
        h = ctypes.c_void_p()
        st = lib().or_kernelmatrix(kernel, _ptr(self.x), len(self.x), _ptr(self.y), len(self.y),
                                   a, b, c, d, rank, blocksize, nthreads, ctypes.byref(h))
        if st == 1:
            raise IndexError("KernelMatrix: indsplit read past the end of the point list")
        if st != 0:
            raise RuntimeError(f"oracle KernelMatrix failed with status {st}")
        self._h = h
        self.rank = rank
        mn = np.zeros(2, dtype=np.int64)
        lib().or_kernelmatrix_size(self._h, mn.ctypes.data_as(_pi64))
        self.shape = (int(mn[0]), int(mn[1]))

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.or_free(self._h)
            self._h = None

    def mul(self, u, v, nthreads=1):
        """u += H v in the reference's order (u, v float64 arrays)."""
        assert u.dtype == np.float64 and v.dtype == np.float64
        st = lib().or_kernelmatrix_mul(self._h, _ptr(u), len(u), _ptr(_f64(v)), len(v), nthreads)
        if st:
            raise IndexError("mul!: vector too short")
        return u

    def __matmul__(self, v):
        u = np.zeros(self.shape[0])
        return self.mul(u, _f64(v))

    def stats(self):
        st = np.zeros(6, dtype=np.int64)
        lib().or_kernelmatrix_stats(self._h, st.ctypes.data_as(_pi64))
        keys = ("bary", "dense", "depth", "bary_rows_cols", "dense_values", "stored_values")
        return dict(zip(keys, (int(v) for v in st)))

    def leaves(self):
        n = lib().or_kernelmatrix_leaves(self._h, 0, None, None)
        meta = np.zeros((n, 6), dtype=np.int64)
        box = np.zeros((n, 4))
        lib().or_kernelmatrix_leaves(self._h, n, meta.ctypes.data_as(_pi64), _ptr(box))
        return meta, box

    def block_data(self, idx, which, shape):
        out = np.zeros(shape[0] * shape[1])
        st = lib().or_kernelmatrix_block_data(self._h, idx, which, _ptr(out))
        if st:
            raise ValueError("no such factor")
        return out.reshape(shape[1], shape[0]).T  # column-major


def dense_mul(y, A, x, istart, jstart, incx=1, incy=1, trans=False):
    """mul!(y, A, x, istart, jstart, INCX, INCY), src/algebra.jl:37-65 (1-based)."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    f = lib().or_dense_mul_t if trans else lib().or_dense_mul
    f(_ptr(y), A.ctypes.data_as(_d), m, n, _ptr(x), istart, jstart, incx, incy)
    return y


def lowrank_mul(y, U, sigma, V, x, istart, jstart, incx=1, incy=1, adjoint=False):
    """mul!(y, L, x, ...) / mul!(y, L', x, ...), src/algebra.jl:110-159."""
    U = np.asfortranarray(U, dtype=np.float64)
    V = np.asfortranarray(V, dtype=np.float64)
    sigma = _f64(sigma)
    m, r = U.shape
    n = V.shape[0]
    f = lib().or_lowrank_mul_t if adjoint else lib().or_lowrank_mul
    f(_ptr(y), U.ctypes.data_as(_d), _ptr(sigma), V.ctypes.data_as(_d), m, n, r, _ptr(x),
      istart, jstart, incx, incy)
    return y


def dense_rows(kernel, x, y, b, rows, nthreads=1):
    """FP64 dense kernel rows sum_j f(x_i, y_j) b_j with compensated summation."""
    x, y, b = _f64(x), _f64(y), _f64(b)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    out = np.zeros(len(rows))
    lib().or_dense_rows(kernel, _ptr(x), _ptr(y), len(y), _ptr(b), rows.ctypes.data_as(_pi64),
                        len(rows), _ptr(out), nthreads)
    return out


def kernel_dense(kernel, x, y):
    """The dense kernel matrix, evaluated like the reference's examples/Kernel.jl:39-41."""
    x = _f64(x)[:, None]
    y = _f64(y)[None, :]
    d = x - y
    if kernel == CAUCHY:
        return 1.0 / d
    if kernel == COULOMB:
        return 1.0 / (d * d)
    if kernel == COULOMB_PRIME:
        return 1.0 / ((d * d) * d)
    return np.log(np.abs(d))


# --- generic HierarchicalMatrix walk (pure Python; small cases only) --------

class PyLowRank:
    def __init__(self, U, sigma, V):
        self.U = np.asfortranarray(U, dtype=np.float64)
        self.sigma = _f64(sigma)
        self.V = np.asfortranarray(V, dtype=np.float64)
        self.shape = (self.U.shape[0], self.V.shape[0])


class PyHier:
    """Mirror of an @hierarchical HierarchicalMatrix: blocks[m][n] is None
    (unassigned, tag 0), a PyHier, a PyLowRank or a dense numpy matrix."""

    def __init__(self, M, N):
        self.blocks = [[None] * N for _ in range(M)]

    def blocksize(self, m, n, k):
        b = self.blocks[m][n]
        if b is None:
            return 0
        return b.shape[k]

    @property
    def shape(self):
        M, N = len(self.blocks), len(self.blocks[0])
        return (sum(self.blocksize(m, N - 1, 0) for m in range(M)),
                sum(self.blocksize(0, n, 1) for n in range(N)))


def hier_mul(y, H, x, istart=1, jstart=1, incx=1, incy=1):
    """mul!(y, H, x, istart, jstart, INCX, INCY)  src/HierarchicalMatrix.jl:24-52."""
    M, N = len(H.blocks), len(H.blocks[0])
    p = 0
    for m in range(M):
        q = 0
        for n in range(N):
            b = H.blocks[m][n]
            if isinstance(b, PyHier):
                hier_mul(y, b, x, istart + p, jstart + q, incx, incy)
            elif isinstance(b, PyLowRank):
                lowrank_mul(y, b.U, b.sigma, b.V, x, istart + p, jstart + q, incx, incy)
            elif b is not None:
                dense_mul(y, b, x, istart + p, jstart + q, incx, incy)
            q += incx * H.blocksize(0, n, 1)
        p += incy * H.blocksize(m, N - 1, 0)
    return y


def dense_mul_generic(y, A, x, istart, jstart, incx=1, incy=1):
    """Element-type-generic restatement of src/algebra.jl:37-48 for Python
    number objects (e.g. fractions.Fraction), list-of-lists A; 1-based offsets."""
    m, n = len(A), len(A[0])
    ishift, jshift = istart - incy, jstart - incx
    for j in range(1, n + 1):
        xj = x[jshift + j * incx - 1]
        for i in range(1, m + 1):
            y[ishift + i * incy - 1] += A[i - 1][j - 1] * xj
    return y


def dense_mul_t_generic(y, A, x, istart, jstart, incx=1, incy=1):
    """Generic restatement of src/algebra.jl:52-65 (y += transpose(A) x)."""
    m, n = len(A), len(A[0])
    ishift, jshift = istart - incy, jstart - incx
    for i in range(1, n + 1):
        yi = 0
        for j in range(1, m + 1):
            yi += A[j - 1][i - 1] * x[jshift + j * incx - 1]
        y[ishift + i * incy - 1] += yi
    return y


def grid_points(n):
    """Interleaved grid x_i = (i-1)/n + 1/(2n), y_j = (j-1)/n, descending."""
    x = (np.arange(n, dtype=np.float64) / n + 1.0 / (2 * n))[::-1].copy()
    y = (np.arange(n, dtype=np.float64) / n)[::-1].copy()
    return x, y


def example_points(family, n):
    """Point families of examples/Kernel.jl: 'chebyshev' (x first kind, y second
    kind on [1,-1], :44-49) and 'quadratic' (x = i(i+1), y = (i+1/2)(i+3/2),
    descending, :73-78).  Returns x, y, (a, b, c, d)."""
    if family == "chebyshev":
        x = chebyshevpoints(n, 1)
        y = chebyshevpoints(n, 2)
        return x, y, (1.0, -1.0, 1.0, -1.0)
    i = np.arange(n, 0, -1, dtype=np.float64)
    x = i * (i + 1)
    y = (i + 0.5) * (i + 1.5)
    return x, y, (float(x.max()), float(x.min()), float(y.max()), float(y.min()))


def beta_points(n, seed, min_gap=1e-9):
    """x, y i.i.d. Beta(1/2, 1/2), sorted descending, minimum gap enforced."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(2):
        p = np.sort(rng.beta(0.5, 0.5, n))
        for i in range(1, n):
            if p[i] - p[i - 1] < min_gap:
                p[i] = p[i - 1] + min_gap
        out.append(p[::-1].copy())
    return out[0], out[1]


# ------------------------------------------------------------ EvenBarycentricMatrix

def even_bary_factors(f, a, b, c, d, n, T=np.float64):
    """W (n x m) and F (p x n) of EvenBarycentricMatrix(T, f, a, b, c, d) in
    FP64, in the loop order of src/BarycentricMatrix.jl:17-45 (f(T, x, j) is
    the user's kernel on the integer grid)."""
    x = chebyshevpoints(n)
    lam = chebyshevbarycentricweights(n)
    m, p = b - a + 1, d - c + 1
    w = np.zeros(m)
    for ii in range(m):
        i = a + ii
        for k in range(n):
            w[ii] += lam[k] * (1.0 / ((2 * i - a - b) - (b - a) * x[k]))
    W = np.zeros((n, m))
    for ii in range(m):
        i = a + ii
        for k in range(n):
            W[k, ii] = lam[k] * (1.0 / (((2 * i - a - b) - (b - a) * x[k]) * w[ii]))
    F = np.zeros((p, n))
    for k in range(n):
        for jj in range(p):
            F[jj, k] = f(T, (a + b) / 2 + (b - a) * x[k] / 2, c + jj)
    return W, F


def even_bary_mul(u, W, F, v, istart, jstart):
    """mul!(u, B::EvenBarycentricMatrix, v, istart, jstart) in the loop order
    of src/algebra.jl:168-239: rows and columns of matching parity (odd with
    odd, even with even when istart + jstart is even; crossed otherwise)."""
    n, m = W.shape
    p = F.shape[0]
    ishift, jshift = istart - 1, jstart - 1
    # (first 1-based column of the inner sum, first 1-based row it feeds)
    pairs = ((1, 1), (2, 2)) if (ishift + jshift) % 2 == 0 else ((2, 1), (1, 2))
    for jfirst, ifirst in pairs:
        beta = np.zeros(n)
        for k in range(n):
            bk = 0.0
            for j in range(jfirst, p + 1, 2):
                bk += v[jshift + j - 1] * F[j - 1, k]
            beta[k] = bk
        for i in range(ifirst, m + 1, 2):
            ui = 0.0
            for k in range(n):
                ui += beta[k] * W[k, i - 1]
            u[ishift + i - 1] += ui
    return u
