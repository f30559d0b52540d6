"""ctypes binding of libhmgpu.so (the C ABI declared in include/hmgpu.h).

The library is built in-tree by ``csrc/build.py``; importing this module never
falls back to anything else: a missing library raises ``ImportError`` with
the build command.
"""
import ctypes
import os

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "lib", "libhmgpu.so")

HM_OK = 0
HM_ERR_INVALID_ARG = 1
HM_ERR_UNSORTED = 2
HM_ERR_BOUNDS = 3
HM_ERR_NAN = 4
HM_ERR_CUDA = 5
HM_ERR_ALLOC = 6
HM_ERR_UNSUPPORTED = 7
HM_ERR_BOX = 8
HM_ERR_DEGENERATE = 9
HM_ERR_NOT_POSDEF = 10
HM_LR_KMAX = 96
HM_SOLVE_TRSM, HM_SOLVE_LR, HM_SOLVE_DENSE, HM_SOLVE_INV, HM_SOLVE_LTRSM = 0, 1, 2, 3, 4

HM_KERNEL_CAUCHY, HM_KERNEL_COULOMB, HM_KERNEL_COULOMB_PRIME, HM_KERNEL_LOG = 0, 1, 2, 3
HM_F64, HM_F32, HM_DF64 = 0, 1, 2
HM_OPT_OVERLAP = 1
HM_OPT_NEAR_STAGES = 2
HM_OPT_TENSOR_CORES = 3
HM_OPT_NEAR_KERNEL = 4
HM_OPT_AUTOTUNED = 5
HM_OPT_PDL = 6
HM_OPT_WAIT_LIMIT_NS = 7
HM_OPT_TEST_STALL = 8
HM_OPT_WIDE_TREE = 9
HM_OPT_RING_TILE = 10
HM_DEV_WAIT_TIMEOUT = 1
HM_PIECE_COEF, HM_PIECE_X, HM_PIECE_TCOEF = 0, 1, 2

# Records of csrc/hm_types.h.
VPANEL = np.dtype([("row0", "<i8"), ("off", "<i8"), ("nrows", "<i4"), ("ld", "<i4"),
                   ("width", "<i4"), ("slot", "<i4"), ("col0", "<i4"), ("pad", "<i4")])
XFER = np.dtype([("slot", "<i4"), ("c0", "<i4"), ("c1", "<i4"), ("pad", "<i4")])
STEP = np.dtype([("e0", "<i4"), ("e1", "<i4")])
TASK = np.dtype([("step0", "<i4"), ("step1", "<i4")])
M2L_ROW = np.dtype([("slot", "<i4"), ("begin", "<i4"), ("end", "<i4"), ("pad", "<i4")])
M2L_ENT = np.dtype([("foff", "<i8"), ("yslot", "<i4"), ("pad", "<i4")])
SEG = np.dtype([("row0", "<i8"), ("poff", "<i8"), ("nrows", "<i4"), ("ld", "<i4"), ("width", "<i4"),
                ("piece0", "<i4"), ("npieces", "<i4"), ("nfar", "<i4")])
PIECE = np.dtype([("src", "<i8"), ("kind", "<i4"), ("width", "<i4")])
FILL_VPANEL = np.dtype([("a", "<f8"), ("b", "<f8")])
FILL_F = np.dtype([("xa", "<f8"), ("xb", "<f8"), ("ya", "<f8"), ("yb", "<f8")])
FILL_SEG = np.dtype([("a", "<f8"), ("b", "<f8"), ("has_basis", "<i4"), ("basis_w", "<i4")])
PLAN_TABLES = {
    "vpanels": (0, VPANEL), "vpanel_fill": (1, FILL_VPANEL), "up": (2, XFER),
    "up_level_ptr": (3, np.dtype("<i4")), "m2l_rows": (4, M2L_ROW), "m2l_ents": (5, M2L_ENT),
    "f_fill": (6, FILL_F), "down": (7, XFER), "down_level_ptr": (8, np.dtype("<i4")),
    "segs": (9, SEG), "pieces": (10, PIECE), "seg_fill": (11, FILL_SEG),
    "T": (12, np.dtype("<f8")), "cheb": (13, np.dtype("<f8")), "lam": (14, np.dtype("<f8")),
    "up_ents": (15, XFER), "up_steps": (16, STEP), "up_tasks": (17, TASK),
    "up_band_ptr": (18, np.dtype("<i4")), "down_ents": (19, XFER), "down_steps": (20, STEP),
    "down_tasks": (21, TASK), "down_band_ptr": (22, np.dtype("<i4")),
}
PLAN_SIZES = ("r", "nx", "ny", "n_xslots", "n_yslots", "vstore", "fstore", "pstore", "max_width",
              "n_bary", "n_dense", "depth", "canonical_values", "reference_values", "stored_values",
              "dense_values", "n_segments")
STATS = ("n_bary", "n_dense", "depth", "n_xslots", "n_yslots", "canonical_values",
         "reference_values", "stored_values", "dense_values", "n_segments", "max_width",
         "device_bytes", "launches_per_mul")
STAGES = ("up", "down", "expand", "far", "product")

EXPORTED = (
    "hm_status_string", "hm_last_error", "hm_version", "hm_blockrank", "hm_indsplit",
    "hm_kernelmatrix_build", "hm_kernelmatrix_batch_build", "hm_mul_t", "hm_mul_drow", "hm_size", "hm_storage", "hm_stats", "hm_device_status", "hm_chebyshev", "hm_mul", "hm_mul_strided",
    "hm_mul_host", "hm_mul_noalloc", "hm_debug_fail_alloc", "hm_direct_rows", "hm_configure", "hm_autotune", "hm_autotune_choice", "hm_profile", "hm_profile_read", "hm_profile_timeline", "hm_free", "hm_plan_create", "hm_plan_table", "hm_plan_sizes",
    "hm_plan_free", "hm_batch_plan_create", "hm_hier_build", "hm_dense_mul", "hm_lowrank_mul",
    "hm_bary_factors", "hm_lr_svd", "hm_gemm_batched", "hm_axpby_batched", "hm_potrf_batched",
    "hm_solve_transposed", "hm_potrf_batched_async", "hm_trtri_batched", "hm_hchol_factor", "hm_hchol_result",
    "hm_hchol_free",
)

_d = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64
_pi64 = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


_c64 = ctypes.c_int64
_c32 = ctypes.c_int32


class LrProblem(ctypes.Structure):
    """hm_lr_problem of include/hmgpu.h."""
    _fields_ = [("m", _c64), ("n", _c64), ("t", _c64), ("a1", _c32), ("a2", _c32), ("b1", _c32), ("b2", _c32),
                ("qr_left", _c32), ("qr_right", _c32), ("P1", _vp), ("P2", _vp), ("Q1", _vp), ("Q2", _vp),
                ("ldp1", _c64), ("ldp2", _c64), ("ldq1", _c64), ("ldq2", _c64), ("s1", _vp), ("s2", _vp),
                ("sign2", ctypes.c_double), ("Xm", _vp), ("Ym", _vp), ("ldx", _c64), ("ldy", _c64),
                ("U", _vp), ("s", _vp), ("V", _vp)]


class GemmProblem(ctypes.Structure):
    """hm_gemm_problem of include/hmgpu.h."""
    _fields_ = [("m", _c64), ("n", _c64), ("k", _c64), ("P", _vp), ("ldp", _c64), ("transp", _c32),
                ("Q", _vp), ("ldq", _c64), ("transq", _c32), ("s", _vp), ("alpha", ctypes.c_double),
                ("beta", ctypes.c_double), ("C", _vp), ("ldc", _c64), ("D", _vp), ("ldd", _c64)]


class AxpbyProblem(ctypes.Structure):
    """hm_axpby_problem of include/hmgpu.h."""
    _fields_ = [("m", _c64), ("n", _c64), ("A", _vp), ("lda", _c64), ("B", _vp), ("ldb", _c64),
                ("dr", _vp), ("dc", _vp), ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("D", _vp), ("ldd", _c64)]


class PotrfProblem(ctypes.Structure):
    """hm_potrf_problem of include/hmgpu.h."""
    _fields_ = [("n", _c64), ("A", _vp), ("lda", _c64), ("R", _vp), ("ldr", _c64)]


class TrtriProblem(ctypes.Structure):
    """hm_trtri_problem of include/hmgpu.h."""
    _fields_ = [("n", _c64), ("R", _vp), ("ldr", _c64), ("W", _vp), ("ldw", _c64)]


class SolveOp(ctypes.Structure):
    """hm_solve_op of include/hmgpu.h."""
    _fields_ = [("kind", _c32), ("r", _c32), ("o1", _c64), ("n1", _c64), ("o2", _c64), ("n2", _c64),
                ("ld", _c64), ("ld2", _c64), ("A", _vp), ("s", _vp), ("B", _vp)]


class HcholNode(ctypes.Structure):
    """hm_hchol_node of include/hmgpu.h."""
    _fields_ = [("n", _c64), ("n1", _c64), ("left", _c32), ("right", _c32), ("D", _vp), ("ldd", _c64),
                ("U", _vp), ("ldu", _c64), ("s", _vp), ("V", _vp), ("ldv", _c64), ("r", _c32)]


class HcholOut(ctypes.Structure):
    """hm_hchol_out of include/hmgpu.h."""
    _fields_ = [("r", _c32), ("U", _vp), ("ldu", _c64), ("s", _vp), ("V", _vp), ("ldv", _c64),
                ("R", _vp), ("ldr", _c64), ("W", _vp), ("ldw", _c64)]


class HMError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class DeviceWaitTimeout(RuntimeError):
    """A kernel gave up a bounded wait (device status HM_DEV_WAIT_TIMEOUT)."""


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python hierarchicalmatrices.jl_gb300/csrc/build.py` (no CPU fallback exists)")
    L = ctypes.CDLL(LIB_PATH)
    L.hm_status_string.restype = ctypes.c_char_p
    L.hm_status_string.argtypes = [ctypes.c_int]
    L.hm_last_error.restype = ctypes.c_char_p
    L.hm_last_error.argtypes = []
    L.hm_version.restype = ctypes.c_int
    L.hm_blockrank.restype = ctypes.c_int
    L.hm_blockrank.argtypes = [ctypes.c_double]
    L.hm_indsplit.restype = ctypes.c_int
    L.hm_indsplit.argtypes = [_d, _i64, _i64, _i64, ctypes.c_double, ctypes.c_double, _pi64]
    L.hm_kernelmatrix_build.restype = ctypes.c_int
    L.hm_kernelmatrix_build.argtypes = [ctypes.c_int, _d, _i64, _d, _i64, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, _i64, ctypes.c_int, _vp,
                                        ctypes.POINTER(_vp)]
    L.hm_kernelmatrix_batch_build.restype = ctypes.c_int
    L.hm_kernelmatrix_batch_build.argtypes = [ctypes.c_int, ctypes.c_int, _pi64, _pi64, _d, _d, _d,
                                              ctypes.c_int, _i64, ctypes.c_int, _vp, ctypes.POINTER(_vp)]
    L.hm_batch_plan_create.restype = ctypes.c_int
    L.hm_batch_plan_create.argtypes = [ctypes.c_int, _pi64, _pi64, _d, _d, _d, ctypes.c_int, _i64,
                                       ctypes.POINTER(_vp)]
    L.hm_hier_build.restype = ctypes.c_int
    L.hm_hier_build.argtypes = [ctypes.c_int, _i64, _i64, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), _pi64,
                                _pi64, _pi64, _pi64, _pi64, _d, _pi64, _vp, ctypes.POINTER(_vp)]
    L.hm_dense_mul.restype = ctypes.c_int
    L.hm_dense_mul.argtypes = [ctypes.c_int, ctypes.c_int, _vp, _i64, _i64, _i64, _vp, _i64, _i64, _i64, _vp,
                               _i64, _i64, _i64, _vp]
    L.hm_lowrank_mul.restype = ctypes.c_int
    L.hm_lowrank_mul.argtypes = [ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _i64, _i64, _i64, _vp,
                                 _i64, _i64, _i64, _vp, _i64, _i64, _i64, _vp]
    L.hm_bary_factors.restype = ctypes.c_int
    L.hm_bary_factors.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double, _d, _i64, _d, _i64, ctypes.c_int, _vp, _vp, _vp, _vp]
    L.hm_lr_svd.restype = ctypes.c_int
    L.hm_lr_svd.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(LrProblem), ctypes.POINTER(ctypes.c_int32), _vp]
    L.hm_gemm_batched.restype = ctypes.c_int
    L.hm_gemm_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(GemmProblem), _vp]
    L.hm_axpby_batched.restype = ctypes.c_int
    L.hm_axpby_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(AxpbyProblem), _vp]
    L.hm_potrf_batched.restype = ctypes.c_int
    L.hm_potrf_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(PotrfProblem),
                                   ctypes.POINTER(ctypes.c_int32), _vp]
    L.hm_potrf_batched_async.restype = ctypes.c_int
    L.hm_potrf_batched_async.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(PotrfProblem), _vp, _vp]
    L.hm_trtri_batched.restype = ctypes.c_int
    L.hm_trtri_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(TrtriProblem), _vp]
    L.hm_solve_transposed.restype = ctypes.c_int
    L.hm_solve_transposed.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(SolveOp), _vp, _i64, _i64, _vp]
    L.hm_hchol_factor.restype = ctypes.c_int
    L.hm_hchol_factor.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(HcholNode), ctypes.c_int32,
                                  ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int32), _vp]
    L.hm_hchol_result.restype = ctypes.c_int
    L.hm_hchol_result.argtypes = [_vp, ctypes.c_int32, ctypes.POINTER(HcholOut)]
    L.hm_hchol_free.restype = ctypes.c_int
    L.hm_hchol_free.argtypes = [_vp]
    L.hm_size.restype = ctypes.c_int
    L.hm_size.argtypes = [_vp, _pi64, _pi64]
    L.hm_storage.restype = ctypes.c_int
    L.hm_storage.argtypes = [_vp]
    L.hm_stats.restype = ctypes.c_int
    L.hm_stats.argtypes = [_vp, _pi64, ctypes.c_int]
    L.hm_device_status.restype = ctypes.c_int
    L.hm_device_status.argtypes = [_vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    L.hm_chebyshev.restype = ctypes.c_int
    L.hm_chebyshev.argtypes = [ctypes.c_int, _d, _d]
    L.hm_mul.restype = ctypes.c_int
    L.hm_mul.argtypes = [_vp, _vp, _i64, _vp, _i64, ctypes.c_int, ctypes.c_int, _vp]
    L.hm_mul_t.restype = ctypes.c_int
    L.hm_mul_t.argtypes = [_vp, _vp, _i64, _vp, _i64, ctypes.c_int, ctypes.c_int, _vp]
    L.hm_mul_drow.restype = ctypes.c_int
    L.hm_mul_drow.argtypes = [_vp, ctypes.c_int, _vp, _i64, _vp, _i64, ctypes.c_int, ctypes.c_int, _vp]
    L.hm_mul_strided.restype = ctypes.c_int
    L.hm_mul_strided.argtypes = [_vp, _vp, _i64, _i64, _i64, _vp, _i64, _i64, _i64, _vp]
    L.hm_mul_host.restype = ctypes.c_int
    L.hm_mul_host.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int]
    L.hm_mul_noalloc.restype = ctypes.c_int
    L.hm_mul_noalloc.argtypes = [_vp, _vp, _vp, ctypes.c_int, _vp]
    L.hm_autotune_choice.restype = ctypes.c_int
    L.hm_autotune_choice.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.c_int]
    L.hm_debug_fail_alloc.restype = ctypes.c_int
    L.hm_debug_fail_alloc.argtypes = [_i64]
    L.hm_direct_rows.restype = ctypes.c_int
    L.hm_direct_rows.argtypes = [_vp, _vp, _vp, _i64, _vp, _vp]
    L.hm_configure.restype = ctypes.c_int
    L.hm_configure.argtypes = [_vp, ctypes.c_int, _i64]
    L.hm_autotune.restype = ctypes.c_int
    L.hm_autotune.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.POINTER(ctypes.c_int32),
                              ctypes.POINTER(ctypes.c_double)]
    L.hm_profile_timeline.restype = ctypes.c_int
    L.hm_profile_timeline.argtypes = [_vp, _vp, ctypes.c_int]
    L.hm_profile.restype = ctypes.c_int
    L.hm_profile.argtypes = [_vp, ctypes.c_int]
    L.hm_profile_read.restype = ctypes.c_int
    L.hm_profile_read.argtypes = [_vp, _d, _pi64, ctypes.c_int, ctypes.c_int]
    L.hm_free.restype = None
    L.hm_free.argtypes = [_vp]
    L.hm_plan_create.restype = ctypes.c_int
    L.hm_plan_create.argtypes = [_d, _i64, _d, _i64, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, _i64,
                                 ctypes.POINTER(_vp)]
    L.hm_plan_table.restype = ctypes.c_int
    L.hm_plan_table.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(_vp), _pi64, _pi64]
    L.hm_plan_sizes.restype = ctypes.c_int
    L.hm_plan_sizes.argtypes = [_vp, _pi64, ctypes.c_int]
    L.hm_plan_free.restype = None
    L.hm_plan_free.argtypes = [_vp]
    return L


lib = _load()


def check(status):
    """Raise HMError for a non-zero status (IndexError for HM_ERR_BOUNDS, as the
    reference raises BoundsError)."""
    if status == HM_OK:
        return
    msg = lib.hm_last_error().decode() or lib.hm_status_string(status).decode()
    text = f"{lib.hm_status_string(status).decode()}: {msg}"
    if status == HM_ERR_BOUNDS:
        raise IndexError(text)
    raise HMError(status, text)


def f64_ptr(a):
    return a.ctypes.data_as(_d)


class Plan:
    """Host-side plan (block tree + flattened tables) without a GPU."""

    def __init__(self, x, y, a, b, c, d, rank=20, blocksize=0, _handle=None):
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        h = _vp()
        if _handle is None:
            check(lib.hm_plan_create(f64_ptr(self.x), len(self.x), f64_ptr(self.y), len(self.y),
                                     a, b, c, d, rank, blocksize, ctypes.byref(h)))
        else:
            h = _handle
        self._h = h
        out = np.zeros(len(PLAN_SIZES), dtype=np.int64)
        n = lib.hm_plan_sizes(self._h, out.ctypes.data_as(_pi64), len(out))
        self.sizes = dict(zip(PLAN_SIZES[:n], (int(v) for v in out[:n])))

    def table(self, name):
        which, dt = PLAN_TABLES[name]
        data, count, es = _vp(), _i64(), _i64()
        check(lib.hm_plan_table(self._h, which, ctypes.byref(data), ctypes.byref(count),
                                ctypes.byref(es)))
        assert es.value == dt.itemsize, (name, es.value, dt.itemsize)
        if count.value == 0:
            return np.zeros(0, dtype=dt)
        buf = (ctypes.c_char * (count.value * es.value)).from_address(data.value)
        return np.frombuffer(bytes(buf), dtype=dt).copy()

    def __del__(self):
        if getattr(self, "_h", None):
            lib.hm_plan_free(self._h)
            self._h = None


def batch_plan(xs, ys, boxes, rank=20, blocksize=0):
    """Merged host plan of many instances (see hm_batch_plan_create)."""
    nx = np.array([len(v) for v in xs], dtype=np.int64)
    ny = np.array([len(v) for v in ys], dtype=np.int64)
    x = np.ascontiguousarray(np.concatenate(xs), dtype=np.float64)
    y = np.ascontiguousarray(np.concatenate(ys), dtype=np.float64)
    bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 4))
    h = _vp()
    check(lib.hm_batch_plan_create(len(xs), nx.ctypes.data_as(_pi64), ny.ctypes.data_as(_pi64),
                                   f64_ptr(x), f64_ptr(y), f64_ptr(bx), rank, blocksize, ctypes.byref(h)))
    return Plan(x, y, 0, 0, 0, 0, _handle=h)


def chebyshev(n):
    """First-kind Chebyshev nodes and barycentric weights in FP64, as the
    library builds them (src/BarycentricMatrix.jl:92-136)."""
    x, lam = np.zeros(n), np.zeros(n)
    check(lib.hm_chebyshev(int(n), f64_ptr(x), f64_ptr(lam)))
    return x, lam
