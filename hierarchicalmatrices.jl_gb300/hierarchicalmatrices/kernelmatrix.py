"""KernelMatrix: the reference's compressed kernel matrix, built and applied on the GPU.

Mirrors src/KernelMatrix.jl of HierarchicalMatrices.jl:
  * ``KernelMatrix(f, x, y, a, b, c, d)``   (src/KernelMatrix.jl:47)
  * ``H @ v`` / ``H * v``                   (src/KernelMatrix.jl:5-12)
  * ``mul_(u, H, v, istart, jstart)``       (src/KernelMatrix.jl:14-45; accumulates into u)

Device arrays are torch CUDA tensors; host arrays are numpy arrays (copied to
the GPU and back inside the call).  Every product runs the CUDA kernels of
libhmgpu.so; there is no CPU path.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import DeviceWaitTimeout, check, lib

_vp = ctypes.c_void_p


class _Kernel:
    """A kernel the GPU library knows, callable like the reference's closures."""

    def __init__(self, name, kid, fn):
        self.__name__ = name
        self.hm_id = kid
        self._fn = fn

    def __call__(self, x, y):
        return self._fn(np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64))

    def __repr__(self):
        return self.__name__


# examples/Kernel.jl:34-37
cauchykernel = _Kernel("cauchykernel", _lib.HM_KERNEL_CAUCHY, lambda x, y: 1.0 / (x - y))
coulombkernel = _Kernel("coulombkernel", _lib.HM_KERNEL_COULOMB, lambda x, y: 1.0 / ((x - y) * (x - y)))
coulombprimekernel = _Kernel("coulombprimekernel", _lib.HM_KERNEL_COULOMB_PRIME,
                             lambda x, y: 1.0 / (((x - y) * (x - y)) * (x - y)))
logkernel = _Kernel("logkernel", _lib.HM_KERNEL_LOG, lambda x, y: np.log(np.abs(x - y)))
KERNELS = {k.__name__: k for k in (cauchykernel, coulombkernel, coulombprimekernel, logkernel)}


def _kernel_id(f):
    if isinstance(f, _Kernel):
        return f.hm_id
    if isinstance(f, str) and f in KERNELS:
        return KERNELS[f].hm_id
    if isinstance(f, int) and 0 <= f <= 3:
        return f
    raise ValueError(f"kernel {f!r} is not one of {sorted(KERNELS)}; the GPU library evaluates "
                     "a fixed kernel set")


DF64 = "df64"   # storage: FP64 vectors and tree passes, row-segment panels as double-float pairs


def _storage_of(dtype):
    """(storage code, numpy dtype of the vectors) for a dtype argument:
    np.float64, np.float32 or "df64" (HM_DF64: the FP64 product with its
    panels stored as double-float pairs and multiplied on the FP32 pipes)."""
    if isinstance(dtype, str) and dtype == DF64:
        return _lib.HM_DF64, np.dtype(np.float64)
    dt = np.dtype(dtype)
    if dt == np.float64:
        return _lib.HM_F64, dt
    if dt == np.float32:
        return _lib.HM_F32, dt
    raise ValueError(f"unsupported storage dtype {dt}")


def _host_f64(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            a = a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.ascontiguousarray(a, dtype=np.float64)


def _stream_ptr(stream):
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


def BLOCKRANK(T=np.float64):
    """BLOCKRANK(T) (src/HierarchicalMatrices.jl:5)."""
    return lib.hm_blockrank(float(np.finfo(T).eps))


def BLOCKSIZE(T=np.float64):
    """BLOCKSIZE(T) = 4 BLOCKRANK(T) (src/HierarchicalMatrices.jl:7)."""
    return 4 * BLOCKRANK(T)


def indsplit(x, ir, a, b):
    """indsplit(x, ir, a, b) (src/BarycentricMatrix.jl:299-307) with 0-based
    Python ranges: returns the two halves of ``ir`` split at (a+b)/2."""
    x = _host_f64(x)
    out = np.zeros(4, dtype=np.int64)
    check(lib.hm_indsplit(_lib.f64_ptr(x), len(x), ir.start, len(ir), float(a), float(b),
                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
    return range(out[0], out[0] + out[1]), range(out[2], out[2] + out[3])


class KernelMatrix:
    """KernelMatrix(f, x, y, a, b, c, d) compressed on the GPU.

    ``x``, ``y`` must be in non-increasing order with ``a > b`` and ``c > d``
    (the reference's convention).  ``dtype`` is the storage type of factors,
    leaves and vectors (float64, or float32 from FP64 compression);
    ``rank`` defaults to BLOCKRANK(Float64) = 20 and ``blocksize`` to 4 rank.
    """

    def __init__(self, f, x, y, a, b, c, d, *, dtype=np.float64, rank=None, blocksize=None,
                 stream=None):
        self.kernel = _kernel_id(f)
        self.f = f
        self.x = _host_f64(x)
        self.y = _host_f64(y)
        self.box = (float(a), float(b), float(c), float(d))
        self.storage, self.dtype = _storage_of(dtype)
        self.rank = int(rank) if rank else BLOCKRANK(np.float64)
        self.blocksize = int(blocksize) if blocksize else 4 * self.rank
        h = _vp()
        check(lib.hm_kernelmatrix_build(self.kernel, _lib.f64_ptr(self.x), len(self.x),
                                        _lib.f64_ptr(self.y), len(self.y), *self.box, self.rank,
                                        self.blocksize, self.storage,
                                        _stream_ptr(stream), ctypes.byref(h)))
        self._h = h
        self.shape = (len(self.x), len(self.y))

    # -- reference surface -------------------------------------------------
    def size(self, dim=None):
        return self.shape if dim is None else self.shape[dim - 1]

    def stats(self):
        out = np.zeros(len(_lib.STATS), dtype=np.int64)
        n = lib.hm_stats(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(out))
        return dict(zip(_lib.STATS[:n], (int(v) for v in out[:n])))

    def device_status(self, reset=False):
        """Device-side status word of the streaming kernels: 0 when clean, 1
        when a kernel gave up waiting for a stage copy (synchronises)."""
        code = ctypes.c_int(0)
        check(lib.hm_device_status(self._h, ctypes.byref(code), 1 if reset else 0))
        return code.value

    def check_device(self):
        """Raises DeviceWaitTimeout (and clears the word) when a kernel of
        this handle gave up a bounded wait since the last check: the products
        issued since then are invalid.  Synchronises the device."""
        code = self.device_status(reset=True)
        if code:
            raise DeviceWaitTimeout(
                f"a kernel of this KernelMatrix gave up waiting (device status {code}): its products are invalid")

    def set_wide_tree(self, enable=True):
        """Tree passes on the lane-per-right-hand-side kernels: True (the
        default) from 32 right-hand sides, "all" from 2, False never (the
        kernels for chunks of 8)."""
        code = 2 if enable == "all" else (1 if enable else 0)
        check(lib.hm_configure(self._h, _lib.HM_OPT_WIDE_TREE, code))

    def set_ring_tile(self, tile):
        """Tile of the per-warp rings (3-8 FP32 right-hand sides): 0 = up to
        768 panel values x 3 stages per warp (default), 1 = 512 x 4,
        2 = 1024 x 3."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_RING_TILE, int(tile)))

    def set_wait_limit(self, ns):
        """Nanoseconds (1 .. 2e9, default 2e9) after which a wait of the
        streamed near-field or tensor-core panel kernel gives up."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_WAIT_LIMIT_NS, int(ns)))

    def _set_test_stall(self, enable):
        """Test hook: the first wait of every CTA of those kernels waits on a
        barrier nothing arrives on, so it runs out after the wait limit."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_TEST_STALL, 1 if enable else 0))

    @property
    def handle(self):
        return self._h

    def _check_dev(self, t, rows, name):
        import torch
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise TypeError(f"{name} must be a CUDA tensor")
        if t.dtype != (torch.float64 if self.dtype == np.float64 else torch.float32):
            raise TypeError(f"{name} must have dtype {self.dtype}")
        if t.dim() == 1:
            if not t.is_contiguous():
                raise ValueError(f"{name} must be contiguous")
            if t.shape[0] < rows:
                raise IndexError(f"{name} has {t.shape[0]} entries, needs {rows}")
            return 1, rows
        if t.dim() == 2:
            # column-major (n x k) storage: stride (1, ld)
            if t.stride(0) != 1:
                raise ValueError(f"{name} must be column-major (t.stride(0) == 1)")
            if t.shape[0] < rows:
                raise IndexError(f"{name} has {t.shape[0]} rows, needs {rows}")
            return t.shape[1], max(t.stride(1), rows)
        raise ValueError(f"{name} must be 1-D or 2-D")

    def mul(self, u, v, *, accumulate=True, stream=None):
        """u (+)= H v on device tensors (1-D, or column-major 2-D for many
        right-hand sides).  accumulate=True is the reference's mul!."""
        ku, ldu = self._check_dev(u, self.shape[0], "u")
        kv, ldv = self._check_dev(v, self.shape[1], "v")
        if ku != kv:
            raise ValueError("u and v have different numbers of columns")
        check(lib.hm_mul(self._h, v.data_ptr(), ldv, u.data_ptr(), ldu, kv, 1 if accumulate else 0,
                         _stream_ptr(stream)))
        return u

    def mul_t(self, u, v, *, accumulate=True, stream=None):
        """u (+)= H^T v on device tensors (u has size(H, 2) rows, v size(H, 1))."""
        ku, ldu = self._check_dev(u, self.shape[1], "u")
        kv, ldv = self._check_dev(v, self.shape[0], "v")
        if ku != kv:
            raise ValueError("u and v have different numbers of columns")
        check(lib.hm_mul_t(self._h, v.data_ptr(), ldv, u.data_ptr(), ldu, kv, 1 if accumulate else 0,
                           _stream_ptr(stream)))
        return u

    def mul_drow(self, u, v, *, transposed=False, accumulate=True, stream=None):
        """Row-derivative products on device tensors:
        transposed=False: u (+)= D_x v with D_x[i, j] = dH[i, j]/dx_i;
        transposed=True:  u (+)= D_y^T v with D_y[i, j] = dH[i, j]/dy_j."""
        rows_u = self.shape[1] if transposed else self.shape[0]
        rows_v = self.shape[0] if transposed else self.shape[1]
        ku, ldu = self._check_dev(u, rows_u, "u")
        kv, ldv = self._check_dev(v, rows_v, "v")
        if ku != kv:
            raise ValueError("u and v have different numbers of columns")
        check(lib.hm_mul_drow(self._h, 1 if transposed else 0, v.data_ptr(), ldv, u.data_ptr(), ldu, kv,
                              1 if accumulate else 0, _stream_ptr(stream)))
        return u

    def loss_and_grad(self, w, t):
        """L = 1/2 |H w - t|^2 and its gradients (dL/dw, dL/dx, dL/dy) with the
        block tree held fixed; w, t device tensors of the handle's dtype.
        The products that do not depend on each other run on two streams
        (H w beside D_x w, then H^T r beside D_y^T r) and the host waits once,
        for the loss, at the end."""
        import torch
        cur = torch.cuda.current_stream(w.device)
        aux = getattr(self, "_aux_stream", None)
        if aux is None or aux.device != w.device:
            aux = self._aux_stream = torch.cuda.Stream(device=w.device)
        dxw = torch.empty(self.shape[0], dtype=w.dtype, device=w.device)
        dyr = torch.empty(self.shape[1], dtype=w.dtype, device=w.device)
        r = torch.empty(self.shape[0], dtype=w.dtype, device=w.device)
        aux.wait_stream(cur)                                   # w ready
        self.mul_drow(dxw, w, accumulate=False, stream=aux)
        self.mul(r, w, accumulate=False, stream=cur)
        r -= t
        aux.wait_stream(cur)                                   # r ready
        self.mul_drow(dyr, r, transposed=True, accumulate=False, stream=aux)
        gw = torch.empty(self.shape[1], dtype=w.dtype, device=w.device)
        self.mul_t(gw, r, accumulate=False, stream=cur)
        loss = 0.5 * torch.dot(r.double(), r.double())
        cur.wait_stream(aux)                                   # the derivative products are done
        gx, gy = r * dxw, w * dyr
        return float(loss), gw, gx, gy

    @property
    def T(self):
        """The transpose as an operator: ``H.T @ v`` runs the transposed product."""
        return _Transposed(self)

    def mul_strided(self, y, x, istart=1, jstart=1, incx=1, incy=1, *, stream=None):
        """mul!(y, H, x, istart, jstart, INCX, INCY) on device vectors (1-based)."""
        self._check_dev(y, 0, "y")
        self._check_dev(x, 0, "x")
        check(lib.hm_mul_strided(self._h, x.data_ptr(), x.numel(), jstart, incx, y.data_ptr(),
                                 y.numel(), istart, incy, _stream_ptr(stream)))
        return y

    def mul_host(self, u, v, *, accumulate=True):
        """u (+)= H v on host numpy arrays (column-major (n, k) for k > 1)."""
        u_ = np.asarray(u)
        v_ = np.asfortranarray(v, dtype=self.dtype)
        if u_.dtype != self.dtype or not (u_.flags.f_contiguous or u_.ndim == 1):
            raise TypeError(f"u must be a Fortran-ordered {self.dtype} array")
        k = 1 if v_.ndim == 1 else v_.shape[1]
        if v_.shape[0] != self.shape[1] or u_.shape[0] != self.shape[0]:
            raise IndexError("dimension mismatch")
        check(lib.hm_mul_host(self._h, v_.ctypes.data, u_.ctypes.data, k, 1 if accumulate else 0))
        return u_

    def __matmul__(self, v):
        """H * v (src/KernelMatrix.jl:5-12): a new result, on the device for a
        CUDA tensor, on the host for a numpy array."""
        try:
            import torch
            if isinstance(v, torch.Tensor):
                shape = (self.shape[0],) if v.dim() == 1 else (v.shape[1], self.shape[0])
                u = torch.zeros(shape, dtype=v.dtype, device=v.device)
                if v.dim() == 2:
                    u = u.t()                        # column-major view
                return self.mul(u, v, accumulate=False)
        except ImportError:
            pass
        v = np.asfortranarray(v, dtype=self.dtype)
        u = np.zeros(v.shape[:1] and ((self.shape[0],) + v.shape[1:]), dtype=self.dtype, order="F")
        return self.mul_host(u, v, accumulate=False)

    __mul__ = __matmul__

    def direct_rows(self, b, rows, *, stream=None):
        """Exact FP64 dense rows sum_j f(x_i, y_j) b_j (device b float64, rows int64)."""
        import torch
        b = b.to(torch.float64).contiguous()
        rows = rows.to(torch.int64).contiguous()
        out = torch.empty(rows.numel(), dtype=torch.float64, device=b.device)
        check(lib.hm_direct_rows(self._h, b.data_ptr(), rows.data_ptr(), rows.numel(),
                                 out.data_ptr(), _stream_ptr(stream)))
        return out

    def set_overlap(self, enable=True):
        """Tree passes on a side stream beside the near-field panels: the near
        field from the start (1), after the upward pass (2; True, the
        default), after the far-field stage (3) or after the leaf-basis
        stage (4); or every stage in order (False or 0)."""
        mode = int(enable) if not isinstance(enable, bool) else (2 if enable else 0)
        check(lib.hm_configure(self._h, _lib.HM_OPT_OVERLAP, mode))

    def set_pdl(self, enable=True):
        """Programmatic dependent launches along the tree passes (default) or
        plain launches."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_PDL, 1 if enable else 0))

    def set_tensor_cores(self, enable=True):
        """FP32 products with 16+ right-hand sides on the tensor cores (default)
        or on the FP32 pipes."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_TENSOR_CORES, 1 if enable else 0))

    def set_near_kernel(self, which):
        """Near-field panels with up to 8 right-hand sides: "auto" (the
        default: per-warp rings for 3-8 FP32 right-hand sides, else one warp
        per row segment), "warp" (one warp per row segment), "stream" (CTAs
        streaming runs of segments through shared memory with cp.async.bulk)
        or "ring" (warps streaming runs of segments through per-warp rings
        with cp.async; FP32 with 3-8 right-hand sides, else as "auto")."""
        code = {"auto": 0, "warp": 1, "stream": 2, "ring": 3}[which]
        check(lib.hm_configure(self._h, _lib.HM_OPT_NEAR_KERNEL, code))

    def set_near_stages(self, n):
        """Shared-memory stages (8 KB each) of the near-field streaming kernel."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_NEAR_STAGES, int(n)))

    def autotune(self, nrhs=1, reps=20, *, stream=None):
        """Time every candidate schedule of a product with ``nrhs`` right-hand
        sides (stream placement of the near field, near-field kernel and ring
        depth, tensor cores, programmatic dependent launches) and keep the fastest for that right-hand-side
        bucket.  Returns the choice and the time per product of it and of the
        configured options."""
        choice = (ctypes.c_int32 * 5)()
        ms = (ctypes.c_double * 2)()
        check(lib.hm_autotune(self._h, int(nrhs), int(reps), _stream_ptr(stream), choice, ms))
        out = self.schedule(nrhs)
        out.update(ms=ms[0], ms_configured=ms[1])
        return out

    def schedule(self, nrhs=1):
        """The schedule products with ``nrhs`` right-hand sides run with (the
        autotuner's choice for its bucket, else the configured options),
        including the ring tile (panel values x stages per warp) and whether the
        tree passes run on the lane-per-right-hand-side kernels."""
        v = (ctypes.c_int32 * 7)()
        n = lib.hm_autotune_choice(self._h, int(nrhs), v, 7)
        if n < 0:
            check(-n)
        tiles = ((768, 3), (512, 4), (1024, 3))
        return {"overlap": v[0], "near_kernel": v[1], "near_stages": v[2], "tensor_cores": bool(v[3]),
                "pdl": bool(v[4]), "ring_tile": {"panel_values": tiles[v[5]][0], "stages": tiles[v[5]][1]},
                "wide_tree": {0: False, 1: True, 2: "all"}.get(v[6], v[6])}

    def forget_autotune(self):
        """Drop the autotuned schedules: products run with the configured options."""
        check(lib.hm_configure(self._h, _lib.HM_OPT_AUTOTUNED, 0))

    def profile(self, stages=_lib.STAGES):
        """Record CUDA events around the launches of the named matvec stages
        (see stage_times); an empty list turns timing off."""
        mask = 0
        for name in stages or ():
            mask |= 1 << _lib.STAGES.index(name)
        check(lib.hm_profile(self._h, mask))

    def stage_times(self, reset=True):
        """{stage: (total ms, launches)} accumulated since the last reset."""
        n = len(_lib.STAGES)
        ms = np.zeros(n)
        cnt = np.zeros(n, dtype=np.int64)
        check(lib.hm_profile_read(self._h, _lib.f64_ptr(ms),
                                  cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n,
                                  1 if reset else 0))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(_lib.STAGES)}

    def free(self):
        if getattr(self, "_h", None):
            lib.hm_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class KernelMatrixBatch(KernelMatrix):
    """Many independent KernelMatrices multiplied together (block-diagonal).

    ``xs``, ``ys``: lists of point arrays (each non-increasing); ``boxes``:
    one (a, b, c, d) per instance.  Rows/columns of instance i follow those of
    instances 0..i-1 in the vectors given to ``mul``; ``offsets`` holds the
    row and column starts.
    """

    def __init__(self, f, xs, ys, boxes, *, dtype=np.float64, rank=None, blocksize=None, stream=None):
        self.kernel = _kernel_id(f)
        self.f = f
        self.storage, self.dtype = _storage_of(dtype)
        self.rank = int(rank) if rank else BLOCKRANK(np.float64)
        self.blocksize = int(blocksize) if blocksize else 4 * self.rank
        nx = np.array([len(v) for v in xs], dtype=np.int64)
        ny = np.array([len(v) for v in ys], dtype=np.int64)
        self.x = np.ascontiguousarray(np.concatenate([_host_f64(v) for v in xs]))
        self.y = np.ascontiguousarray(np.concatenate([_host_f64(v) for v in ys]))
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 4))
        if len(bx) != len(xs) or len(ys) != len(xs):
            raise ValueError("one point list pair and one box per instance")
        h = _vp()
        check(lib.hm_kernelmatrix_batch_build(
            self.kernel, len(xs), nx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            ny.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _lib.f64_ptr(self.x), _lib.f64_ptr(self.y),
            _lib.f64_ptr(bx), self.rank, self.blocksize, self.storage, _stream_ptr(stream),
            ctypes.byref(h)))
        self._h = h
        self.ninst = len(xs)
        self.row_offsets = np.concatenate([[0], np.cumsum(nx)])
        self.col_offsets = np.concatenate([[0], np.cumsum(ny)])
        self.shape = (int(nx.sum()), int(ny.sum()))

    def mul_t(self, *a, **k):
        raise NotImplementedError("the transposed product is not available for batched handles")


class _Transposed:
    def __init__(self, H):
        self.H = H
        self.shape = (H.shape[1], H.shape[0])

    def __matmul__(self, v):
        import torch
        shape = (self.shape[0],) if v.dim() == 1 else (v.shape[1], self.shape[0])
        u = torch.empty(shape, dtype=v.dtype, device=v.device)        # overwritten (accumulate=False)
        if v.dim() == 2:
            u = u.t()
        return self.H.mul_t(u, v, accumulate=False)
