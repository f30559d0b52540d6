"""hm_mul_noalloc: the product for callers that cannot let the library allocate
device memory (memory reserved up front by another allocator, or loops that
must not call cudaMalloc/cudaFree after start-up).  Its coefficient scratch is
reserved per handle when the handle is built.

The tests call the entry point through the C ABI and check it against hm_mul:
repeated calls, overwrite and accumulate, and two handles driven alternately
from two streams (calls on one handle are ordered by the library; different
handles share nothing)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import _lib  # noqa: E402
from oracle import oracle as O  # noqa: E402

TOL = {np.float64: 1e-12, np.float32: 1e-6}
TDT = {np.float64: torch.float64, np.float32: torch.float32}


def relerr(a, b):
    return float(torch.linalg.norm((a - b).double()) / torch.linalg.norm(b.double()))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_noalloc_matches_mul_twice(dtype):
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    g = torch.Generator(device="cuda").manual_seed(3)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        v = torch.randn(n, device="cuda", dtype=TDT[dtype], generator=g)
        u0 = torch.randn(n, device="cuda", dtype=TDT[dtype], generator=g)
        ref = u0.clone()
        _lib.check(_lib.lib.hm_mul(H.handle, v.data_ptr(), n, ref.data_ptr(), n, 1, 1, stream))
        got = u0.clone()
        _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), got.data_ptr(), 1, stream))
        torch.cuda.synchronize()
        assert relerr(got, ref) <= TOL[dtype], call
        over = torch.empty(n, device="cuda", dtype=TDT[dtype])
        _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), over.data_ptr(), 0, stream))
        torch.cuda.synchronize()
        assert relerr(over, ref - u0) <= TOL[dtype], call
    H.free()


def test_noalloc_two_handles_two_streams():
    n = 32768
    x, y = O.grid_points(n)
    Ha = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    Hb = hm.KernelMatrix(hm.coulombkernel, x, y, 1.0, 0.0, 1.0, 0.0)
    g = torch.Generator(device="cuda").manual_seed(5)
    vs = [torch.randn(n, device="cuda", dtype=torch.float64, generator=g) for _ in range(6)]
    refs = [(H @ v) for v in vs for H in (Ha, Hb)]
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = [torch.empty(n, device="cuda", dtype=torch.float64) for _ in refs]
    i = 0
    for v in vs:
        for H in (Ha, Hb):
            st = (s1 if i % 3 else s2).cuda_stream          # the same handle on both streams
            _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), outs[i].data_ptr(), 0, st))
            i += 1
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        assert relerr(o, r) <= 1e-13
    Ha.free()
    Hb.free()


def test_noalloc_rejects_null():
    st = _lib.lib.hm_mul_noalloc(None, None, None, 1, None)
    assert st == _lib.HM_ERR_INVALID_ARG
    assert ctypes.c_int(st).value != 0
