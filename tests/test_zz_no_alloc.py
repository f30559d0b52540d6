"""hm_mul_noalloc: the product for callers that cannot let the library allocate
device memory (memory reserved up front by another allocator, or loops that
must not call cudaMalloc/cudaFree after start-up).  Its coefficient scratch is
a fixed array inside libhmgpu.so.

The test calls the entry point through the C ABI and checks it against hm_mul,
twice in a row (the second call runs on whatever the first left in the shared
scratch).  This file is collected last so that a failing run that stops at
the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import _lib  # noqa: E402
from oracle import oracle as O  # noqa: E402

TOL = {np.float64: 1e-12, np.float32: 1e-6}


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_noalloc_matches_mul_twice(dtype):
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    g = torch.Generator(device="cuda").manual_seed(3)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        v = torch.randn(n, device="cuda", dtype=tdt, generator=g)
        u0 = torch.randn(n, device="cuda", dtype=tdt, generator=g)
        ref = u0.clone()
        _lib.check(_lib.lib.hm_mul(H.handle, v.data_ptr(), n, ref.data_ptr(), n, 1, 1, stream))
        got = u0.clone()
        _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), got.data_ptr(), 1, stream))
        torch.cuda.synchronize()
        err = float(torch.linalg.norm((got - ref).double()) / torch.linalg.norm(ref.double()))
        assert err <= TOL[dtype], (call, err)
        over = torch.empty(n, device="cuda", dtype=tdt)
        _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), over.data_ptr(), 0, stream))
        torch.cuda.synchronize()
        err = float(torch.linalg.norm((over - (ref - u0)).double()) / torch.linalg.norm((ref - u0).double()))
        assert err <= TOL[dtype], (call, err)


def test_noalloc_rejects_null():
    st = _lib.lib.hm_mul_noalloc(None, None, None, 1, None)
    assert st == _lib.HM_ERR_INVALID_ARG
    assert ctypes.c_int(st).value != 0
