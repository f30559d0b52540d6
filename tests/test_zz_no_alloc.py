"""hm_mul_noalloc: the single right-hand-side product for callers that cannot
let the library allocate device memory while they run — processes whose GPU
memory is claimed up front by another allocator, and loops that must not call
cudaMalloc/cudaFree after start-up because those calls can synchronise the
device.  Its coefficient scratch is a fixed 16 MiB array inside libhmgpu.so.

The tests call the entry point through the C ABI and compare it with hm_mul,
the entry point that allocates its own scratch, on two calls in a row (the
second call starts from whatever the first left in the shared array), with
the tolerances of the other product tests.  This file is collected last, so a
run that stops at its first failure has already run every other test; it
passes alone in a fresh process as well (the first call looks up the array's
device address)."""
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
    # the device's free memory does not move across a call (after the first
    # call on this handle set up its kernels' attributes)
    v = torch.randn(n, device="cuda", dtype=TDT[dtype], generator=g)
    u = torch.zeros(n, device="cuda", dtype=TDT[dtype])
    _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), u.data_ptr(), 0, stream))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), u.data_ptr(), 0, stream))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    for call in range(2):
        v = torch.randn(n, device="cuda", dtype=TDT[dtype], generator=g)
        u0 = torch.randn(n, device="cuda", dtype=TDT[dtype], generator=g)
        ref = u0.clone()
        _lib.check(_lib.lib.hm_mul(H.handle, v.data_ptr(), n, ref.data_ptr(), n, 1, 1, stream))
        got = u0.clone()
        _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), got.data_ptr(), 1, stream))
        torch.cuda.synchronize()
        assert relerr(got, ref) <= TOL[dtype], ("accumulate", call)
        over = torch.empty(n, device="cuda", dtype=TDT[dtype])
        _lib.check(_lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), over.data_ptr(), 0, stream))
        torch.cuda.synchronize()
        assert relerr(over, ref - u0) <= TOL[dtype], ("overwrite", call)
    H.free()


def test_noalloc_rejects_matrix_beyond_fixed_scratch():
    # rank 32 with 20-point leaves at n = 2^19: (32,764 + 32,764) slots x 32 x 8 B
    # of FP64 coefficients = 32 MiB, twice the fixed array
    n = 1 << 19
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, rank=32, blocksize=20)
    v = torch.zeros(n, device="cuda", dtype=torch.float64)
    u = torch.zeros(n, device="cuda", dtype=torch.float64)
    st = _lib.lib.hm_mul_noalloc(H.handle, v.data_ptr(), u.data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.HM_ERR_UNSUPPORTED
    assert "scratch" in _lib.lib.hm_last_error().decode()
    H.free()


def test_noalloc_rejects_null():
    st = _lib.lib.hm_mul_noalloc(None, None, None, 1, None)
    assert st == _lib.HM_ERR_INVALID_ARG
    assert ctypes.c_int(st).value != 0
