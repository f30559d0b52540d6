"""Failure paths, exercised without faulting the GPU.

* Bounded waits: the streamed near-field kernel and the tensor-core panel
  kernel wait on mbarriers (copies landing, MMAs completing) with a limit.  The
  test hook HM_OPT_TEST_STALL makes the first wait of every CTA wait on a
  barrier nothing arrives on, with a short HM_OPT_WAIT_LIMIT_NS: the kernels
  must give up, record HM_DEV_WAIT_TIMEOUT, let their copies and MMAs in flight
  land, release their tensor memory and return; the Python layer raises; the
  next product with the hook off is clean and exact.
* Allocation failure: hm_debug_fail_alloc makes the n-th device allocation of
  the library fail without calling CUDA; builds and products return
  HM_ERR_ALLOC, free what they had allocated, and work again afterwards.

The reference's own failure surface is Julia's @assert
(src/BarycentricMatrix.jl:249-250) and BoundsError from indsplit (:299-307);
those are covered by the status-code tests of the planner and the product.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import _lib  # noqa: E402
from oracle import oracle as O  # noqa: E402

TDT = {np.float64: torch.float64, np.float32: torch.float32}


def grid_matrix(n, dtype):
    x, y = O.grid_points(n)
    return hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)


def stalled_product(H, B):
    """One product with every CTA's first bounded wait running out after
    2 microseconds; returns after checking the timeout was reported."""
    H.set_wait_limit(2000)
    H._set_test_stall(True)
    try:
        U = torch.zeros_like(B)
        H.mul(U, B, accumulate=False)
        with pytest.raises(hm.DeviceWaitTimeout):
            H.check_device()
    finally:
        H._set_test_stall(False)
        H.set_wait_limit(2_000_000_000)
    H.check_device()                           # the word was cleared


@pytest.mark.parametrize("dtype,k", [(np.float32, 1), (np.float64, 1), (np.float32, 8)])
def test_streamed_near_field_wait_runs_out(dtype, k):
    n = 65536
    H = grid_matrix(n, dtype)
    H.set_near_kernel("stream")
    g = torch.Generator(device="cuda").manual_seed(k)
    B = torch.randn(k, n, device="cuda", dtype=TDT[dtype], generator=g).t()
    if k == 1:
        B = B[:, 0].contiguous()
    ref = H @ B
    H.check_device()
    stalled_product(H, B)
    assert torch.equal(H @ B, ref)
    H.check_device()
    H.free()


def test_tensor_core_wait_runs_out():
    n = 65536
    H = grid_matrix(n, np.float32)
    g = torch.Generator(device="cuda").manual_seed(5)
    B = torch.randn(32, n, device="cuda", dtype=torch.float32, generator=g).t()
    ref = H @ B                                # 32 right-hand sides: tensor-core panels
    H.check_device()
    stalled_product(H, B)
    # twice in a row: every CTA released its tensor memory, so new CTAs get theirs
    stalled_product(H, B)
    assert torch.equal(H @ B, ref)
    H.check_device()
    H.free()


def test_wait_limit_option_range():
    H = grid_matrix(2048, np.float32)
    for bad in (0, -5, 3_000_000_000):
        with pytest.raises(hm.HMError):
            H.set_wait_limit(bad)
    H.free()


def test_allocation_failure_in_build_and_product():
    n = 65536
    x, y = O.grid_points(n)
    lib = _lib.lib
    # warm-up: modules loaded and torch's tensors allocated before free memory is read
    H0 = grid_matrix(n, np.float32)
    b = torch.randn(n, device="cuda", dtype=torch.float32)
    u = torch.empty_like(b)
    ref = (H0 @ b).clone()
    H0.free()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    try:
        for after in (0, 3, 12):
            _lib.check(lib.hm_debug_fail_alloc(after))
            with pytest.raises(hm.HMError) as e:
                hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
            assert e.value.status == _lib.HM_ERR_ALLOC
        _lib.check(lib.hm_debug_fail_alloc(-1))
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0          # the failed builds freed what they had
        H = grid_matrix(n, np.float32)
        s = torch.cuda.Stream()                               # its scratch is allocated on first use
        _lib.check(lib.hm_debug_fail_alloc(0))
        with torch.cuda.stream(s):
            with pytest.raises(hm.HMError) as e:
                H.mul(u, b, accumulate=False, stream=s)
        assert e.value.status == _lib.HM_ERR_ALLOC
        _lib.check(lib.hm_debug_fail_alloc(-1))
        with torch.cuda.stream(s):
            H.mul(u, b, accumulate=False, stream=s)
        s.synchronize()
        assert torch.equal(u, ref)
        H.check_device()
        H.free()
    finally:
        lib.hm_debug_fail_alloc(-1)
