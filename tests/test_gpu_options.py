"""Product options on the GPU: the stream schedule (HM_OPT_OVERLAP) leaves the
result unchanged, and the two near-field kernels (one warp per row segment;
CTAs streaming runs of segments through shared memory with cp.async.bulk)
agree within the storage type's tolerance for 1, 2 and 8 right-hand sides."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from oracle import oracle as O  # noqa: E402

TOL = {np.float64: 1e-13, np.float32: 1e-6}
TDT = {np.float64: torch.float64, np.float32: torch.float32}


def colrel(a, b):
    a, b = a.double().reshape(a.shape[0], -1), b.double().reshape(b.shape[0], -1)
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


@pytest.fixture(scope="module", params=[np.float32, np.float64])
def mat(request):
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=request.param)
    yield n, request.param, H
    H.free()


def test_overlap_modes(mat):
    n, dt, H = mat
    b = torch.randn(n, device="cuda", dtype=TDT[dt])
    ref = H @ b
    try:
        for mode in (1, 3, 2):
            H.set_overlap(mode)
            assert torch.equal(H @ b, ref)
        H.set_overlap(False)
        assert colrel(H @ b, ref) <= TOL[dt]
    finally:
        H.set_overlap(True)
    assert H.device_status() == 0


@pytest.mark.parametrize("k", [1, 2, 8])
def test_near_kernels_agree(mat, k):
    n, dt, H = mat
    B = torch.randn(k, n, device="cuda", dtype=TDT[dt]).t()
    if k == 1:
        B = B[:, 0].contiguous()
    try:
        H.set_near_kernel("warp")
        Uw = H @ B
        H.set_near_kernel("stream")
        Us = H @ B
    finally:
        H.set_near_kernel("auto")
    assert colrel(Us, Uw) <= TOL[dt]
    assert H.device_status() == 0


@pytest.mark.parametrize("k", [3, 4, 5, 8])
def test_ring_kernel_agrees(mat, k):
    """Per-warp rings (the default for 3-8 FP32 right-hand sides) against the
    one-warp-per-segment kernel, near and far parts, accumulate on and off;
    FP64 falls back to the warp kernel (bitwise equal)."""
    n, dt, H = mat
    B = torch.randn(k, n, device="cuda", dtype=TDT[dt]).t()
    U0 = torch.randn(k, n, device="cuda", dtype=TDT[dt]).t()
    try:
        for acc in (False, True):
            H.set_near_kernel("warp")
            Uw = U0.clone()
            H.mul(Uw, B, accumulate=acc)
            H.set_near_kernel("ring")
            Ur = U0.clone()
            H.mul(Ur, B, accumulate=acc)
            if dt == np.float64:
                assert torch.equal(Ur, Uw)
            else:
                assert colrel(Ur, Uw) <= 5e-7, acc
            for mode in (0, 1, 4):
                H.set_overlap(mode)
                again = U0.clone()
                H.mul(again, B, accumulate=acc)
                assert colrel(again, Ur) <= (1e-15 if mode else 5e-7)
            H.set_overlap(True)
    finally:
        H.set_near_kernel("auto")
        H.set_overlap(True)
    assert H.device_status() == 0


def test_host_buffer_product_replays(mat):
    # hm_mul_host runs plainly once, then replays a captured graph; options
    # changed in between are followed (the graph is dropped and captured again)
    n, dt, H = mat
    rng = np.random.default_rng(9)
    v = rng.standard_normal(n).astype(dt)
    ref = (H @ torch.tensor(v, device="cuda")).cpu().numpy()
    outs = []
    for i in range(4):
        u = np.zeros(n, dtype=dt)
        H.mul_host(u, v, accumulate=False)
        outs.append(u)
        if i == 1:
            H.set_overlap(1)
    H.set_overlap(True)
    for u in outs:
        assert np.array_equal(u, ref)
    u0 = rng.standard_normal(n).astype(dt)
    u = u0.copy()
    for _ in range(3):
        u = u0.copy()
        H.mul_host(u, v, accumulate=True)
    np.testing.assert_allclose(u, u0 + ref, rtol=TOL[dt], atol=TOL[dt] * np.abs(ref).max())


@pytest.mark.parametrize("k", [1, 4, 32])
def test_programmatic_launches_change_nothing(mat, k):
    """Launching the tree passes as programmatic dependents (HM_OPT_PDL) runs
    the same kernels on the same data: results equal bit for bit, for every
    stream schedule (one stream, side stream, near field after each stage)."""
    n, dt, H = mat
    B = torch.randn(k, n, device="cuda", dtype=TDT[dt]).t()
    try:
        for mode in (0, 1, 2, 3, 4):
            H.set_overlap(mode)
            H.set_pdl(False)
            U0 = torch.empty(k, n, device="cuda", dtype=TDT[dt]).t()
            H.mul(U0, B, accumulate=False)
            H.set_pdl(True)
            for _ in range(3):
                U1 = torch.empty(k, n, device="cuda", dtype=TDT[dt]).t()
                H.mul(U1, B, accumulate=False)
                assert torch.equal(U1, U0), (mode, k)
    finally:
        H.set_overlap(True)
        H.set_pdl(True)


@pytest.mark.parametrize("k", [1, 3, 8])
def test_split_schedules_accumulate_like_serial(mat, k):
    """u += H v with the tree passes on a side stream: the near and far parts
    of each row segment are combined by whichever kernel finishes second, as
    (u + near) + far, which is what the one-stream schedule computes; results
    equal it bit for bit, call after call."""
    n, dt, H = mat
    B = torch.randn(k, n, device="cuda", dtype=TDT[dt]).t()
    U0 = torch.randn(k, n, device="cuda", dtype=TDT[dt]).t()
    try:
        H.set_overlap(0)
        ref = U0.clone()
        H.mul(ref, B, accumulate=True)
        for mode in (1, 2, 3, 4):
            H.set_overlap(mode)
            for _ in range(3):
                got = U0.clone()
                H.mul(got, B, accumulate=True)
                assert torch.equal(got, ref), (mode, k)
    finally:
        H.set_overlap(True)


def test_profile_timeline(mat):
    """hm_profile_timeline: one record per timed stage of the last product,
    each inside the whole-product record, consumed when read."""
    import ctypes
    from hierarchicalmatrices import _lib
    n, dt, H = mat
    b = torch.randn(n, device="cuda", dtype=TDT[dt])
    u = torch.empty_like(b)
    H.profile()
    try:
        H.mul(u, b, accumulate=False)
        out = np.zeros(3 * 16)
        k = _lib.lib.hm_profile_timeline(H.handle, out.ctypes.data_as(ctypes.c_void_p), 16)
        recs = out[:3 * k].reshape(k, 3)
        names = [_lib.STAGES[int(s)] for s in recs[:, 0]]
        assert sorted(names) == sorted(_lib.STAGES)
        whole = recs[names.index("product")]
        assert whole[1] == 0.0 and whole[2] > 0.0
        for st, t0, t1 in recs:
            assert whole[1] <= t0 <= t1 <= whole[2] + 1e-3
        assert _lib.lib.hm_profile_timeline(H.handle, out.ctypes.data_as(ctypes.c_void_p), 16) == 0
    finally:
        H.profile([])
        H.stage_times(reset=True)
