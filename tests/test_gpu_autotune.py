"""The autotuner (hm_autotune): it returns a valid schedule for each
right-hand-side bucket, products of a tuned bucket give the same result as
before within the storage type's tolerance (the stream placement alone leaves
the result bitwise unchanged; the two near-field kernels sum in different
orders), forgetting the tuned schedules restores the configured product bit
for bit, and the tuned schedule is what a captured CUDA graph replays."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import _lib  # noqa: E402
from oracle import oracle as O  # noqa: E402

TOL = {np.float64: 1e-13, np.float32: 1e-6}
TDT = {np.float64: torch.float64, np.float32: torch.float32}


def colrel(a, b):
    a, b = a.double().reshape(a.shape[0], -1), b.double().reshape(b.shape[0], -1)
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


def valid(choice, k, dtype):
    assert 0 <= choice["overlap"] <= 4
    assert choice["near_kernel"] in (0, 1, 2)       # 1 (warp per segment) is a candidate for 3-8 FP32 RHS
    assert (choice["ring_tile"]["panel_values"], choice["ring_tile"]["stages"]) in ((768, 3), (512, 4), (1024, 3))
    assert choice["wide_tree"] in (True, False, "all")
    assert 2 <= choice["near_stages"] <= 16
    if dtype == np.float64 or k < 16:
        assert choice["tensor_cores"]          # the configured value, untouched
    assert 0 < choice["ms"] <= choice["ms_configured"]


@pytest.mark.parametrize("dtype,k", [(np.float32, 1), (np.float32, 4), (np.float32, 32), (np.float64, 1)])
def test_autotuned_product_matches(dtype, k):
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    g = torch.Generator(device="cuda").manual_seed(9)
    B = torch.randn(k, n, device="cuda", dtype=TDT[dtype], generator=g).t()
    U0 = torch.empty(k, n, device="cuda", dtype=TDT[dtype]).t()
    H.mul(U0, B, accumulate=False)
    choice = H.autotune(k, reps=5)
    valid(choice, k, dtype)
    U1 = torch.empty_like(U0)
    H.mul(U1, B, accumulate=False)
    assert colrel(U1, U0) <= TOL[dtype]
    H.set_overlap(True)                             # an explicit option replaces the tuned schedules
    U2 = torch.empty_like(U0)
    H.mul(U2, B, accumulate=False)
    assert torch.equal(U2, U0)
    H.autotune(k, reps=5)
    H.forget_autotune()
    H.mul(U2, B, accumulate=False)
    assert torch.equal(U2, U0)
    if k == 1:
        ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ B[:, 0].double().cpu().numpy()
        err = np.linalg.norm(U1[:, 0].double().cpu().numpy() - ref) / np.linalg.norm(ref)
        assert err <= (1e-12 if dtype == np.float64 else 1e-6)
    H.free()


def test_autotuned_batch_in_graph():
    rng = np.random.default_rng(41)
    xs, ys, boxes = [], [], []
    for _ in range(16):
        m = int(np.exp(rng.uniform(np.log(1024), np.log(16384))))
        xs.append(np.sort(rng.random(m))[::-1].copy())
        ys.append(np.sort(rng.random(m))[::-1].copy())
        boxes.append((1.0, 0.0, 1.0, 0.0))
    Hb = hm.KernelMatrixBatch(hm.cauchykernel, xs, ys, boxes, dtype=np.float32)
    k = 8
    B = torch.randn(k, Hb.shape[1], device="cuda", dtype=torch.float32).t()
    U0 = torch.empty(k, Hb.shape[0], device="cuda", dtype=torch.float32).t()
    Hb.mul(U0, B, accumulate=False)
    valid(Hb.autotune(k, reps=5), k, np.float32)
    U1 = torch.empty_like(U0)
    cs = torch.cuda.Stream()
    cs.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cs):
        Hb.mul(U1, B, accumulate=False, stream=cs)  # scratch and side stream before capture
    cs.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=cs):
        Hb.mul(U1, B, accumulate=False, stream=cs)
    U1.zero_()
    torch.cuda.synchronize()
    graph.replay()
    torch.cuda.synchronize()
    assert colrel(U1, U0) <= TOL[np.float32]
    Hb.free()


def test_autotune_rejects_bad_arguments():
    assert _lib.lib.hm_autotune(None, 1, 1, None, None, None) == _lib.HM_ERR_INVALID_ARG
    n = 4096
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert _lib.lib.hm_autotune(H.handle, 0, 1, None, None, None) == _lib.HM_ERR_INVALID_ARG
    assert _lib.lib.hm_autotune(H.handle, 1, 0, None, None, None) == _lib.HM_ERR_INVALID_ARG
    assert _lib.lib.hm_configure(H.handle, _lib.HM_OPT_AUTOTUNED, 1) == _lib.HM_ERR_INVALID_ARG
    H.free()
