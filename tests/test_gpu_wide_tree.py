"""Tree passes for 32 and more right-hand sides on the lane-per-right-hand-side
kernels (leaf_up_w, xfer_task_w, m2l_w) against the kernels for chunks of 8
(HM_OPT_WIDE_TREE 0) and, in FP64, against the oracle's reference-order
product (src/KernelMatrix.jl:17-45, src/algebra.jl:243-277); the ring tiles
for 3-8 FP32 right-hand sides against each other; the schedule query."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from oracle import oracle as O  # noqa: E402

TDT = {np.float64: torch.float64, np.float32: torch.float32}


def colrel(a, b):
    a, b = a.double(), b.double()
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


@pytest.fixture(scope="module", params=["grid", "uniform"])
def points(request):
    n = 8192
    if request.param == "grid":
        x, y = O.grid_points(n)
    else:
        rng = np.random.default_rng(17)
        x = np.sort(rng.random(n))[::-1].copy()
        y = np.sort(rng.random(n))[::-1].copy()
    return n, x, y


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("k", [32, 33, 64, 100])
def test_wide_tree_matches_narrow(points, dtype, k):
    n, x, y = points
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    g = torch.Generator(device="cuda").manual_seed(k)
    B = torch.randn(k, n, device="cuda", dtype=TDT[dtype], generator=g).t()
    H.set_tensor_cores(False)               # the same panel kernel on both sides
    assert H.schedule(k)["wide_tree"]
    Uw = H @ B
    H.set_wide_tree(False)
    assert not H.schedule(k)["wide_tree"]
    Un = H @ B
    H.set_wide_tree(True)
    assert colrel(Uw, Un) <= (1e-13 if dtype == np.float64 else 5e-7)
    if dtype == np.float64:
        Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
        Bh = B.cpu().numpy()
        for q in (0, k // 2, k - 1):
            ref = Ho @ Bh[:, q].copy()
            got = Uw[:, q].cpu().numpy()
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-12
    assert H.device_status() == 0
    H.free()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("k", [2, 3, 8, 12, 20])
def test_grouped_wide_tree_matches_narrow(points, dtype, k):
    """Fewer than 32 right-hand sides on the grouped lane-per-RHS kernels
    (HM_OPT_WIDE_TREE 2: four groups of 8 lanes up to 8, two of 16 up to 16,
    a warp beyond) against the chunk-of-8 kernels."""
    n, x, y = points
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    g = torch.Generator(device="cuda").manual_seed(100 + k)
    B = torch.randn(k, n, device="cuda", dtype=TDT[dtype], generator=g).t()
    H.set_near_kernel("warp")                # the same panel kernel on both sides
    H.set_wide_tree("all")
    assert H.schedule(k)["wide_tree"] == "all"
    Uw = H @ B
    H.set_wide_tree(False)
    Un = H @ B
    assert colrel(Uw, Un) <= (1e-13 if dtype == np.float64 else 5e-7)
    if dtype == np.float64:
        Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
        ref = Ho @ B[:, k - 1].cpu().numpy().copy()
        got = Uw[:, k - 1].cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-12
    assert H.device_status() == 0
    H.free()


def test_wide_tree_batch_and_transpose():
    # a batched (block-diagonal) plan, and the transposed product's own plan
    rng = np.random.default_rng(40)
    xs, ys = [], []
    for _ in range(6):
        n = int(np.exp(rng.uniform(np.log(1024), np.log(20000))))
        xs.append(np.sort(rng.random(n))[::-1].copy())
        ys.append(np.sort(rng.random(n))[::-1].copy())
    Hb = hm.KernelMatrixBatch(hm.cauchykernel, xs, ys, [(1.0, 0.0, 1.0, 0.0)] * 6, dtype=np.float64)
    k = 40
    B = torch.randn(k, Hb.shape[1], device="cuda", dtype=torch.float64).t()
    Uw = Hb @ B
    Hb.set_wide_tree(False)
    Un = Hb @ B
    assert colrel(Uw, Un) <= 1e-13
    B8 = B[:, :8].contiguous().t().contiguous().t()            # 8 right-hand sides, column-major
    Hb.set_wide_tree("all")
    W8 = Hb @ B8
    Hb.set_wide_tree(False)
    assert colrel(W8, Hb @ B8) <= 1e-13
    x = np.sort(rng.random(12000))[::-1].copy()
    y = np.sort(rng.random(9000))[::-1].copy()
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    V = torch.randn(k, 12000, device="cuda", dtype=torch.float64).t()
    Tw = H.T @ V
    H.set_wide_tree(False)
    Tn = H.T @ V
    assert colrel(Tw, Tn) <= 1e-13


@pytest.mark.parametrize("k", [4, 8])
def test_ring_tiles_agree(points, k):
    n, x, y = points
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    B = torch.randn(k, n, device="cuda", dtype=torch.float32).t()
    H.set_near_kernel("warp")
    ref = H @ B
    H.set_near_kernel("auto")
    for tile, shape in ((0, (768, 3)), (1, (512, 4)), (2, (1024, 3))):
        H.set_ring_tile(tile)
        sc = H.schedule(k)
        assert (sc["ring_tile"]["panel_values"], sc["ring_tile"]["stages"]) == shape
        assert colrel(H @ B, ref) <= 5e-7, tile
    with pytest.raises(hm.HMError):
        H.set_ring_tile(3)
    H.set_ring_tile(0)
    sc = H.autotune(k, reps=2)
    assert sc["ms"] > 0 and "ring_tile" in sc
    assert colrel(H @ B, ref) <= 5e-7
    H.free()
