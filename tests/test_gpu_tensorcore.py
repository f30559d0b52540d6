"""FP32 products with many right-hand sides on the tensor cores (tcgen05
kind::f16: each FP32 operand split exactly into three BF16 pieces, six piece
products, FP32 accumulation in tensor memory) against the FP64-storage
product (<= 1e-12 of the dense FP64 one) and against the same FP32 factors on
the FP32 pipes.  Tolerance: 1e-6 relative 2-norm error per column."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from oracle import oracle as O  # noqa: E402

TOL32 = 1e-6


def colrel(a, b):
    a, b = a.double(), b.double()
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


@pytest.fixture(scope="module", params=["grid", "beta"])
def pair(request):
    n = 8192
    x, y = O.grid_points(n) if request.param == "grid" else O.beta_points(n, 3)
    H32 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    H64 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    yield n, H32, H64
    H32.free()
    H64.free()


@pytest.mark.parametrize("k", [16, 40, 130])
def test_tensor_core_panels(pair, k):
    n, H32, H64 = pair
    g = torch.Generator(device="cuda").manual_seed(k)
    B = torch.randn(k, n, device="cuda", dtype=torch.float32, generator=g).t()     # column-major n x k
    U = H32 @ B
    ref = H64 @ B.double()
    assert colrel(U, ref) <= TOL32
    H32.set_tensor_cores(False)
    try:
        Uf = H32 @ B
    finally:
        H32.set_tensor_cores(True)
    assert colrel(U, Uf) <= TOL32
    # accumulate (mul! semantics) into a column-major block
    U0 = torch.randn(k, n, device="cuda", dtype=torch.float32, generator=g).t()
    Ua = U0.clone()
    H32.mul(Ua, B, accumulate=True)
    assert colrel(Ua - U0, ref) <= TOL32
    assert H32.device_status() == 0
