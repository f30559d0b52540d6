"""HM_DF64 storage: the FP64 KernelMatrix product with its row-segment panels
stored as double-float pairs and multiplied on the FP32 pipes, against the
oracle's reference-order FP64 product (src/KernelMatrix.jl:17-45,
src/algebra.jl:243-277) at the FP64 tolerance, 1e-12 relative, and against the
native FP64 storage of the same build."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import _lib  # noqa: E402
from oracle import oracle as O  # noqa: E402

TOL64 = 1e-12
KFUN = {O.CAUCHY: hm.cauchykernel, O.COULOMB: hm.coulombkernel,
        O.COULOMB_PRIME: hm.coulombprimekernel, O.LOG: hm.logkernel}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def dev(a):
    return torch.tensor(np.asarray(a), device="cuda", dtype=torch.float64)


@pytest.mark.parametrize("n", [128, 2048, 65536])
def test_grid_matches_oracle(n):
    x, y = O.grid_points(n)
    b = np.random.default_rng(n).standard_normal(n)
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    assert H.storage == _lib.HM_DF64 and _lib.lib.hm_storage(H.handle) == _lib.HM_DF64
    u = (H @ dev(b)).cpu().numpy()
    assert rel(u, ref) <= TOL64
    H64 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert rel(u, (H64 @ dev(b)).cpu().numpy()) <= 1e-13
    assert H.stats()["stored_values"] == H64.stats()["stored_values"]


@pytest.mark.parametrize("kernel", [O.CAUCHY, O.COULOMB, O.COULOMB_PRIME, O.LOG])
def test_example_kernels_and_points(kernel):
    # examples/Kernel.jl:58-78 (Chebyshev points) and :88-107 (quadratic spacing)
    for family, n in (("chebyshev", 10000), ("quadratic", 4000)):
        x, y, box = O.example_points(family, n)
        b = np.random.default_rng(3).standard_normal(n)
        ref = O.OracleKernelMatrix(kernel, x, y, *box) @ b
        H = hm.KernelMatrix(KFUN[kernel], x, y, *box, dtype="df64")
        assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64, family


def test_beta_points_matches_oracle():
    x, y = O.beta_points(65536, 21)
    b = np.random.default_rng(1).standard_normal(65536)
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64


@pytest.mark.parametrize("k", [2, 3, 8, 12, 20])
def test_multi_rhs_columns(k):
    """Up to 8 right-hand sides run the near and far parts on two streams;
    more run every column in chunks of 8."""
    n = 8192
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    B = torch.randn(k, n, device="cuda", dtype=torch.float64).t()
    U0 = torch.randn(k, n, device="cuda", dtype=torch.float64).t()
    U = U0.clone()
    H.mul(U, B, accumulate=True)
    Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    Bh = B.cpu().numpy()
    for q in range(k):
        ref = Ho @ Bh[:, q].copy()
        assert rel((U[:, q] - U0[:, q]).cpu().numpy(), ref) <= TOL64, q


def test_transposed_strided_and_host():
    rng = np.random.default_rng(31)
    x = np.sort(rng.random(20000))[::-1].copy()
    y = np.sort(rng.random(13000))[::-1].copy()
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    v = rng.standard_normal(20000)
    ref = -(O.OracleKernelMatrix(O.CAUCHY, y, x, 1.0, 0.0, 1.0, 0.0) @ v)
    assert rel((H.T @ dev(v)).cpu().numpy(), ref) <= TOL64
    w = rng.standard_normal(13000)
    refw = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ w
    xs = rng.standard_normal(3 + 2 * 13000)
    xs[1:1 + 2 * 13000:2] = w
    ys = np.zeros(5 + 3 * 20000)
    yd = dev(ys)
    H.mul_strided(yd, dev(xs), istart=4, jstart=2, incx=2, incy=3)
    assert rel(yd.cpu().numpy()[3:3 + 3 * 20000:3], refw) <= TOL64
    u = H @ w                                                  # host arrays: hm_mul_host
    assert isinstance(u, np.ndarray) and rel(u, refw) <= TOL64


def test_row_derivative_matches_fp64():
    rng = np.random.default_rng(2)
    x = np.sort(rng.random(16384))[::-1].copy()
    y = np.sort(rng.random(16384))[::-1].copy()
    b = dev(rng.standard_normal(16384))
    out = []
    for dt in (np.float64, "df64"):
        H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dt)
        u = torch.empty(16384, device="cuda", dtype=torch.float64)
        H.mul_drow(u, b, accumulate=False)
        v = torch.empty(16384, device="cuda", dtype=torch.float64)
        H.mul_drow(v, b, transposed=True, accumulate=False)
        out.append((u.cpu().numpy(), v.cpu().numpy()))
    assert rel(out[1][0], out[0][0]) <= 1e-12
    assert rel(out[1][1], out[0][1]) <= 1e-12


def test_autotuned_schedule_and_noalloc():
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    b = dev(np.random.default_rng(4).standard_normal(n))
    ref = H @ b
    H.autotune(1, reps=3)
    assert float(torch.linalg.norm(H @ b - ref) / torch.linalg.norm(ref)) <= 1e-15
    u = torch.empty_like(b)
    _lib.check(_lib.lib.hm_mul_noalloc(H.handle, b.data_ptr(), u.data_ptr(), 0,
                                       torch.cuda.current_stream().cuda_stream))
    assert float(torch.linalg.norm(u - ref) / torch.linalg.norm(ref)) <= 1e-15
    assert H.device_status() == 0


def test_values_beyond_double_float_range_are_rejected():
    """Coulomb' 1/(x - y)^3 with one gap of 1e-13 gives a near-field value of
    1e39, beyond FP32's exponent range: HM_DF64 refuses the build, FP64 builds."""
    x, y = O.grid_points(256)
    y = y.copy()
    y[100] = x[100] - 1e-13
    H64 = hm.KernelMatrix(hm.coulombprimekernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert np.isfinite((H64 @ dev(np.ones(256))).cpu().numpy()).all()
    with pytest.raises(hm.HMError) as e:
        hm.KernelMatrix(hm.coulombprimekernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    assert e.value.status == _lib.HM_ERR_UNSUPPORTED


def test_2pow20_full_vector_matches_oracle():
    n = 1 << 20
    x, y = O.grid_points(n)
    b = np.random.default_rng(1234).standard_normal(n)
    Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0, nthreads=os.cpu_count())
    ref = np.zeros(n)
    Ho.mul(ref, b, nthreads=os.cpu_count())
    del Ho
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype="df64")
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64
    H.free()
