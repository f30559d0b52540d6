"""GPU parity of the KernelMatrix build + matvec (CUDA kernels through the C ABI)
against the CPU oracle.

Tolerances (the benchmark spec): FP64 storage <= 1e-12 relative 2-norm error against
the oracle's reference-order product; FP32 storage <= 1e-6 against the FP64
dense product.
"""
import glob
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from oracle import oracle as O  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12
TOL32 = 1e-6
KFUN = {O.CAUCHY: hm.cauchykernel, O.COULOMB: hm.coulombkernel,
        O.COULOMB_PRIME: hm.coulombprimekernel, O.LOG: hm.logkernel}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def dev(a, dtype=torch.float64):
    return torch.tensor(np.asarray(a), device="cuda", dtype=dtype)


@pytest.mark.parametrize("n", [128, 2048, 65536])
def test_grid_fp64_matches_oracle(n):
    x, y = O.grid_points(n)
    b = np.random.default_rng(n).standard_normal(n)
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    u = (H @ dev(b)).cpu().numpy()
    assert rel(u, ref) <= TOL64


def test_beta_fp64_matches_oracle():
    x, y = O.beta_points(65536, 21)
    b = np.random.default_rng(1).standard_normal(65536)
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_golden_fp64(path):
    d = np.load(path)
    kname = os.path.basename(path)[:-4].split("_")[1]
    f = {"cauchy": hm.cauchykernel, "coulomb": hm.coulombkernel,
         "coulombprime": hm.coulombprimekernel, "log": hm.logkernel}[kname]
    H = hm.KernelMatrix(f, d["x"], d["y"], *d["box"])
    st = H.stats()
    assert [st["n_bary"], st["n_dense"], st["depth"]] == d["stats"][:3].tolist()
    u = (H @ dev(d["b"])).cpu().numpy()
    assert rel(u, d["u"]) <= TOL64
    assert rel(u, d["u_dense"]) <= 1e-12


@pytest.mark.parametrize("kernel", [O.CAUCHY, O.COULOMB, O.COULOMB_PRIME, O.LOG])
def test_example_chebyshev_10000(kernel):
    # examples/Kernel.jl:58-78 at N = 10000
    x, y, box = O.example_points("chebyshev", 10000)
    b = np.random.default_rng(3).standard_normal(10000)
    ref = O.OracleKernelMatrix(kernel, x, y, *box) @ b
    H = hm.KernelMatrix(KFUN[kernel], x, y, *box)
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64


def test_fp32_against_dense():
    n = 65536
    x, y = O.grid_points(n)
    b = np.random.default_rng(5).standard_normal(n).astype(np.float32)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    u = (H @ dev(b, torch.float32)).cpu().numpy().astype(np.float64)
    rows = np.arange(0, n, 61)
    ref = O.dense_rows(O.CAUCHY, x, y, b.astype(np.float64), rows, nthreads=os.cpu_count())
    assert rel(u[rows], ref) <= TOL32


@pytest.mark.parametrize("dtype,k", [(np.float64, 3), (np.float64, 8), (np.float64, 12), (np.float32, 5),
                                     (np.float32, 12), (np.float32, 32)])
def test_multi_rhs_matches_columns(dtype, k):
    n = 8192
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    B = torch.randn(k, n, device="cuda", dtype=tdt).t()          # column-major n x k
    U = H @ B
    Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    Bh = B.double().cpu().numpy()
    for q in range(k):
        ref = Ho @ Bh[:, q].copy()
        assert rel(U[:, q].double().cpu().numpy(), ref) <= (TOL64 if dtype == np.float64 else TOL32)
        single = (H @ B[:, q].contiguous()).double().cpu().numpy()
        assert rel(U[:, q].double().cpu().numpy(), single) <= (1e-14 if dtype == np.float64 else 5e-7)


def test_mul_accumulates_like_reference():
    # LinearAlgebra.mul!(u, H, v) = mul!(u, H, v, 1, 1) adds into u
    n = 2048
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    b = dev(np.random.default_rng(0).standard_normal(n))
    u0 = dev(np.random.default_rng(1).standard_normal(n))
    u = u0.clone()
    hm.mul_(u, H, b)
    Hb = H @ b
    assert torch.allclose(u, u0 + Hb, rtol=1e-14, atol=1e-9)


def test_strided_mul():
    # mul!(y, H, x, istart, jstart, INCX, INCY) semantics
    n = 2048
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    rng = np.random.default_rng(2)
    xs = rng.standard_normal(3 + 2 * n)
    ys = rng.standard_normal(5 + 3 * n)
    xd, yd = dev(xs), dev(ys)
    H.mul_strided(yd, xd, istart=4, jstart=2, incx=2, incy=3)
    ref = ys.copy()
    ref[3:3 + 3 * n:3] += O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ xs[1:1 + 2 * n:2].copy()
    got = yd.cpu().numpy()
    assert rel(got[3:3 + 3 * n:3], ref[3:3 + 3 * n:3]) <= TOL64
    mask = np.ones(len(ys), dtype=bool)
    mask[3:3 + 3 * n:3] = False
    assert np.array_equal(got[mask], ys[mask])          # untouched elements
    with pytest.raises(IndexError):
        H.mul_strided(yd, xd, istart=4, jstart=10, incx=2, incy=3)


def test_host_api_and_errors():
    n = 2048
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    b = np.random.default_rng(6).standard_normal(n)
    u = H @ b                                              # numpy in -> host path
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    assert isinstance(u, np.ndarray) and rel(u, ref) <= TOL64
    with pytest.raises(IndexError):
        H.mul(torch.zeros(n - 1, device="cuda", dtype=torch.float64), dev(b))
    with pytest.raises(TypeError):
        H.mul(torch.zeros(n, device="cuda", dtype=torch.float32), dev(b))


def test_direct_rows_matches_oracle():
    n = 8192
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    b = np.random.default_rng(8).standard_normal(n)
    rows = np.arange(0, n, 37)
    got = H.direct_rows(dev(b), torch.tensor(rows, device="cuda")).cpu().numpy()
    ref = O.dense_rows(O.CAUCHY, x, y, b, rows)
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-12)
    bad = H.direct_rows(dev(b), torch.tensor([0, n, -1], device="cuda")).cpu().numpy()
    assert np.isfinite(bad[0]) and np.isnan(bad[1]) and np.isnan(bad[2])


def test_small_dense_only():
    # fewer points than BLOCKSIZE: four dense blocks, no far field
    x, y = O.grid_points(100)
    b = np.random.default_rng(1).standard_normal(100)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert H.stats()["n_bary"] == 0
    ref = O.kernel_dense(O.CAUCHY, x, y) @ b
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= 1e-14


def test_rectangular_uniform():
    rng = np.random.default_rng(12)
    x = np.sort(rng.random(30000))[::-1].copy()
    y = np.sort(rng.random(17000))[::-1].copy()
    b = rng.standard_normal(17000)
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64


def test_profile_stage_times():
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    b = dev(np.random.default_rng(0).standard_normal(n), torch.float32)
    u = torch.empty(n, device="cuda", dtype=torch.float32)
    H.profile()
    for _ in range(3):
        H.mul(u, b, accumulate=False)
    st = H.stage_times()
    H.profile([])
    assert st["expand"][1] == 3 and st["expand"][0] > 0
    assert st["down"][1] == 3 and st["up"][1] == 3 and st["far"][1] == 3


# ---- full size (n = 2^20): size-independent properties ---------------------

@pytest.fixture(scope="module")
def big():
    n = 1 << 20
    x, y = O.grid_points(n)
    H64 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    H32 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    yield n, x, y, H64, H32
    H64.free()
    H32.free()


def test_2pow20_tree(big):
    n, x, y, H64, H32 = big
    st = H64.stats()
    assert (st["n_bary"], st["n_dense"], st["depth"]) == (98214, 49150, 13)
    assert st["canonical_values"] == 785863520


def test_2pow20_linearity_and_sampled_rows(big):
    n, x, y, H64, H32 = big
    g = torch.Generator(device="cuda").manual_seed(0)
    b1 = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    b2 = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    u1, u2 = H64 @ b1, H64 @ b2
    u12 = H64 @ (2.0 * b1 - 0.5 * b2)
    assert float(torch.linalg.norm(u12 - (2.0 * u1 - 0.5 * u2)) / torch.linalg.norm(u12)) <= 1e-14
    rows_np = np.sort(np.random.default_rng(4).choice(n, 64, replace=False))
    ref = O.dense_rows(O.CAUCHY, x, y, b1.cpu().numpy(), rows_np, nthreads=os.cpu_count())
    assert rel(u1.cpu().numpy()[rows_np], ref) <= TOL64
    rows = torch.tensor(rows_np, device="cuda")
    assert rel(H64.direct_rows(b1, rows).cpu().numpy(), ref) <= 1e-14


def test_2pow20_fp32_error(big):
    n, x, y, H64, H32 = big
    g = torch.Generator(device="cuda").manual_seed(1)
    b = torch.randn(n, device="cuda", dtype=torch.float32, generator=g)
    u32 = H32 @ b
    rows = torch.tensor(np.sort(np.random.default_rng(5).choice(n, 4096, replace=False)), device="cuda")
    ref = H64.direct_rows(b.double(), rows)
    err = float(torch.linalg.norm(u32.double()[rows] - ref) / torch.linalg.norm(ref))
    assert err <= TOL32
    u64 = H64 @ b.double()
    assert float(torch.linalg.norm(u32.double() - u64) / torch.linalg.norm(u64)) <= TOL32
    assert H32.device_status() == 0 and H64.device_status() == 0


def test_2pow20_fp64_full_vector_matches_oracle(big):
    """Plain FP64 product at n = 2^20 (interleaved grid): every entry of the
    GPU vector against the oracle's reference-order product (reference
    per-block layout and loop order, src/KernelMatrix.jl:17-45,
    src/algebra.jl:243-277), relative 2-norm <= 1e-12."""
    n, x, y, H64, H32 = big
    b = np.random.default_rng(1234).standard_normal(n)
    Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0, nthreads=os.cpu_count())
    ref = np.zeros(n)
    Ho.mul(ref, b, nthreads=os.cpu_count())
    del Ho
    u = (H64 @ dev(b)).cpu().numpy()
    assert rel(u, ref) <= TOL64


def test_2pow20_beta_fp64_full_vector_matches_oracle():
    """The clustered variant of the same workload: x, y i.i.d. Beta(1/2, 1/2)
    at n = 2^20, sorted, minimum gap 1e-9, seed 21 (the benchmark's points),
    FP64; the whole vector against the oracle at <= 1e-12."""
    n = 1 << 20
    x, y = O.beta_points(n, 21)
    hi = float(max(x[0], y[0], 1.0))
    b = np.random.default_rng(21).standard_normal(n)
    Ho = O.OracleKernelMatrix(O.CAUCHY, x, y, hi, 0.0, hi, 0.0, nthreads=os.cpu_count())
    ref = np.zeros(n)
    Ho.mul(ref, b, nthreads=os.cpu_count())
    st_o = Ho.stats()
    del Ho
    H = hm.KernelMatrix(hm.cauchykernel, x, y, hi, 0.0, hi, 0.0)
    st = H.stats()
    assert (st["n_bary"], st["n_dense"]) == (st_o["bary"], st_o["dense"])
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64
    assert H.device_status() == 0
    H.free()


def _dense_rows_fp64(x, y, B64, rows, chunk=512):
    """FP64 dense rows sum_j 1/(x_i - y_j) B[j, q] for every column q of B:
    the Cauchy kernel block of the sampled rows formed in FP64 on the device
    (one rounding for the difference, one for the reciprocal, as the
    reference evaluates it) and multiplied in FP64, a chunk of rows at a time."""
    xd = torch.tensor(x, device="cuda", dtype=torch.float64)
    yd = torch.tensor(y, device="cuda", dtype=torch.float64)
    out = torch.empty(len(rows), B64.shape[1], device="cuda", dtype=torch.float64)
    for i0 in range(0, len(rows), chunk):
        r = torch.tensor(rows[i0:i0 + chunk], device="cuda")
        K = torch.reciprocal(xd[r][:, None] - yd[None, :])
        out[i0:i0 + chunk] = K @ B64
        del K
    return out


@pytest.mark.parametrize("k", [32, 256])
def test_2pow20_fp32_multi_rhs_every_column(big, k):
    """FP32 storage with a block of k right-hand sides at n = 2^20: every
    column on 4096 sampled rows against the FP64 dense product, <= 1e-6
    relative, with the tensor-core panels on (the default for 16 or more
    right-hand sides) and off (FP32 pipes).  The FP64 dense rows are pinned to
    the oracle's compensated dense rows on one column."""
    n, x, y, H64, H32 = big
    g = torch.Generator(device="cuda").manual_seed(k)
    B = torch.randn(k, n, device="cuda", dtype=torch.float32, generator=g).t()     # column-major n x k
    rows = np.sort(np.random.default_rng(k).choice(n, 4096, replace=False))
    ref = _dense_rows_fp64(x, y, B.double(), rows)
    pin = O.dense_rows(O.CAUCHY, x, y, B[:, 0].double().cpu().numpy(), rows[:64], nthreads=os.cpu_count())
    assert rel(ref[:64, 0].cpu().numpy(), pin) <= 1e-12
    rt = torch.tensor(rows, device="cuda")
    for tc in (True, False):
        H32.set_tensor_cores(tc)
        U = torch.empty(k, n, device="cuda", dtype=torch.float32).t()
        H32.mul(U, B, accumulate=False)
        got = U.index_select(0, rt).double()
        err = torch.linalg.norm(got - ref, dim=0) / torch.linalg.norm(ref, dim=0)
        assert float(err.max()) <= TOL32, (tc, int(err.argmax()), float(err.max()))
        assert H32.device_status() == 0
    H32.set_tensor_cores(True)


def test_repeated_calls_and_streams():
    # the single-launch passes reset their synchronisation words: repeated
    # products, and products on a second stream, give identical results
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    b = torch.randn(n, device="cuda", dtype=torch.float64)
    u1 = H @ b
    for _ in range(5):
        u2 = H @ b
        assert torch.equal(u1, u2)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        u3 = H @ b
    s.synchronize()
    assert torch.equal(u1, u3)
    assert H.device_status() == 0


@pytest.mark.parametrize("kernel,sign", [(O.CAUCHY, -1.0), (O.COULOMB, 1.0), (O.COULOMB_PRIME, -1.0), (O.LOG, 1.0)])
def test_transposed_product(kernel, sign):
    # H^T = the KernelMatrix of (y, x) with the kernel's arguments swapped:
    # f(x, y) = sign * f(y, x) for the example kernels
    rng = np.random.default_rng(31)
    x = np.sort(rng.random(20000))[::-1].copy()
    y = np.sort(rng.random(13000))[::-1].copy()
    H = hm.KernelMatrix(KFUN[kernel], x, y, 1.0, 0.0, 1.0, 0.0)
    v = rng.standard_normal(20000)
    ref = sign * (O.OracleKernelMatrix(kernel, y, x, 1.0, 0.0, 1.0, 0.0) @ v)
    got = (H.T @ dev(v)).cpu().numpy()
    assert rel(got, ref) <= TOL64
    # <H w, v> == <w, H^T v>
    w = dev(rng.standard_normal(13000))
    lhs = float(torch.dot(H @ w, dev(v)))
    rhs = float(torch.dot(w, dev(got)))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


def test_transposed_fp32_multi_rhs():
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    V = torch.randn(4, n, device="cuda", dtype=torch.float32).t()
    U = H.T @ V
    Ho = O.OracleKernelMatrix(O.CAUCHY, y, x, 1.0, 0.0, 1.0, 0.0)
    for q in range(4):
        ref = -(Ho @ V[:, q].double().cpu().numpy().copy())
        assert rel(U[:, q].double().cpu().numpy(), ref) <= TOL32


@pytest.mark.parametrize("dtype,k", [(np.float64, 1), (np.float32, 8)])
def test_batch_matches_instances(dtype, k):
    rng = np.random.default_rng(40)
    xs, ys, boxes = [], [], []
    for i in range(24):
        n = int(np.exp(rng.uniform(np.log(1024), np.log(20000))))
        xs.append(np.sort(rng.random(n))[::-1].copy())
        ys.append(np.sort(rng.random(n))[::-1].copy())
        boxes.append((1.0, 0.0, 1.0, 0.0))
    Hb = hm.KernelMatrixBatch(hm.cauchykernel, xs, ys, boxes, dtype=dtype)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    B = torch.randn(k, Hb.shape[1], device="cuda", dtype=tdt).t()
    U = Hb @ B if k > 1 else Hb @ B[:, 0].contiguous()
    U = U.reshape(Hb.shape[0], k) if k == 1 else U
    for i in (0, 5, 23):
        r0, r1 = Hb.row_offsets[i], Hb.row_offsets[i + 1]
        c0, c1 = Hb.col_offsets[i], Hb.col_offsets[i + 1]
        Ho = O.OracleKernelMatrix(O.CAUCHY, xs[i], ys[i], *boxes[i])
        for q in range(k):
            ref = Ho @ B[c0:c1, q].double().cpu().numpy().copy()
            assert rel(U[r0:r1, q].double().cpu().numpy(), ref) <= (TOL64 if dtype == np.float64 else TOL32)


@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 2), (1, 79), (79, 1), (79, 79), (80, 80), (81, 81),
                                   (40, 200), (159, 161), (160, 160), (320, 321)])
def test_threshold_and_ragged_sizes(nx, ny):
    """One point per side, sizes on either side of the leaf rule (BLOCKSIZE 80:
    all four halves below it, src/KernelMatrix.jl:55) and uneven rectangles:
    the GPU product equals the oracle's, FP64 and FP32."""
    rng = np.random.default_rng(nx * 7919 + ny)
    x = np.sort(rng.random(nx))[::-1].copy()
    y = np.sort(rng.random(ny))[::-1].copy()
    b = rng.standard_normal(ny)
    ref = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    assert rel((H @ dev(b)).cpu().numpy(), ref) <= TOL64
    H32 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    ref32 = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0) @ b.astype(np.float32).astype(np.float64)
    got32 = (H32 @ torch.tensor(b, device="cuda", dtype=torch.float32)).cpu().numpy()
    assert rel(got32, ref32) <= TOL32
    # no right-hand sides: nothing is written
    U = torch.full((nx, 0), 7.0, device="cuda", dtype=torch.float64)
    H.mul(U, torch.zeros((ny, 0), device="cuda", dtype=torch.float64))
    H.free()
    H32.free()


@pytest.mark.parametrize("nx,ny", [(1, 5000), (5000, 1), (3, 4097)])
def test_very_uneven_sizes_raise_like_reference(nx, ny):
    """Very uneven point lists make the reference's recursion split an empty
    range, whose indsplit reads past the end (src/BarycentricMatrix.jl:299-307,
    a BoundsError): the oracle and the GPU build raise IndexError alike."""
    rng = np.random.default_rng(nx * 7919 + ny)
    x = np.sort(rng.random(nx))[::-1].copy()
    y = np.sort(rng.random(ny))[::-1].copy()
    with pytest.raises(IndexError):
        O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    with pytest.raises(IndexError):
        hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("k", [1, 4])
@pytest.mark.parametrize("accumulate", [False, True])
def test_host_product_pinned_and_pageable(dtype, k, accumulate):
    """hm_mul_host with host buffers: a page-locked source is read by the leaf
    stage and a page-locked destination written by the product's last kernel
    directly, pageable ones go through copies; all equal the device product
    bit for bit, call after call."""
    n = 65536
    x, y = O.grid_points(n)
    H = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=dtype)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    g = torch.Generator().manual_seed(k)
    B = torch.randn(k, n, generator=g, dtype=tdt)                    # column-major n x k as k rows
    U0 = torch.randn(k, n, generator=g, dtype=tdt)
    ref = U0.clone().cuda().t()
    H.mul(ref, B.cuda().t(), accumulate=accumulate)
    ref = ref.t().cpu()
    for pinned in (True, False):
        for _ in range(3):                                           # plain call, then graph replays
            hb = B.clone().pin_memory() if pinned else B.clone()
            hu = U0.clone().pin_memory() if pinned else U0.clone()
            H.mul_host(hu.numpy().T, hb.numpy().T, accumulate=accumulate)    # (n, k) Fortran-ordered views
            assert torch.equal(hu, ref), (pinned, k, accumulate)
    H.free()
