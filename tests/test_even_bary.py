"""EvenBarycentricMatrix (src/BarycentricMatrix.jl:5-58, product
src/algebra.jl:168-239): the host factors against the oracle's restatement,
the oracle's reference-order product against the dense operator, and the GPU
product (two stride-2 low-rank products) against the oracle."""
import numpy as np
import pytest

import hierarchicalmatrices as hm
from oracle import oracle as O


def kern(T, x, j):
    # smooth in x over the row interval, columns on a disjoint integer range
    return 1.0 / (x - j) + 0.25 * np.cos(0.01 * j)


BOX = (1, 97, 240, 311)          # rows a:b, columns c:d (odd and even sizes)


def test_factors_match_oracle():
    a, b, c, d = BOX
    W, F = hm.EvenBarycentricMatrix.factors(kern, a, b, c, d, 20)
    Wo, Fo = O.even_bary_factors(kern, a, b, c, d, 20)
    np.testing.assert_array_equal(W, Wo)
    np.testing.assert_array_equal(F, Fo)


@pytest.mark.parametrize("istart,jstart", [(1, 1), (2, 1), (1, 4), (5, 8)])
def test_oracle_product_is_the_parity_operator(istart, jstart):
    a, b, c, d = BOX
    W, F = O.even_bary_factors(kern, a, b, c, d, 20)
    m, p = b - a + 1, d - c + 1
    rng = np.random.default_rng(istart + 10 * jstart)
    v = rng.standard_normal(p + jstart)
    u = np.zeros(m + istart)
    O.even_bary_mul(u, W, F, v, istart, jstart)
    M = (F @ W).T
    ii, jj = np.meshgrid(np.arange(1, m + 1), np.arange(1, p + 1), indexing="ij")
    M = np.where((ii + jj + istart + jstart) % 2 == 0, M, 0.0)
    ref = M @ v[jstart - 1:jstart - 1 + p]
    np.testing.assert_allclose(u[istart - 1:istart - 1 + m], ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    # and the interpolation is the kernel where it couples
    exact = np.array([[kern(np.float64, a + i, c + j) for j in range(p)] for i in range(m)])
    mask = (ii + jj + istart + jstart) % 2 == 0
    assert np.abs((F @ W).T - exact)[mask].max() <= 1e-12 * np.abs(exact).max()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-13), (np.float32, 1e-6)])
@pytest.mark.parametrize("istart,jstart,incx,incy", [(1, 1, 1, 1), (2, 1, 1, 1), (3, 6, 2, 3)])
def test_gpu_product_matches_oracle(dtype, tol, istart, jstart, incx, incy):
    torch = pytest.importorskip("torch")
    a, b, c, d = BOX
    B = hm.EvenBarycentricMatrix(kern, a, b, c, d, dtype=dtype, rank=20)
    m, p = B.shape
    rng = np.random.default_rng(3)
    v = rng.standard_normal(jstart + (p - 1) * incx)
    u0 = rng.standard_normal(istart + (m - 1) * incy)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    u = torch.tensor(u0, device="cuda", dtype=tdt)
    hm.mul_(u, B, torch.tensor(v, device="cuda", dtype=tdt), istart, jstart, incx, incy)
    got = u.double().cpu().numpy()[istart - 1::incy][:m] - u0[istart - 1::incy][:m]
    # the oracle's product (unit strides, as mul! has) on the strided entries
    vv = v[jstart - 1::incx][:p]
    uu = np.zeros(m + istart)
    O.even_bary_mul(uu, B.W, B.F, np.concatenate([np.zeros(jstart - 1), vv]), istart, jstart)
    ref = uu[istart - 1:istart - 1 + m]
    assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref)
