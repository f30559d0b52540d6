"""Gradients of L = 1/2 |H(x, y) w - t|^2 on the GPU (hm_mul_t, hm_mul_drow),
with the block tree held fixed: against the numpy executor of the same plan,
the dense-kernel FP64 gradient and FP64 central differences (h = 1e-6)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import hierarchicalmatrices as hm  # noqa: E402
from hierarchicalmatrices import _lib  # noqa: E402
from hierarchicalmatrices.autograd import kernel_matvec  # noqa: E402
from oracle import oracle as O  # noqa: E402
from plan_emulator import emulate, kernel_dx_np  # noqa: E402
from test_plan import nearest_gap  # noqa: E402


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def uniform_points(n, seed):
    rng = np.random.default_rng(seed)
    return (np.sort(rng.random(n))[::-1].copy(), np.sort(rng.random(n))[::-1].copy())


@pytest.mark.parametrize("kernel,f", [(O.CAUCHY, hm.cauchykernel), (O.COULOMB_PRIME, hm.coulombprimekernel),
                                      (O.LOG, hm.logkernel)])
def test_drow_matches_plan_executor(kernel, f):
    x, y = uniform_points(16384, 2)
    H = hm.KernelMatrix(f, x, y, 1.0, 0.0, 1.0, 0.0)
    b = np.random.default_rng(3).standard_normal(16384)
    u = torch.empty(16384, device="cuda", dtype=torch.float64)
    H.mul_drow(u, torch.tensor(b, device="cuda"), accumulate=False)
    ref = emulate(_lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0), kernel, b, drow=True)
    assert rel(u.cpu().numpy(), ref) <= 1e-12
    v = torch.empty(16384, device="cuda", dtype=torch.float64)
    H.mul_drow(v, torch.tensor(b, device="cuda"), transposed=True, accumulate=False)
    reft = emulate(_lib.Plan(y, x, 1.0, 0.0, 1.0, 0.0), kernel, b, drow=True, swap=True)
    assert rel(v.cpu().numpy(), reft) <= 1e-12


@pytest.fixture(scope="module")
def grad_case():
    # differentiation workload: n = 65536 uniform sorted points, w, t ~ N(0,1),
    # FP32 forward
    n = 65536
    x, y = uniform_points(n, 5)
    rng = np.random.default_rng(6)
    w = rng.standard_normal(n)
    t = rng.standard_normal(n)
    H32 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0, dtype=np.float32)
    H64 = hm.KernelMatrix(hm.cauchykernel, x, y, 1.0, 0.0, 1.0, 0.0)
    return n, x, y, w, t, H32, H64


def test_grad_fp32_against_dense_fp64(grad_case):
    n, x, y, w, t, H32, H64 = grad_case
    loss, gw, gx, gy = H32.loss_and_grad(torch.tensor(w, device="cuda", dtype=torch.float32),
                                         torch.tensor(t, device="cuda", dtype=torch.float32))
    r = (H64 @ torch.tensor(w, device="cuda")).cpu().numpy() - t       # dense-accurate to ~1e-14
    rng = np.random.default_rng(7)
    rows = rng.choice(n, 512, replace=False)
    cols = rng.choice(n, 512, replace=False)
    gx_ref = r[rows] * (kernel_dx_np(O.CAUCHY, x[rows][:, None], y[None, :]) @ w)
    K_cols = O.kernel_dense(O.CAUCHY, x, y[cols])                          # n x 512
    gw_ref = K_cols.T @ r
    gy_ref = w[cols] * ((K_cols ** 2).T @ r)                               # d/dy 1/(x-y) = 1/(x-y)^2
    assert abs(loss - 0.5 * float(r @ r)) <= 1e-5 * abs(loss)
    assert rel(gx.double().cpu().numpy()[rows], gx_ref) <= 1e-5
    assert rel(gw.double().cpu().numpy()[cols], gw_ref) <= 1e-5
    assert rel(gy.double().cpu().numpy()[cols], gy_ref) <= 1e-5


@pytest.fixture(scope="module")
def central_differences(grad_case):
    """FP64 central differences (h = 1e-6, Richardson-extrapolated) of L with
    the block tree held fixed, on 1024 rows and 1024 columns whose nearest
    point of the other side is at least 20 h away.  dL/dx_i = r_i d(row_i . w)/dx_i
    and dL/dy_j = w_j d(col_j . r)/dy_j: a row of H (a row of H^T, the
    KernelMatrix of (y, x) with swapped arguments) depends only on its own
    point, so one shifted product per step gives every row's quotient."""
    n, x, y, w, t, H32, H64 = grad_case
    P = _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)
    PT = _lib.Plan(y, x, 1.0, 0.0, 1.0, 0.0)
    r = emulate(P, O.CAUCHY, w) - t
    h = 1e-6

    def cdx(hh):
        return (emulate(P, O.CAUCHY, w, x=x + hh) - emulate(P, O.CAUCHY, w, x=x - hh)) / (2 * hh)

    def cdy(hh):
        return (emulate(PT, O.CAUCHY, r, swap=True, x=y + hh)
                - emulate(PT, O.CAUCHY, r, swap=True, x=y - hh)) / (2 * hh)
    fdx = r * (4 * cdx(h / 2) - cdx(h)) / 3
    fdy = w * (4 * cdy(h / 2) - cdy(h)) / 3
    rng = np.random.default_rng(8)
    subx = rng.choice(np.nonzero(nearest_gap(x, y) >= 20 * h)[0], 1024, replace=False)
    suby = rng.choice(np.nonzero(nearest_gap(y, x) >= 20 * h)[0], 1024, replace=False)
    return fdx, fdy, subx, suby


def test_grad_fp64_against_central_differences(grad_case, central_differences):
    n, x, y, w, t, H32, H64 = grad_case
    fdx, fdy, subx, suby = central_differences
    loss, gw, gx, gy = H64.loss_and_grad(torch.tensor(w, device="cuda"), torch.tensor(t, device="cuda"))
    assert rel(gx.cpu().numpy()[subx], fdx[subx]) <= 1e-5
    assert rel(gy.cpu().numpy()[suby], fdy[suby]) <= 1e-5


def test_grad_fp32_forward_against_central_differences(grad_case, central_differences):
    """The FP32 forward (FP32 factors from FP64 compression, FP32 w and t):
    dL/dx and dL/dy against the same FP64 central differences, <= 1e-5."""
    n, x, y, w, t, H32, H64 = grad_case
    fdx, fdy, subx, suby = central_differences
    loss, gw, gx, gy = H32.loss_and_grad(torch.tensor(w, device="cuda", dtype=torch.float32),
                                         torch.tensor(t, device="cuda", dtype=torch.float32))
    assert rel(gx.double().cpu().numpy()[subx], fdx[subx]) <= 1e-5
    assert rel(gy.double().cpu().numpy()[suby], fdy[suby]) <= 1e-5


def test_autograd_function(grad_case):
    n, x, y, w, t, H32, H64 = grad_case
    wt = torch.tensor(w, device="cuda", requires_grad=True)
    xt = torch.tensor(x, device="cuda", requires_grad=True)
    yt = torch.tensor(y, device="cuda", requires_grad=True)
    tt = torch.tensor(t, device="cuda")
    loss = 0.5 * ((kernel_matvec(H64, wt, xt, yt) - tt) ** 2).sum()
    loss.backward()
    l2, gw, gx, gy = H64.loss_and_grad(wt.detach(), tt)
    assert abs(loss.detach().item() - l2) <= 1e-12 * abs(l2)
    for a, b in ((wt.grad, gw), (xt.grad, gx), (yt.grad, gy)):
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) <= 1e-14
