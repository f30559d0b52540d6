"""Host planner of the product (no GPU): the block tree must be the
reference's, and the flattened nested-basis tables, executed with numpy,
must reproduce the oracle's product."""
import numpy as np
import pytest

import hierarchicalmatrices as hm
from hierarchicalmatrices import _lib
from oracle import oracle as O
from plan_emulator import emulate


def _cases():
    x, y = O.grid_points(2048)
    yield "grid2048", O.CAUCHY, x, y, (1.0, 0.0, 1.0, 0.0)
    x, y = O.grid_points(4096)
    yield "grid4096", O.CAUCHY, x, y, (1.0, 0.0, 1.0, 0.0)
    x, y = O.beta_points(4096, 11)
    yield "beta4096", O.CAUCHY, x, y, (1.0, 0.0, 1.0, 0.0)
    for fam in ("chebyshev", "quadratic"):
        for k in (O.CAUCHY, O.COULOMB, O.COULOMB_PRIME, O.LOG):
            x, y, box = O.example_points(fam, 1000)
            yield f"{fam}1000_k{k}", k, x, y, box
    rng = np.random.default_rng(5)
    x = np.sort(rng.random(3000))[::-1].copy()
    y = np.sort(rng.random(1700))[::-1].copy()
    yield "uniform_rect", O.CAUCHY, x, y, (1.0, 0.0, 1.0, 0.0)
    x, y = O.grid_points(100)
    yield "small_dense_only", O.CAUCHY, x, y, (1.0, 0.0, 1.0, 0.0)


CASES = list(_cases())


@pytest.mark.parametrize("name,kernel,x,y,box", CASES, ids=[c[0] for c in CASES])
def test_plan_tree_matches_oracle(name, kernel, x, y, box):
    P = _lib.Plan(x, y, *box)
    H = O.OracleKernelMatrix(kernel, x, y, *box)
    st = H.stats()
    assert (P.sizes["n_bary"], P.sizes["n_dense"], P.sizes["depth"]) == (st["bary"], st["dense"], st["depth"])
    assert P.sizes["reference_values"] == st["stored_values"]
    assert P.sizes["dense_values"] == st["dense_values"]


@pytest.mark.parametrize("name,kernel,x,y,box", CASES, ids=[c[0] for c in CASES])
def test_plan_emulation_matches_oracle(name, kernel, x, y, box):
    P = _lib.Plan(x, y, *box)
    b = np.random.default_rng(7).standard_normal(len(y))
    u = O.OracleKernelMatrix(kernel, x, y, *box) @ b
    e = emulate(P, kernel, b)
    assert np.linalg.norm(e - u) / np.linalg.norm(u) <= 1e-13


def test_plan_multi_rhs():
    x, y = O.grid_points(2048)
    P = _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)
    B = np.random.default_rng(8).standard_normal((2048, 3))
    E = emulate(P, O.CAUCHY, B)
    H = O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    for q in range(3):
        u = H @ B[:, q]
        assert np.linalg.norm(E[:, q] - u) / np.linalg.norm(u) <= 1e-13


def test_plan_2pow20_counts():
    # tree of the n = 2^20 interleaved grid: counts of the partition simulation
    x, y = O.grid_points(1 << 20)
    P = _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)
    s = P.sizes
    assert (s["n_bary"], s["n_dense"], s["depth"]) == (98214, 49150, 13)
    assert s["canonical_values"] == 785863520
    assert s["reference_values"] == 1750568800
    assert s["dense_values"] == 49150 * 64 * 64


def test_segments_cover_rows_once():
    x, y = O.beta_points(8192, 3)
    P = _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)
    segs = P.table("segs")
    cov = np.zeros(8192, dtype=np.int64)
    for s in segs:
        cov[s["row0"]:s["row0"] + s["nrows"]] += 1
    assert np.all(cov == 1)
    pieces = P.table("pieces")
    for s in segs:
        ps = pieces[s["piece0"]:s["piece0"] + s["npieces"]]
        assert ps["width"].sum() == s["width"]
        assert s["ld"] >= s["nrows"] and s["ld"] % 4 == 0 and s["poff"] % 32 == 0
        # far-field pieces first; nfar counts their columns (the streaming
        # kernels copy [0, nfar) and [nfar, width) as 16-byte aligned runs)
        far = ps["kind"] != _lib.HM_PIECE_X
        assert not np.any(far[1:] & ~far[:-1])
        assert ps["width"][far].sum() == s["nfar"]


def test_validation_errors():
    x = np.array([0.9, 0.5, 0.1])
    with pytest.raises(hm.HMError) as e:
        _lib.Plan(x[::-1].copy(), x, 1.0, 0.0, 1.0, 0.0)
    assert e.value.status == _lib.HM_ERR_UNSORTED
    with pytest.raises(hm.HMError) as e:
        _lib.Plan(np.array([0.9, np.nan, 0.1]), x, 1.0, 0.0, 1.0, 0.0)
    assert e.value.status == _lib.HM_ERR_NAN
    with pytest.raises(hm.HMError) as e:
        _lib.Plan(x, x, 0.0, 1.0, 1.0, 0.0)
    assert e.value.status == _lib.HM_ERR_BOX
    with pytest.raises(hm.HMError) as e:
        _lib.Plan(x, x, 1.0, 0.0, 1.0, 0.0, rank=33)
    assert e.value.status == _lib.HM_ERR_UNSUPPORTED
    with pytest.raises(IndexError):                  # the reference's BoundsError (indsplit on [])
        _lib.Plan(np.zeros(0), x, 1.0, 0.0, 1.0, 0.0)


def test_bounds_error_like_reference():
    # All points in the upper half at every level: the last cluster empties
    # and the reference's indsplit reads past the end (BoundsError).
    n = 400
    x = np.linspace(0.999, 0.99, n)
    y = np.linspace(0.999, 0.99, n)
    with pytest.raises(IndexError):
        O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    with pytest.raises(IndexError):
        _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)


def test_indsplit_matches_oracle():
    rng = np.random.default_rng(1)
    x = np.sort(rng.random(50))[::-1].copy()
    for s, l, a, b in [(0, 50, 1.0, 0.0), (10, 20, 0.8, 0.2), (5, 0, 1.0, 0.0), (49, 1, 1.0, 0.0)]:
        r1, r2 = hm.indsplit(x, range(s, s + l), a, b)
        (s1, l1), (s2, l2) = O.indsplit(x, s, l, a, b)
        assert (r1.start, len(r1), r2.start, len(r2)) == (s1, l1, s2, l2)
    with pytest.raises(IndexError):
        hm.indsplit(x, range(50, 50), 1.0, 0.0)


def _batch_instances(seed, count, lo=600, hi=5000):
    rng = np.random.default_rng(seed)
    xs, ys, boxes = [], [], []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        m = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        xs.append(np.sort(rng.random(n))[::-1].copy())
        ys.append(np.sort(rng.random(m))[::-1].copy())
        boxes.append((1.0, 0.0, 1.0, 0.0))
    return xs, ys, boxes


def test_batch_plan_emulation_matches_instances():
    xs, ys, boxes = _batch_instances(3, 9)
    P = _lib.batch_plan(xs, ys, boxes)
    assert P.sizes["nx"] == sum(map(len, xs)) and P.sizes["ny"] == sum(map(len, ys))
    b = np.random.default_rng(4).standard_normal(P.sizes["ny"])
    u = emulate(P, O.CAUCHY, b)
    r0 = c0 = 0
    for x, y, box in zip(xs, ys, boxes):
        ref = O.OracleKernelMatrix(O.CAUCHY, x, y, *box) @ b[c0:c0 + len(y)]
        got = u[r0:r0 + len(x)]
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-13
        r0 += len(x)
        c0 += len(y)


def nearest_gap(x, y):
    """min_j |x_i - y_j| for every i (y sorted in either order)."""
    ya = np.sort(y)
    k = np.clip(np.searchsorted(ya, x), 1, len(ya) - 1)
    return np.minimum(np.abs(x - ya[k - 1]), np.abs(x - ya[k]))


@pytest.mark.parametrize("kernel", [O.CAUCHY, O.COULOMB, O.LOG])
def test_row_derivative_matches_finite_differences(kernel):
    # D_x b from the analytic basis / kernel derivatives against central
    # differences of the compressed product with the tree held fixed
    # (Richardson-extrapolated, h = 1e-6); rows depend only on their own point
    rng = np.random.default_rng(6)
    n = 4096
    x = np.sort(rng.random(n))[::-1].copy()
    y = np.sort(rng.random(n))[::-1].copy()
    P = _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)
    b = rng.standard_normal(n)
    d = emulate(P, kernel, b, drow=True)
    h = 1e-6

    def cd(hh):
        return (emulate(P, kernel, b, x=x + hh) - emulate(P, kernel, b, x=x - hh)) / (2 * hh)
    fd = (4 * cd(h / 2) - cd(h)) / 3
    # central differences resolve a row only when its nearest source point is
    # well beyond the step: sample 1024 rows with a gap of at least 20 h
    ok = np.nonzero(nearest_gap(x, y) >= 20 * h)[0]
    sub = rng.choice(ok, 1024, replace=False)
    assert np.linalg.norm(fd[sub] - d[sub]) / np.linalg.norm(d[sub]) <= 1e-5


def test_transposed_row_derivative_is_column_derivative():
    # D_y^T r (row derivative of the transposed plan) equals the column
    # derivative of the forward product: sum_i r_i dH_ij/dy_j
    rng = np.random.default_rng(8)
    n = 3000
    x = np.sort(rng.random(n))[::-1].copy()
    y = np.sort(rng.random(n))[::-1].copy()
    PT = _lib.Plan(y, x, 1.0, 0.0, 1.0, 0.0)
    r = rng.standard_normal(n)
    d = emulate(PT, O.CAUCHY, r, drow=True, swap=True)
    ref = (O.kernel_dense(O.CAUCHY, x, y) ** 2).T @ r     # d/dy 1/(x - y) = 1/(x - y)^2
    assert np.linalg.norm(d - ref) / np.linalg.norm(ref) <= 1e-12


def test_empty_and_tiny_inputs_like_reference():
    # src/KernelMatrix.jl:49-50 runs indsplit first, which reads x[first(ir)]
    # (src/BarycentricMatrix.jl:299-307): an empty point list is a BoundsError,
    # as in the oracle; a single point on each side is one dense leaf
    one = np.array([0.25])
    for x, y in ((np.zeros(0), one), (one, np.zeros(0))):
        with pytest.raises(IndexError):
            _lib.Plan(x, y, 1.0, 0.0, 1.0, 0.0)
        with pytest.raises(Exception):
            O.OracleKernelMatrix(O.CAUCHY, x, y, 1.0, 0.0, 1.0, 0.0)
    P = _lib.Plan(np.array([0.75]), np.array([0.25]), 1.0, 0.0, 1.0, 0.0)
    assert P.sizes["nx"] == 1 and len(P.table("segs")) == 1
    assert emulate(P, O.CAUCHY, np.array([2.0]))[0] == 2.0 / (0.75 - 0.25)
