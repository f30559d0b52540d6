"""numpy executor of the product's plan tables (test infrastructure).

Runs the fill and matvec stages of csrc/hm_kernels.cu on the host tables
returned by hm_plan_create, in FP64, so the planner and the nested-basis
algebra can be checked against the oracle without a GPU.
"""
import numpy as np


def box_nodes(a, b, cheb):
    ab2 = 0.5 * (a + b)
    ba2 = 0.5 * (b - a)
    return ab2 + ba2 * cheb


def kernel_dx_np(kernel, x, y):
    d = x - y
    if kernel == 0:
        return -1.0 / (d * d)
    if kernel == 1:
        return -2.0 / ((d * d) * d)
    if kernel == 2:
        return -3.0 / ((d * d) * (d * d))
    return 1.0 / d


def basis_drow(pts, a, b, cheb, lam):
    nodes = box_nodes(a, b, cheb)
    diff = pts[:, None] - nodes[None, :]
    U = basis(pts, a, b, cheb, lam)
    sd = (U / diff).sum(axis=1, keepdims=True)
    return U * (sd - 1.0 / diff)


def kernel_np(kernel, x, y):
    d = x - y
    if kernel == 0:
        return 1.0 / d
    if kernel == 1:
        return 1.0 / (d * d)
    if kernel == 2:
        return 1.0 / ((d * d) * d)
    return np.log(np.abs(d))


def basis(pts, a, b, cheb, lam):
    nodes = box_nodes(a, b, cheb)
    w = lam[None, :] * (1.0 / (pts[:, None] - nodes[None, :]))
    return w / w.sum(axis=1, keepdims=True)


def _banded(plan, which):
    """Transfer records in launch order: band by band, task by task, step by step."""
    ents = plan.table(f"{which}_ents")
    steps = plan.table(f"{which}_steps")
    tasks = plan.table(f"{which}_tasks")
    bptr = plan.table(f"{which}_band_ptr")
    assert len(ents) == len(plan.table(which))
    for bd in range(len(bptr) - 1):
        for tk in tasks[bptr[bd]:bptr[bd + 1]]:
            for st in steps[tk["step0"]:tk["step1"]]:
                yield from ents[st["e0"]:st["e1"]]


def emulate(plan, kernel, b, drow=False, swap=False, x=None, y=None):
    """Returns H @ b (b: (ny,) or (ny, k)) computed from the plan tables.
    drow=True: the row-derivative product D b (entries differentiated with
    respect to their row point); swap=True: entries f(col, row) (the
    transposed matrix); x / y replace the plan's points in the entries (the
    tree stays the plan's)."""
    S = plan.sizes
    r = S["r"]
    x = plan.x if x is None else np.asarray(x, dtype=np.float64)
    y = plan.y if y is None else np.asarray(y, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    squeeze = b.ndim == 1
    B = b[:, None] if squeeze else b
    k = B.shape[1]
    cheb, lam = plan.table("cheb"), plan.table("lam")
    T = plan.table("T").reshape(2, r, r)           # T[c][m', m]
    t = np.zeros((S["n_yslots"], r, k))
    s = np.zeros((S["n_xslots"], r, k))
    # explicit column bases -> leaf coefficients
    for vp, vf in zip(plan.table("vpanels"), plan.table("vpanel_fill")):
        rows = slice(vp["row0"], vp["row0"] + vp["nrows"])
        V = basis(y[rows], vf["a"], vf["b"], cheb, lam)
        t[vp["slot"]] = V.T @ B[rows]
    # upward transfers in band / task / step order (as the GPU runs them);
    # `done` checks that every child is final before its parent reads it
    done = np.zeros(S["n_yslots"], dtype=bool)
    done[[vp["slot"] for vp in plan.table("vpanels")]] = True
    for e in _banded(plan, "up"):
        assert done[e["c0"]] and done[e["c1"]] and not done[e["slot"]]
        t[e["slot"]] = T[0].T @ t[e["c0"]] + T[1].T @ t[e["c1"]]
        done[e["slot"]] = True
    # far field
    ents, ff = plan.table("m2l_ents"), plan.table("f_fill")
    for row in plan.table("m2l_rows"):
        acc = np.zeros((r, k))
        for e in range(row["begin"], row["end"]):
            f = ff[e]
            xn = box_nodes(f["xa"], f["xb"], cheb)[:, None]
            yn = box_nodes(f["ya"], f["yb"], cheb)[None, :]
            F = kernel_np(kernel, yn, xn) if swap else kernel_np(kernel, xn, yn)
            acc += F @ t[ents[e]["yslot"]]
        s[row["slot"]] = acc
    # downward transfers in band / task / step order; a parent is final once
    # its own parent has pushed into it
    pushed = np.zeros(S["n_xslots"], dtype=bool)
    has_parent = np.zeros(S["n_xslots"], dtype=bool)
    for e in plan.table("down"):
        has_parent[e["c0"]] = has_parent[e["c1"]] = True
    for e in _banded(plan, "down"):
        assert pushed[e["slot"]] or not has_parent[e["slot"]]
        s[e["c0"]] += T[0] @ s[e["slot"]]
        s[e["c1"]] += T[1] @ s[e["slot"]]
        pushed[e["c0"]] = pushed[e["c1"]] = True
    # row segments
    out = np.zeros((S["nx"], k))
    covered = np.zeros(S["nx"], dtype=np.int64)
    pieces, sf = plan.table("pieces"), plan.table("seg_fill")
    for sg, fi in zip(plan.table("segs"), sf):
        rows = slice(sg["row0"], sg["row0"] + sg["nrows"])
        covered[rows] += 1
        cols, g = [], []
        for p in pieces[sg["piece0"]:sg["piece0"] + sg["npieces"]]:
            if p["kind"] == 0:
                bf = basis_drow if drow else basis
                cols.append(bf(x[rows], fi["a"], fi["b"], cheb, lam))
                g.append(s[p["src"]])
            else:
                yy = y[p["src"]:p["src"] + p["width"]]
                xr = x[rows][:, None]
                if drow:
                    blk = -kernel_dx_np(kernel, yy[None, :], xr) if swap else kernel_dx_np(kernel, xr, yy[None, :])
                else:
                    blk = kernel_np(kernel, yy[None, :], xr) if swap else kernel_np(kernel, xr, yy[None, :])
                cols.append(blk)
                g.append(B[p["src"]:p["src"] + p["width"]])
        if cols:
            P = np.concatenate(cols, axis=1)
            assert P.shape[1] == sg["width"]
            out[rows] = P @ np.concatenate(g, axis=0)
    assert np.all(covered == 1), "every row must be in exactly one segment"
    return out[:, 0] if squeeze else out
