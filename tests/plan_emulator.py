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


def _tasks(plan, which):
    """Transfer tasks in launch order (band by band, task by task): for each,
    its records and the step (level) index of each record within the task."""
    ents = plan.table(f"{which}_ents")
    steps = plan.table(f"{which}_steps")
    tasks = plan.table(f"{which}_tasks")
    bptr = plan.table(f"{which}_band_ptr")
    assert len(ents) == len(plan.table(which))
    for bd in range(len(bptr) - 1):
        for tk in tasks[bptr[bd]:bptr[bd + 1]]:
            recs, lev = [], []
            for j, st in enumerate(steps[tk["step0"]:tk["step1"]]):
                recs.extend(ents[st["e0"]:st["e1"]])
                lev.extend([j] * (st["e1"] - st["e0"]))
            yield recs, lev


def emulate(plan, kernel, b, drow=False, swap=False, x=None, y=None, segments=None):
    """Returns H @ b (b: (ny,) or (ny, k)) computed from the plan tables.
    drow=True: the row-derivative product D b (entries differentiated with
    respect to their row point); swap=True: entries f(col, row) (the
    transposed matrix); x / y replace the plan's points in the entries (the
    tree stays the plan's); segments=(lo, hi) computes only the rows of those
    row segments (the others are 0), as one rank of a row-sharded product."""
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
    # upward transfers task by task with task-local vectors, as the GPU runs
    # them: record i produces local i; its children (locals pad & 0xffff,
    # pad >> 16) were produced at an earlier level of the task or are
    # external (numbered after the records) and final before the launch
    done = np.zeros(S["n_yslots"], dtype=bool)
    done[[vp["slot"] for vp in plan.table("vpanels")]] = True
    for recs, lev in _tasks(plan, "up"):
        nrec, L, made = len(recs), {}, {}
        for e in recs:
            for lc, c in ((int(e["pad"]) & 0xffff, e["c0"]), (int(e["pad"]) >> 16, e["c1"])):
                if lc >= nrec:
                    assert lc not in L and done[c]
                    L[lc], made[lc] = t[c].copy(), -1
        for i, (e, lv) in enumerate(zip(recs, lev)):
            l0, l1 = int(e["pad"]) & 0xffff, int(e["pad"]) >> 16
            assert made[l0] < lv and made[l1] < lv and not done[e["slot"]]
            L[i], made[i] = T[0].T @ L[l0] + T[1].T @ L[l1], lv
            t[e["slot"]] = L[i]
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
    # downward transfers task by task with task-local vectors: record i's
    # children are locals 2i, 2i + 1 (starting from their far-field values);
    # its parent (local pad) is a child of an earlier level of the task or
    # external, and then final (pushed by its own parent) before the launch
    pushed = np.zeros(S["n_xslots"], dtype=bool)
    has_parent = np.zeros(S["n_xslots"], dtype=bool)
    for e in plan.table("down"):
        has_parent[e["c0"]] = has_parent[e["c1"]] = True
    for recs, lev in _tasks(plan, "down"):
        nrec, L, made = len(recs), {}, {}
        for i, e in enumerate(recs):
            L[2 * i], L[2 * i + 1] = s[e["c0"]].copy(), s[e["c1"]].copy()
            lp = int(e["pad"])
            if lp >= 2 * nrec:
                assert lp not in L and (pushed[e["slot"]] or not has_parent[e["slot"]])
                L[lp], made[lp] = s[e["slot"]].copy(), -1
        for i, (e, lv) in enumerate(zip(recs, lev)):
            lp = int(e["pad"])
            assert made[lp] < lv
            L[2 * i] = L[2 * i] + T[0] @ L[lp]
            L[2 * i + 1] = L[2 * i + 1] + T[1] @ L[lp]
            made[2 * i] = made[2 * i + 1] = lv
            s[e["c0"]], s[e["c1"]] = L[2 * i], L[2 * i + 1]
            pushed[e["c0"]] = pushed[e["c1"]] = True
    # row segments
    out = np.zeros((S["nx"], k))
    covered = np.zeros(S["nx"], dtype=np.int64)
    pieces, sf = plan.table("pieces"), plan.table("seg_fill")
    seg_lo, seg_hi = segments if segments is not None else (0, len(sf))
    for j, (sg, fi) in enumerate(zip(plan.table("segs"), sf)):
        rows = slice(sg["row0"], sg["row0"] + sg["nrows"])
        covered[rows] += 1
        if not seg_lo <= j < seg_hi:
            continue
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
