// Host planner for KernelMatrix: block tree + nested cluster bases.
//
// The block tree is the reference's (src/KernelMatrix.jl:49-116): a pair of
// clusters is split at the box midpoints (indsplit, src/BarycentricMatrix.jl:
// 299-307, points >= midpoint go first); diagonal pairs recurse, off-diagonal
// pairs produce three barycentric children and recurse on the child whose
// boxes touch; a pair becomes a leaf when all four halves hold fewer than
// BLOCKSIZE points.
//
// The representation differs from the reference's: each barycentric block
// of the reference stores its own U = Lagrange basis of its row box at the
// row points and V likewise.  Because the boxes are nested halvings and the
// basis is degree r-1 polynomial interpolation at Chebyshev points, the basis
// of a box restricted to a child box equals the child's basis times one of two
// fixed r x r transfer matrices.  So only the deepest boxes store explicit
// bases; coarser coefficients move through the transfer matrices.  The
// product is the same matrix up to rounding (the tests bound the difference).
#include "hm_plan.h"

#include <algorithm>

namespace hm {

static Node make_node(int64_t lo, int64_t hi, double a, double b, int level, int parent)
{
    Node n;
    n.lo = lo; n.hi = hi; n.a = a; n.b = b; n.level = level; n.parent = parent;
    n.child[0] = n.child[1] = -1;
    n.used = n.sub_used = false;
    n.kind = 0; n.slot = -1;
    return n;
}

void Tree::init(const double *pts, int64_t npts, double a, double b)
{
    x = pts; n = npts;
    nodes.clear();
    nodes.push_back(make_node(0, npts, a, b, 0, -1));
}

int Tree::split(int id)
{
    if (nodes[id].child[0] >= 0) return PLAN_OK;
    const int64_t lo = nodes[id].lo, hi = nodes[id].hi;
    const double a = nodes[id].a, b = nodes[id].b;
    const double mid = 0.5 * (a + b);
    int64_t s;
    if (lo >= hi) {
        // An empty range: the reference still reads x[first(ir)].
        if (lo >= n) return PLAN_ERR_BOUNDS;
        if (x[lo] >= mid) return PLAN_ERR_DEGENERATE;
        s = lo;
    } else {
        // First index with !(x[i] >= mid); x is non-increasing, so the
        // reference's linear scan and this binary search agree.
        int64_t L = lo, R = hi;
        while (L < R) {
            int64_t M = L + (R - L) / 2;
            if (x[M] >= mid) L = M + 1; else R = M;
        }
        s = L;
    }
    const int lev = nodes[id].level + 1;
    int c0 = (int)nodes.size();
    nodes.push_back(make_node(lo, s, a, mid, lev, id));
    nodes.push_back(make_node(s, std::max(s, hi), mid, b, lev, id));
    nodes[id].child[0] = c0;
    nodes[id].child[1] = c0 + 1;
    return PLAN_OK;
}

namespace {

struct Builder {
    Plan &P;
    int64_t leaf;
    int err = 0;
    int64_t depth = 0;

    void rec(int kind, int xn, int yn)
    {
        if (err) return;
        int e = P.X.split(xn);
        if (!e) e = P.Y.split(yn);
        if (e) { err = e; return; }
        depth = std::max<int64_t>(depth, P.X.nodes[xn].level);
        const int x1 = P.X.nodes[xn].child[0], x2 = P.X.nodes[xn].child[1];
        const int y1 = P.Y.nodes[yn].child[0], y2 = P.Y.nodes[yn].child[1];
        const bool lf = P.X.size(x1) < leaf && P.X.size(x2) < leaf &&
                        P.Y.size(y1) < leaf && P.Y.size(y2) < leaf;
        if (kind == 0) {            // KernelMatrix, src/KernelMatrix.jl:49-70
            if (lf) {
                P.dense.push_back({x1, y1}); P.dense.push_back({x1, y2});
                P.dense.push_back({x2, y1}); P.dense.push_back({x2, y2});
            } else {
                rec(0, x1, y1); rec(1, x1, y2); rec(2, x2, y1); rec(0, x2, y2);
            }
        } else if (kind == 1) {     // KernelMatrix1, src/KernelMatrix.jl:72-93
            P.bary.push_back({x1, y1}); P.bary.push_back({x1, y2});
            if (lf) P.dense.push_back({x2, y1}); else rec(1, x2, y1);
            P.bary.push_back({x2, y2});
        } else {                    // KernelMatrix2, src/KernelMatrix.jl:95-116
            P.bary.push_back({x1, y1});
            if (lf) P.dense.push_back({x1, y2}); else rec(2, x1, y2);
            P.bary.push_back({x2, y1}); P.bary.push_back({x2, y2});
        }
    }
};

void mark_sub_used(Tree &T)
{
    for (size_t i = 0; i < T.nodes.size(); ++i) {
        if (!T.nodes[i].used) continue;
        int p = T.nodes[i].parent;
        while (p >= 0 && !T.nodes[p].sub_used) {
            T.nodes[p].sub_used = true;
            p = T.nodes[p].parent;
        }
    }
}

void assign_basis(Tree &T, int id, bool above)
{
    const bool inb = above || T.nodes[id].used;
    if (T.nodes[id].sub_used) {
        assign_basis(T, T.nodes[id].child[0], inb);
        assign_basis(T, T.nodes[id].child[1], inb);
        if (inb) T.nodes[id].kind = 1;
    } else if (inb) {
        T.nodes[id].kind = 2;
    }
}

// Slots in (level, lo) order; returns the slot count.
int assign_slots(Tree &T)
{
    std::vector<int> ids;
    for (size_t i = 0; i < T.nodes.size(); ++i)
        if (T.nodes[i].kind) ids.push_back((int)i);
    std::sort(ids.begin(), ids.end(), [&](int u, int v) {
        if (T.nodes[u].level != T.nodes[v].level) return T.nodes[u].level < T.nodes[v].level;
        if (T.nodes[u].lo != T.nodes[v].lo) return T.nodes[u].lo < T.nodes[v].lo;
        return u < v;
    });
    for (size_t k = 0; k < ids.size(); ++k) T.nodes[ids[k]].slot = (int)k;
    return (int)ids.size();
}

// Transfer steps for the internal basis nodes, grouped by level.
void transfer_steps(const Tree &T, bool deepest_first, std::vector<hm_xfer> &out,
                    std::vector<int> &ptr)
{
    int maxlev = 0;
    for (const Node &n : T.nodes) if (n.kind == 1) maxlev = std::max(maxlev, n.level);
    std::vector<std::vector<hm_xfer>> by(maxlev + 1);
    for (const Node &n : T.nodes)
        if (n.kind == 1)
            by[n.level].push_back({n.slot, T.nodes[n.child[0]].slot, T.nodes[n.child[1]].slot, 0});
    out.clear(); ptr.clear();
    ptr.push_back(0);
    for (int k = 0; k <= maxlev; ++k) {
        int lev = deepest_first ? maxlev - k : k;
        auto &v = by[lev];
        if (v.empty()) continue;
        std::sort(v.begin(), v.end(), [](const hm_xfer &p, const hm_xfer &q) { return p.slot < q.slot; });
        out.insert(out.end(), v.begin(), v.end());
        ptr.push_back((int)out.size());
    }
}

inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// Groups the internal basis nodes into bands of kBandLevels levels (counted
// from the deepest internal level).  Within a band, a task is the set of
// nodes sharing the same topmost in-band ancestor; its steps are its levels,
// deepest first for the upward pass, topmost first for the downward pass.
void band_transfers(const Tree &T, bool upward, std::vector<hm_xfer> &ents, std::vector<hm_step> &steps,
                    std::vector<hm_task> &tasks, std::vector<int> &band_ptr)
{
    ents.clear(); steps.clear(); tasks.clear(); band_ptr.clear();
    int maxlev = -1;
    for (const Node &n : T.nodes) if (n.kind == 1) maxlev = std::max(maxlev, n.level);
    band_ptr.push_back(0);
    if (maxlev < 0) return;
    const int nbands = maxlev / kBandLevels + 1;
    auto band_of = [&](int level) { return (maxlev - level) / kBandLevels; };
    // task root of every internal node: climb while the parent is internal and in the same band
    std::vector<std::vector<std::pair<int, int>>> members(nbands);   // (root id, node id)
    for (size_t i = 0; i < T.nodes.size(); ++i) {
        if (T.nodes[i].kind != 1) continue;
        int root = (int)i;
        const int b = band_of(T.nodes[i].level);
        while (T.nodes[root].parent >= 0 && T.nodes[T.nodes[root].parent].kind == 1 &&
               band_of(T.nodes[T.nodes[root].parent].level) == b)
            root = T.nodes[root].parent;
        members[b].push_back({root, (int)i});
    }
    for (int k = 0; k < nbands; ++k) {
        const int b = upward ? k : nbands - 1 - k;
        auto &mem = members[b];
        std::sort(mem.begin(), mem.end(), [&](const std::pair<int, int> &p, const std::pair<int, int> &q) {
            if (p.first != q.first) return T.nodes[p.first].slot < T.nodes[q.first].slot;
            const int lp = T.nodes[p.second].level, lq = T.nodes[q.second].level;
            if (lp != lq) return upward ? lp > lq : lp < lq;
            return T.nodes[p.second].slot < T.nodes[q.second].slot;
        });
        for (size_t i = 0; i < mem.size(); ++i) {
            const Node &n = T.nodes[mem[i].second];
            const bool new_task = i == 0 || mem[i].first != mem[i - 1].first;
            const bool new_step = new_task || n.level != T.nodes[mem[i - 1].second].level;
            if (new_task) tasks.push_back({(int32_t)steps.size(), (int32_t)steps.size()});
            if (new_step) {
                steps.push_back({(int32_t)ents.size(), (int32_t)ents.size()});
                tasks.back().step1 = (int32_t)steps.size();
            }
            ents.push_back({n.slot, T.nodes[n.child[0]].slot, T.nodes[n.child[1]].slot, 0});
            steps.back().e1 = (int32_t)ents.size();
        }
        band_ptr.push_back((int)tasks.size());
    }
    // Task-local numbering, so a task keeps its coefficients in shared memory:
    // upward, record i of a task produces local i and its children are either
    // produced earlier in the task or external (numbered after the records);
    // pad = local(c0) | local(c1) << 16.  Downward, record i's children are
    // locals 2i and 2i + 1 and its parent is an earlier child or external
    // (numbered after the children); pad = local(parent).
    for (const hm_task &tk : tasks) {
        const int e0 = steps[tk.step0].e0, e1 = steps[tk.step1 - 1].e1;
        const int nrec = e1 - e0;
        std::vector<std::pair<int32_t, int32_t>> made;     // (slot, local), small per task
        auto find = [&](int32_t slot) {
            for (auto &m : made) if (m.first == slot) return m.second;
            return -1;
        };
        int next = 0;
        for (int e = e0; e < e1; ++e) {
            hm_xfer &X = ents[e];
            if (upward) {
                int l0 = find(X.c0), l1 = find(X.c1);
                if (l0 < 0) l0 = nrec + next++;
                if (l1 < 0) l1 = nrec + next++;
                X.pad = l0 | (l1 << 16);
                made.push_back({X.slot, e - e0});
            } else {
                int lp = find(X.slot);
                if (lp < 0) lp = 2 * nrec + next++;
                X.pad = lp;
                made.push_back({X.c0, 2 * (e - e0)});
                made.push_back({X.c1, 2 * (e - e0) + 1});
            }
        }
    }
}

}  // namespace

int build_plan(const double *x, int64_t nx, const double *y, int64_t ny, double a, double b,
               double c, double d, int r, int64_t leaf, int seg_rows, Plan &P)
{
    P = Plan();
    P.r = r; P.nx = nx; P.ny = ny;
    P.X.init(x, nx, a, b);
    P.Y.init(y, ny, c, d);
    Builder B{P, leaf};
    B.rec(0, 0, 0);
    if (B.err) return B.err;

    for (auto &e : P.bary) { P.X.nodes[e.first].used = true; P.Y.nodes[e.second].used = true; }
    mark_sub_used(P.X);
    mark_sub_used(P.Y);
    assign_basis(P.X, 0, false);
    assign_basis(P.Y, 0, false);
    P.n_xslots = assign_slots(P.X);
    P.n_yslots = assign_slots(P.Y);
    transfer_steps(P.Y, true, P.up, P.up_level_ptr);
    transfer_steps(P.X, false, P.down, P.down_level_ptr);

    // Explicit column bases at the deepest basis nodes of the column tree.
    {
        std::vector<int> leaves;
        for (size_t i = 0; i < P.Y.nodes.size(); ++i)
            if (P.Y.nodes[i].kind == 2) leaves.push_back((int)i);
        std::sort(leaves.begin(), leaves.end(),
                  [&](int u, int v) { return P.Y.nodes[u].slot < P.Y.nodes[v].slot; });
        int64_t off = 0;
        for (int id : leaves) {
            const Node &n = P.Y.nodes[id];
            hm_vpanel vp;
            vp.row0 = n.lo;
            vp.nrows = (int32_t)(n.hi - n.lo);
            vp.ld = r;                         // row-major: r values per point
            vp.width = r;
            vp.slot = n.slot;
            vp.col0 = 0;
            vp.pad = 0;
            vp.off = off;
            off += round_up((int64_t)vp.nrows * r, 32);
            P.vpanels.push_back(vp);
            P.vpanel_fill.push_back({n.a, n.b});
        }
        P.vstore_elems = off;
    }

    band_transfers(P.Y, true, P.up_ents, P.up_steps, P.up_tasks, P.up_band_ptr);
    band_transfers(P.X, false, P.down_ents, P.down_steps, P.down_tasks, P.down_band_ptr);

    // M2L rows: barycentric blocks grouped by row cluster.
    P.fstride = (int)round_up((int64_t)r * r, 4);
    {
        std::vector<std::pair<int, int>> bs;   // (xslot, index into bary)
        for (size_t i = 0; i < P.bary.size(); ++i)
            bs.push_back({P.X.nodes[P.bary[i].first].slot, (int)i});
        std::sort(bs.begin(), bs.end(), [&](const std::pair<int, int> &p, const std::pair<int, int> &q) {
            if (p.first != q.first) return p.first < q.first;
            return P.Y.nodes[P.bary[p.second].second].slot < P.Y.nodes[P.bary[q.second].second].slot;
        });
        // One row per row-basis slot (slots without blocks get empty ranges, so
        // the far-field pass writes every coefficient).
        for (int sl = 0; sl < P.n_xslots; ++sl) P.m2l_rows.push_back({sl, 0, 0, 0});
        for (size_t k = 0; k < bs.size(); ++k) {
            const int xn = P.bary[bs[k].second].first, yn = P.bary[bs[k].second].second;
            hm_m2l_row &row = P.m2l_rows[bs[k].first];
            if (row.end == 0) row.begin = (int32_t)k;
            row.end = (int32_t)(k + 1);
            hm_m2l_ent e;
            e.foff = (int64_t)k * P.fstride;
            e.yslot = P.Y.nodes[yn].slot;
            e.pad = 0;
            P.m2l_ents.push_back(e);
            P.f_fill.push_back({P.X.nodes[xn].a, P.X.nodes[xn].b, P.Y.nodes[yn].a, P.Y.nodes[yn].b});
        }
        P.fstore_elems = (int64_t)bs.size() * P.fstride;
    }

    // Row segments: elementary row intervals of {row-basis leaves, dense rows}.
    {
        std::vector<int> xleaves;
        for (size_t i = 0; i < P.X.nodes.size(); ++i)
            if (P.X.nodes[i].kind == 2 && P.X.size((int)i) > 0) xleaves.push_back((int)i);
        std::sort(xleaves.begin(), xleaves.end(),
                  [&](int u, int v) { return P.X.nodes[u].lo < P.X.nodes[v].lo; });
        std::vector<int64_t> cuts = {0, nx};
        for (int id : xleaves) { cuts.push_back(P.X.nodes[id].lo); cuts.push_back(P.X.nodes[id].hi); }
        for (auto &e : P.dense) {
            if (P.X.size(e.first) == 0 || P.Y.size(e.second) == 0) continue;
            cuts.push_back(P.X.nodes[e.first].lo);
            cuts.push_back(P.X.nodes[e.first].hi);
        }
        std::sort(cuts.begin(), cuts.end());
        cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
        const size_t nint = cuts.size() - 1;
        std::vector<std::vector<int>> dl(nint);
        for (size_t k = 0; k < P.dense.size(); ++k) {
            const Node &xn = P.X.nodes[P.dense[k].first];
            if (xn.hi <= xn.lo || P.Y.size(P.dense[k].second) == 0) continue;
            size_t i0 = std::lower_bound(cuts.begin(), cuts.end(), xn.lo) - cuts.begin();
            size_t i1 = std::lower_bound(cuts.begin(), cuts.end(), xn.hi) - cuts.begin();
            for (size_t i = i0; i < i1; ++i) dl[i].push_back((int)k);
        }
        size_t lp = 0;
        int64_t poff = 0;
        for (size_t iv = 0; iv < nint; ++iv) {
            const int64_t p = cuts[iv], q = cuts[iv + 1];
            if (q <= p) continue;
            while (lp < xleaves.size() && P.X.nodes[xleaves[lp]].hi <= p) ++lp;
            int leafid = -1;
            if (lp < xleaves.size() && P.X.nodes[xleaves[lp]].lo <= p) leafid = xleaves[lp];
            auto &ds = dl[iv];
            std::sort(ds.begin(), ds.end(), [&](int u, int v) {
                return P.Y.nodes[P.dense[u].second].lo < P.Y.nodes[P.dense[v].second].lo;
            });
            for (int64_t r0 = p; r0 < q; r0 += seg_rows) {
                hm_seg s;
                s.row0 = r0;
                s.nrows = (int32_t)std::min<int64_t>(seg_rows, q - r0);
                s.ld = (int32_t)round_up(s.nrows, 4);
                s.piece0 = (int32_t)P.pieces.size();
                s.width = 0;
                hm_fill_seg f;
                f.has_basis = 0; f.basis_w = 0; f.a = 0; f.b = 0;
                if (leafid >= 0) {
                    hm_piece pc;
                    pc.kind = HM_PIECE_COEF; pc.src = P.X.nodes[leafid].slot; pc.width = r;
                    P.pieces.push_back(pc);
                    s.width += r;
                    f.has_basis = 1; f.basis_w = r;
                    f.a = P.X.nodes[leafid].a; f.b = P.X.nodes[leafid].b;
                }
                for (int k : ds) {
                    const Node &yn = P.Y.nodes[P.dense[k].second];
                    hm_piece pc;
                    pc.kind = HM_PIECE_X; pc.src = yn.lo; pc.width = (int32_t)(yn.hi - yn.lo);
                    P.pieces.push_back(pc);
                    s.width += pc.width;
                }
                s.npieces = (int32_t)P.pieces.size() - s.piece0;
                s.poff = poff;
                s.nfar = leafid >= 0 ? r : 0;
                poff += round_up((int64_t)s.ld * std::max(s.width, 1), 32);
                P.max_width = std::max(P.max_width, s.width);
                P.segs.push_back(s);
                P.seg_fill.push_back(f);
            }
        }
        P.pstore_elems = poff;
    }

    // Statistics.
    PlanStats &S = P.stats;
    S.n_bary = (int64_t)P.bary.size();
    S.n_dense = (int64_t)P.dense.size();
    S.depth = B.depth;
    S.n_xslots = P.n_xslots; S.n_yslots = P.n_yslots;
    int64_t ux = 0, uy = 0;
    for (const Node &n : P.X.nodes) if (n.used) ux += n.hi - n.lo;
    for (const Node &n : P.Y.nodes) if (n.used) uy += n.hi - n.lo;
    int64_t dv = 0, refv = 0;
    for (auto &e : P.dense) dv += P.X.size(e.first) * P.Y.size(e.second);
    for (auto &e : P.bary) refv += (P.X.size(e.first) + P.Y.size(e.second)) * r + (int64_t)r * r;
    S.dense_values = dv;
    S.canonical_values = (ux + uy) * r + S.n_bary * r * r + dv;
    S.reference_values = refv + dv;
    int64_t st = (int64_t)P.bary.size() * r * r;
    for (auto &v : P.vpanels) st += (int64_t)v.nrows * v.width;
    for (auto &s : P.segs) st += (int64_t)s.nrows * s.width;
    S.stored_values = st;
    S.n_segments = (int64_t)P.segs.size();
    S.max_width = P.max_width;
    return PLAN_OK;
}

namespace {

void merge_bands(const std::vector<Plan> &parts, bool upward, Plan &out)
{
    std::vector<hm_xfer> &ents = upward ? out.up_ents : out.down_ents;
    std::vector<hm_step> &steps = upward ? out.up_steps : out.down_steps;
    std::vector<hm_task> &tasks = upward ? out.up_tasks : out.down_tasks;
    std::vector<int> &bptr = upward ? out.up_band_ptr : out.down_band_ptr;
    size_t nb = 0;
    for (const Plan &p : parts) {
        const std::vector<int> &pb = upward ? p.up_band_ptr : p.down_band_ptr;
        nb = std::max(nb, pb.size() ? pb.size() - 1 : 0);
    }
    bptr.assign(1, 0);
    std::vector<int32_t> xs_off(parts.size()), ys_off(parts.size());
    int32_t xo = 0, yo = 0;
    for (size_t i = 0; i < parts.size(); ++i) { xs_off[i] = xo; ys_off[i] = yo; xo += parts[i].n_xslots; yo += parts[i].n_yslots; }
    for (size_t b = 0; b < nb; ++b) {
        for (size_t i = 0; i < parts.size(); ++i) {
            const Plan &p = parts[i];
            const std::vector<int> &pb = upward ? p.up_band_ptr : p.down_band_ptr;
            if (b + 1 >= pb.size()) continue;
            const std::vector<hm_task> &pt = upward ? p.up_tasks : p.down_tasks;
            const std::vector<hm_step> &ps = upward ? p.up_steps : p.down_steps;
            const std::vector<hm_xfer> &pe = upward ? p.up_ents : p.down_ents;
            const int32_t so = upward ? ys_off[i] : xs_off[i];
            for (int t = pb[b]; t < pb[b + 1]; ++t) {
                hm_task nt{(int32_t)steps.size(), (int32_t)steps.size()};
                for (int st = pt[t].step0; st < pt[t].step1; ++st) {
                    hm_step ns{(int32_t)ents.size(), (int32_t)ents.size()};
                    for (int e = ps[st].e0; e < ps[st].e1; ++e)
                        ents.push_back({pe[e].slot + so, pe[e].c0 + so, pe[e].c1 + so, pe[e].pad});
                    ns.e1 = (int32_t)ents.size();
                    steps.push_back(ns);
                }
                nt.step1 = (int32_t)steps.size();
                tasks.push_back(nt);
            }
        }
        bptr.push_back((int)tasks.size());
    }
}

}  // namespace

void merge_plans(const std::vector<Plan> &parts, Plan &P)
{
    P = Plan();
    if (parts.empty()) return;
    P.r = parts[0].r;
    P.fstride = parts[0].fstride;
    int64_t row0 = 0, col0 = 0, voff = 0, foff = 0, poff = 0;
    int32_t xs = 0, ys = 0, ent0 = 0;
    for (const Plan &p : parts) {
        for (hm_vpanel v : p.vpanels) { v.row0 += col0; v.off += voff; v.slot += ys; P.vpanels.push_back(v); }
        P.vpanel_fill.insert(P.vpanel_fill.end(), p.vpanel_fill.begin(), p.vpanel_fill.end());
        for (hm_m2l_row rw : p.m2l_rows) { rw.slot += xs; rw.begin += ent0; rw.end += ent0; P.m2l_rows.push_back(rw); }
        for (hm_m2l_ent e : p.m2l_ents) { e.foff += foff; e.yslot += ys; P.m2l_ents.push_back(e); }
        P.f_fill.insert(P.f_fill.end(), p.f_fill.begin(), p.f_fill.end());
        const int32_t piece0 = (int32_t)P.pieces.size();
        for (hm_piece q : p.pieces) {
            if (q.kind == HM_PIECE_COEF) q.src += xs; else q.src += col0;
            P.pieces.push_back(q);
        }
        for (hm_seg g : p.segs) { g.row0 += row0; g.poff += poff; g.piece0 += piece0; P.segs.push_back(g); }
        P.seg_fill.insert(P.seg_fill.end(), p.seg_fill.begin(), p.seg_fill.end());
        for (hm_xfer e : p.up) { e.slot += ys; e.c0 += ys; e.c1 += ys; P.up.push_back(e); }
        for (hm_xfer e : p.down) { e.slot += xs; e.c0 += xs; e.c1 += xs; P.down.push_back(e); }
        P.max_width = std::max(P.max_width, p.max_width);
        PlanStats &S = P.stats;
        const PlanStats &Q = p.stats;
        S.n_bary += Q.n_bary; S.n_dense += Q.n_dense; S.depth = std::max(S.depth, Q.depth);
        S.canonical_values += Q.canonical_values; S.reference_values += Q.reference_values;
        S.stored_values += Q.stored_values; S.dense_values += Q.dense_values; S.n_segments += Q.n_segments;
        S.max_width = std::max(S.max_width, Q.max_width);
        row0 += p.nx; col0 += p.ny; voff += p.vstore_elems; foff += p.fstore_elems; poff += p.pstore_elems;
        xs += p.n_xslots; ys += p.n_yslots; ent0 += (int32_t)p.m2l_ents.size();
    }
    P.nx = row0; P.ny = col0;
    P.vstore_elems = voff; P.fstore_elems = foff; P.pstore_elems = poff;
    P.n_xslots = xs; P.n_yslots = ys;
    P.stats.n_xslots = xs; P.stats.n_yslots = ys;
    merge_bands(parts, true, P);
    merge_bands(parts, false, P);
    // level tables are per instance only; the merged plan keeps them empty
    P.up_level_ptr.assign(1, 0);
    P.down_level_ptr.assign(1, 0);
}

int build_hier_plan(int64_t m, int64_t n, const std::vector<HierBlock> &blocks, Plan &P,
                    std::vector<double> &vstore, std::vector<double> &fstore, std::vector<double> &pstore)
{
    P = Plan();
    P.nx = m; P.ny = n;
    int R = 1;
    bool has_core = false;
    for (const HierBlock &b : blocks) {
        if (b.kind != 0) R = std::max<int64_t>(R, b.rank);
        if (b.kind == 2) has_core = true;
    }
    if (has_core && R > 32) return PLAN_ERR_DEGENERATE;
    P.r = R;
    P.fstride = (int)round_up((int64_t)R * R, 4);
    std::vector<int> slot(blocks.size(), -1);
    int ns = 0;
    vstore.clear(); fstore.clear(); pstore.clear();
    for (size_t i = 0; i < blocks.size(); ++i) {
        const HierBlock &b = blocks[i];
        if (b.kind == 0 || b.rank <= 0 || b.rows <= 0 || b.cols <= 0) continue;
        slot[i] = ns++;
        // basis panel(s): V (diag(sigma) folded in for low-rank blocks), row-major, <= 32 columns each
        const double *V = b.kind == 1 ? b.data + b.rows * b.rank + b.rank : b.data + b.rows * b.rank + b.rank * b.rank;
        const double *sig = b.kind == 1 ? b.data + b.rows * b.rank : nullptr;
        for (int64_t c0 = 0; c0 < b.rank; c0 += 32) {
            const int w = (int)std::min<int64_t>(32, b.rank - c0);
            hm_vpanel vp;
            vp.row0 = b.col0; vp.nrows = (int32_t)b.cols; vp.ld = w; vp.width = w; vp.slot = slot[i];
            vp.col0 = (int32_t)c0; vp.pad = 0;
            vp.off = (int64_t)vstore.size();
            for (int64_t j = 0; j < b.cols; ++j)
                for (int c = 0; c < w; ++c) {
                    double v = V[j + b.cols * (c0 + c)];
                    if (sig) v *= sig[c0 + c];
                    vstore.push_back(v);
                }
            vstore.resize(round_up((int64_t)vstore.size(), 32), 0.0);
            P.vpanels.push_back(vp);
        }
        if (b.kind == 2) {
            hm_m2l_ent e;
            e.foff = (int64_t)fstore.size(); e.yslot = slot[i]; e.pad = 0;
            fstore.resize(fstore.size() + P.fstride, 0.0);
            const double *C = b.data + b.rows * b.rank;
            for (int64_t q = 0; q < b.rank; ++q)
                for (int64_t p = 0; p < b.rank; ++p) fstore[e.foff + p + R * q] = C[p + b.rank * q];
            P.m2l_rows.push_back({slot[i], (int32_t)P.m2l_ents.size(), (int32_t)P.m2l_ents.size() + 1, 0});
            P.m2l_ents.push_back(e);
            P.stats.n_bary += 1;
        }
    }
    P.n_xslots = P.n_yslots = ns;
    P.vstore_elems = (int64_t)vstore.size();
    P.fstore_elems = (int64_t)fstore.size();
    // elementary row intervals
    std::vector<int64_t> cuts = {0, m};
    for (const HierBlock &b : blocks)
        if (b.rows > 0 && b.cols > 0 && (b.kind == 0 || b.rank > 0)) {
            cuts.push_back(std::min(std::max<int64_t>(b.row0, 0), m));
            cuts.push_back(std::min(std::max<int64_t>(b.row0 + b.rows, 0), m));
        }
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    const size_t nint = cuts.size() - 1;
    std::vector<std::vector<int>> cover(nint);
    for (size_t i = 0; i < blocks.size(); ++i) {
        const HierBlock &b = blocks[i];
        if (b.rows <= 0 || b.cols <= 0 || (b.kind != 0 && b.rank <= 0)) continue;
        const size_t i0 = std::lower_bound(cuts.begin(), cuts.end(), b.row0) - cuts.begin();
        const size_t i1 = std::lower_bound(cuts.begin(), cuts.end(), b.row0 + b.rows) - cuts.begin();
        for (size_t iv = i0; iv < i1; ++iv) cover[iv].push_back((int)i);
    }
    const int seg_rows = 64;
    for (size_t iv = 0; iv < nint; ++iv) {
        const int64_t p0 = cuts[iv], q0 = cuts[iv + 1];
        if (q0 <= p0) continue;
        // far-field pieces first, then dense pieces (each part is a contiguous column run)
        std::vector<int> order;
        for (int i : cover[iv]) if (blocks[i].kind != 0) order.push_back(i);
        for (int i : cover[iv]) if (blocks[i].kind == 0) order.push_back(i);
        for (int64_t r0 = p0; r0 < q0; r0 += seg_rows) {
            hm_seg g;
            g.row0 = r0;
            g.nrows = (int32_t)std::min<int64_t>(seg_rows, q0 - r0);
            g.ld = (int32_t)round_up(g.nrows, 4);
            g.piece0 = (int32_t)P.pieces.size();
            g.width = 0;
            g.nfar = 0;
            for (int i : order) {
                const HierBlock &b = blocks[i];
                hm_piece pc;
                if (b.kind == 0) { pc.kind = HM_PIECE_X; pc.src = b.col0; pc.width = (int32_t)b.cols; }
                else { pc.kind = b.kind == 1 ? HM_PIECE_TCOEF : HM_PIECE_COEF; pc.src = slot[i]; pc.width = (int32_t)b.rank; }
                P.pieces.push_back(pc);
                g.width += pc.width;
                if (b.kind != 0) g.nfar += pc.width;
            }
            g.npieces = (int32_t)P.pieces.size() - g.piece0;
            g.poff = (int64_t)pstore.size();
            pstore.resize(pstore.size() + round_up((int64_t)g.ld * std::max(g.width, 1), 32), 0.0);
            int col = 0;
            for (int i : order) {
                const HierBlock &b = blocks[i];
                const int64_t w = b.kind == 0 ? b.cols : b.rank;
                const int64_t ldb = b.rows;          // A (rows x cols) or U (rows x r), column-major
                for (int64_t c = 0; c < w; ++c)
                    for (int rr = 0; rr < g.nrows; ++rr)
                        pstore[g.poff + rr + (int64_t)g.ld * (col + c)] = b.data[(r0 + rr - b.row0) + ldb * c];
                col += (int)w;
            }
            P.max_width = std::max(P.max_width, g.width);
            P.segs.push_back(g);
            P.seg_fill.push_back({0.0, 0.0, 0, 0});
        }
    }
    P.pstore_elems = (int64_t)pstore.size();
    P.up_band_ptr.assign(1, 0);
    P.down_band_ptr.assign(1, 0);
    P.up_level_ptr.assign(1, 0);
    P.down_level_ptr.assign(1, 0);
    PlanStats &S = P.stats;
    S.n_xslots = S.n_yslots = ns;
    for (const HierBlock &b : blocks) {
        if (b.kind == 0) { S.n_dense += 1; S.dense_values += b.rows * b.cols; }
        S.reference_values += b.kind == 0 ? b.rows * b.cols : (b.rows + b.cols) * b.rank + (b.kind == 1 ? b.rank : b.rank * b.rank);
    }
    S.canonical_values = S.reference_values;
    S.stored_values = P.vstore_elems + P.fstore_elems + P.pstore_elems;
    S.n_segments = (int64_t)P.segs.size();
    S.max_width = P.max_width;
    return PLAN_OK;
}

}  // namespace hm
