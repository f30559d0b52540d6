// CUDA kernels: batched compression (fill) and the hierarchical matvec.
#include "hm_kernels.cuh"
#include "hm_async.cuh"

#include <type_traits>

namespace hm {

// ============================================================== fill kernels

// Explicit column bases: V[j, m] = (lam_m / (y_j - yh_m)) / sum_m' (...),
// the second barycentric form of src/BarycentricMatrix.jl:276-287, computed in
// FP64 and stored row-major (r values per point).  One CTA per panel.
template <typename S>
__global__ void fill_vpanels(FillArgs fa, const hm_vpanel *vp, const hm_fill_vpanel *vf,
                             int npanels, S *V)
{
    __shared__ double nodes[HM_RMAX], lam[HM_RMAX];
    const int p = blockIdx.x;
    if (p >= npanels) return;
    const hm_vpanel P = vp[p];
    const int r = fa.r;
    if (threadIdx.x < r) {
        nodes[threadIdx.x] = box_node(vf[p].a, vf[p].b, fa.cheb[threadIdx.x]);
        lam[threadIdx.x] = fa.lam[threadIdx.x];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < P.nrows; j += blockDim.x) {
        const double yj = fa.y[P.row0 + j];
        double w[HM_RMAX];
        double sum = 0.0;
#pragma unroll
        for (int m = 0; m < HM_RMAX; ++m) {
            if (m < r) {
                w[m] = __dmul_rn(lam[m], 1.0 / __dsub_rn(yj, nodes[m]));
                sum = __dadd_rn(sum, w[m]);
            }
        }
        S *row = V + P.off + (int64_t)j * P.ld;
#pragma unroll
        for (int m = 0; m < HM_RMAX; ++m)
            if (m < r) row[m] = (S)(w[m] / sum);
    }
}

// F[m + r n] = f(xh_m, yh_n)  (src/BarycentricMatrix.jl:147-178).  One CTA per block.
template <typename S>
__global__ void fill_f(FillArgs fa, const hm_fill_f *ff, const hm_m2l_ent *ents, int nblocks, S *F)
{
    __shared__ double xh[HM_RMAX], yh[HM_RMAX];
    const int e = blockIdx.x;
    if (e >= nblocks) return;
    const int r = fa.r;
    if (threadIdx.x < r) {
        xh[threadIdx.x] = box_node(ff[e].xa, ff[e].xb, fa.cheb[threadIdx.x]);
        yh[threadIdx.x] = box_node(ff[e].ya, ff[e].yb, fa.cheb[threadIdx.x]);
    }
    __syncthreads();
    S *Fe = F + ents[e].foff;
    for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
        const int m = idx % r, n = idx / r;
        Fe[idx] = (S)fill_kernel(fa, xh[m], yh[n]);
    }
}

// Segment panels: the first basis_w columns hold the row basis U[i, m] of the
// segment's deepest row box (src/BarycentricMatrix.jl:256-267), the rest the
// near-field dense blocks f(x_i, y_j) (src/KernelMatrix.jl:57-60).  Column-major
// with leading dimension ld.  One CTA per segment.  DROW = true fills the
// derivative of every entry with respect to its row point instead: the basis
// derivative U_m'(x) = U_m(x) (sum_k U_k(x)/(x - xh_k) - 1/(x - xh_m)) and
// d f / d(row point) for the dense blocks.
template <typename S, bool DROW>
__global__ void fill_segments(FillArgs fa, const hm_seg *segs, const hm_piece *pieces,
                              const hm_fill_seg *sf, int nsegs, S *P)
{
    __shared__ double nodes[HM_RMAX], lam[HM_RMAX];
    const int sidx = blockIdx.x;
    if (sidx >= nsegs) return;
    const hm_seg G = segs[sidx];
    const hm_fill_seg Fi = sf[sidx];
    const int r = fa.r;
    S *Pg = P + G.poff;
    int col = 0;
    if (Fi.has_basis) {
        if (threadIdx.x < r) {
            nodes[threadIdx.x] = box_node(Fi.a, Fi.b, fa.cheb[threadIdx.x]);
            lam[threadIdx.x] = fa.lam[threadIdx.x];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < G.nrows; i += blockDim.x) {
            const double xi = fa.x[G.row0 + i];
            double w[HM_RMAX];
            double sum = 0.0;
#pragma unroll
            for (int m = 0; m < HM_RMAX; ++m) {
                if (m < r) {
                    w[m] = __dmul_rn(lam[m], 1.0 / __dsub_rn(xi, nodes[m]));
                    sum = __dadd_rn(sum, w[m]);
                }
            }
            if (DROW) {
                double sd = 0.0;
#pragma unroll
                for (int m = 0; m < HM_RMAX; ++m)
                    if (m < r) sd += (w[m] / sum) / __dsub_rn(xi, nodes[m]);
#pragma unroll
                for (int m = 0; m < HM_RMAX; ++m)
                    if (m < r) Pg[i + (int64_t)G.ld * m] = (S)((w[m] / sum) * (sd - 1.0 / __dsub_rn(xi, nodes[m])));
            } else {
#pragma unroll
                for (int m = 0; m < HM_RMAX; ++m)
                    if (m < r) Pg[i + (int64_t)G.ld * m] = (S)(w[m] / sum);
            }
        }
        col = Fi.basis_w;
    }
    for (int pc = (Fi.has_basis ? 1 : 0); pc < G.npieces; ++pc) {
        const hm_piece Q = pieces[G.piece0 + pc];
        const int64_t tot = (int64_t)Q.width * G.nrows;
        for (int64_t idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int i = (int)(idx % G.nrows), j = (int)(idx / G.nrows);
            Pg[i + (int64_t)G.ld * (col + j)] =
                (S)(DROW ? fill_kernel_drow(fa, fa.x[G.row0 + i], fa.y[Q.src + j])
                         : fill_kernel(fa, fa.x[G.row0 + i], fa.y[Q.src + j]));
        }
        col += Q.width;
    }
}

template __global__ void fill_vpanels<double>(FillArgs, const hm_vpanel *, const hm_fill_vpanel *, int, double *);
template __global__ void fill_vpanels<float>(FillArgs, const hm_vpanel *, const hm_fill_vpanel *, int, float *);
template __global__ void fill_f<double>(FillArgs, const hm_fill_f *, const hm_m2l_ent *, int, double *);
template __global__ void fill_f<float>(FillArgs, const hm_fill_f *, const hm_m2l_ent *, int, float *);
template __global__ void fill_segments<double, false>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, double *);
template __global__ void fill_segments<float, false>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, float *);
template __global__ void fill_segments<double, true>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, double *);
template __global__ void fill_segments<float, true>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, float *);

// ============================================================== matvec kernels
//
// Coefficients of slot `sl` for right-hand side q live at coef[(sl*k + q)*r + m].
// A product runs the tree passes (leaf_up, xfer_up per level, m2l, xfer_down
// per level) on a side stream while expand_part<.., false> streams the
// near-field dense panels on the caller's stream; after the join
// expand_part<.., true> adds the far field U s.


// N consecutive values from 16-byte aligned shared memory, as 16-byte loads
// where N values fill them (the chunks of right-hand sides below are stored
// right-hand side fastest, so that one step's N values are adjacent).
template <int N, typename A>
__device__ __forceinline__ void ld_vec(const A *p, A *v)
{
    if constexpr (sizeof(A) == 4 && N % 4 == 0) {
#pragma unroll
        for (int i = 0; i < N / 4; ++i) {
            const float4 w = reinterpret_cast<const float4 *>(p)[i];
            v[4 * i] = w.x; v[4 * i + 1] = w.y; v[4 * i + 2] = w.z; v[4 * i + 3] = w.w;
        }
    } else if constexpr (sizeof(A) == 8 && N % 2 == 0) {
#pragma unroll
        for (int i = 0; i < N / 2; ++i) {
            const double2 w = reinterpret_cast<const double2 *>(p)[i];
            v[2 * i] = w.x; v[2 * i + 1] = w.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = p[i];
    }
}

// t[slot][col0 + m] = (V^T x)[m] for each explicit basis panel.  One warp
// per panel, looping over chunks of QC right-hand sides; lane m owns column m
// of the row-major panel (width <= 32, row stride ld).  Panels of up to cap
// rows and wcap columns (the handle's largest, up to 128 rows) are staged
// once in shared memory (cp.async) and the chunks' x values double-buffered
// beside them; longer panels are read directly.  Plain FMA accumulation
// (the coefficients feed only the far field).  Coefficients of a slot are r
// apart per right-hand side.
template <typename S, typename A, int QC>
__global__ void leaf_up(MulArgs<S> ma, const hm_vpanel *vp, int npanels, const S *V, A *t, int r, int cap, int wcap)
{
    extern __shared__ unsigned char smem_raw[];
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= (int64_t)npanels) return;
    const hm_vpanel P = vp[w];
    const int pw = P.width;
    const S *Vp = V + P.off;
    const int k = ma.k;
    // right-hand sides read from xin (and copied into x as they pass) or from x
    const S *xsrc = ma.xin ? ma.xin : ma.x;
    S *xcopy = ma.xin ? const_cast<S *>(ma.x) : nullptr;
    auto store = [&](int q0, int qc, PlainAcc<A> *acc) {
        if (lane < pw) {
#pragma unroll
            for (int qq = 0; qq < QC; ++qq)
                if (qq < qc) t[((int64_t)P.slot * k + q0 + qq) * r + P.col0 + lane] = acc[qq].value();
        }
    };
    if (P.nrows <= cap && P.ld == pw && pw <= wcap) {
        // the panel once; x chunks of QC right-hand sides double-buffered,
        // row major xs[b][j * QC + qq] (lanes walk rows)
        S *Vs = reinterpret_cast<S *>(smem_raw + (size_t)wib * leaf_up_warp_bytes<S, A, QC>(cap, wcap));
        A *xs = reinterpret_cast<A *>(Vs + cap * wcap);
        const int nel = P.nrows * pw;
        if (sizeof(S) * nel % 16 == 0 && (P.off * sizeof(S)) % 16 == 0) {
            const char *src = reinterpret_cast<const char *>(Vp);
            char *dst = reinterpret_cast<char *>(Vs);
            for (int i = lane; i < (int)(nel * sizeof(S) / 16); i += 32) async_copy16(dst + 16 * i, src + 16 * i);
        } else {
            for (int i = lane; i < nel; i += 32) async_copy<sizeof(S)>(Vs + i, Vp + i);
        }
        auto fetch = [&](int q0, int b) {
            const int qc = min(QC, k - q0);
            A *d = xs + b * cap * QC;
#pragma unroll
            for (int qq = 0; qq < QC; ++qq)
                for (int j = lane; j < P.nrows; j += 32) {
                    const int64_t e = (P.row0 + j) * ma.incx + (int64_t)(q0 + qq) * ma.ldx;
                    if (qq >= qc) {
                        d[j * QC + qq] = A(0);
                    } else if (xcopy) {
                        // host-mapped source: plain loads, stored here and into x
                        const S v = xsrc[e];
                        d[j * QC + qq] = (A)v;
                        xcopy[e] = v;
                    } else {
                        async_copy<sizeof(A)>(d + j * QC + qq, ma.x + e);
                    }
                }
            async_commit();
        };
        fetch(0, 0);
        for (int q0 = 0, b = 0; q0 < k; q0 += QC, b ^= 1) {
            if (q0 + QC < k) {
                fetch(q0 + QC, b ^ 1);
                asm volatile("cp.async.wait_group 1;" ::: "memory");
            } else {
                async_wait_all();
            }
            __syncwarp();
            PlainAcc<A> acc[QC];
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) acc[qq].zero();
            const A *xb = xs + b * cap * QC;
            if (lane < pw) {
                for (int j = 0; j < P.nrows; ++j) {
                    const A v = (A)Vs[j * pw + lane];
                    A xv[QC];
                    ld_vec<QC>(xb + j * QC, xv);
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq) acc[qq].add(v, xv[qq]);
                }
            }
            store(q0, min(QC, k - q0), acc);
            __syncwarp();                                 // buffer b is refilled next
        }
    } else {
        for (int q0 = 0; q0 < k; q0 += QC) {
            const int qc = min(QC, k - q0);
            PlainAcc<A> acc[QC];
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) acc[qq].zero();
            if (lane < pw) {
                const S *col = Vp + lane;
                for (int j = 0; j < P.nrows; ++j) {
                    const A v = (A)col[(int64_t)j * P.ld];
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq)
                        if (qq < qc) acc[qq].add(v, (A)xsrc[(P.row0 + j) * ma.incx + (int64_t)(q0 + qq) * ma.ldx]);
                }
            }
            if (xcopy)
                for (int qq = 0; qq < qc; ++qq)
                    for (int j = lane; j < P.nrows; j += 32) {
                        const int64_t e = (P.row0 + j) * ma.incx + (int64_t)(q0 + qq) * ma.ldx;
                        xcopy[e] = xsrc[e];
                    }
            store(q0, qc, acc);
        }
    }
}

// Upward transfers of one band: t[parent][m] = sum_c sum_m' T_c[m', m] t[child_c][m'].
// One CTA per task (a subtree cut to the band's levels); the task's steps
// (levels, deepest first) run in order with a CTA barrier between them, warps
// taking (record, chunk of QC right-hand sides) pairs.  T (T_0 then T_1, each
// r x r with T_c[m' * r + m]) and the children's coefficients are staged in
// shared memory.
template <typename A, int QC>
__global__ void xfer_up_band(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *t,
                             int r, int k)
{
    extern __shared__ unsigned char smem_raw[];
    A *Ts = reinterpret_cast<A *>(smem_raw);
    A *cs = Ts + 2 * HM_RMAX * HM_RMAX + (threadIdx.x >> 5) * 2 * QC * HM_RMAX;   // [c][qq][m']
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) Ts[i] = T[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int nq = (k + QC - 1) / QC;
    const hm_task tk = tasks[blockIdx.x];
    for (int st = tk.step0; st < tk.step1; ++st) {
        const hm_step S = steps[st];
        for (int64_t w = threadIdx.x >> 5; w < (int64_t)(S.e1 - S.e0) * nq; w += nw) {
            const hm_xfer X = ents[S.e0 + w / nq];
            const int q0 = (int)(w % nq) * QC, qc = min(QC, k - q0);
            for (int i = lane; i < QC * r; i += 32) {
                const int qq = i / r, m = i % r;
                cs[qq * HM_RMAX + m] = qq < qc ? t[((int64_t)X.c0 * k + q0 + qq) * r + m] : (A)0;
                cs[(QC + qq) * HM_RMAX + m] = qq < qc ? t[((int64_t)X.c1 * k + q0 + qq) * r + m] : (A)0;
            }
            __syncwarp();
            if (lane < r) {
                A acc[QC];
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) acc[qq] = 0;
                for (int mp = 0; mp < r; ++mp) {
                    const A a0 = Ts[mp * r + lane], a1 = Ts[r * r + mp * r + lane];
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq)
                        acc[qq] += a0 * cs[qq * HM_RMAX + mp] + a1 * cs[(QC + qq) * HM_RMAX + mp];
                }
#pragma unroll
                for (int qq = 0; qq < QC; ++qq)
                    if (qq < qc) t[((int64_t)X.slot * k + q0 + qq) * r + lane] = acc[qq];
            }
            __syncwarp();
        }
        __syncthreads();
    }
}

// Band tasks with shared-memory-resident coefficients, one CTA per (task,
// chunk of QC right-hand sides: blockIdx.y): the task's
// external inputs (and T) are fetched once with cp.async, every level then
// reads and writes shared memory only, with a CTA barrier between levels;
// each coefficient the task produces is also written to global memory.
// Task-local numbering (records' pad, set by the planner): upward, record i
// produces local i and reads locals pad & 0xffff, pad >> 16; downward,
// record i's children are locals 2i, 2i + 1 and its parent is local pad.
// Upward, L holds r x QC values per local, right-hand side fastest
// (L[local][m][qq]); downward QC x r (L[local][qq][m]).
template <typename A, int QC>
__global__ void xfer_up_task(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *t,
                             int r, int k, int early)
{
    extern __shared__ unsigned char smem_raw[];
    A *Ts = reinterpret_cast<A *>(smem_raw);
    A *L = Ts + 2 * HM_RMAX * HM_RMAX;
    const hm_task tk = tasks[blockIdx.x];
    const int e0 = steps[tk.step0].e0, e1 = steps[tk.step1 - 1].e1, nrec = e1 - e0;
    const int q0 = blockIdx.y * QC, qc = min(QC, k - q0);      // this CTA's right-hand sides
    if (early) pdl_trigger();     // the next band may be scheduled now (a small grid; not before a large one)
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) async_copy<sizeof(A)>(Ts + i, T + i);
    pdl_wait();                                                // the children's coefficients are ready
    // external children: warps take records, lanes coefficients
    for (int rec = threadIdx.x >> 5; rec < nrec; rec += blockDim.x >> 5) {
        const hm_xfer X = ents[e0 + rec];
        const int ln = threadIdx.x & 31;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int lc = c ? (X.pad >> 16) : (X.pad & 0xffff);
            if (lc < nrec || ln >= r) continue;           // produced by an earlier level of this task
            const A *src = t + ((int64_t)(c ? X.c1 : X.c0) * k + q0) * r + ln;
            A *d = L + (int64_t)lc * QC * r + ln * QC;
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) {
                if (qq < qc) async_copy<sizeof(A)>(d + qq, src + (int64_t)qq * r);
                else d[qq] = A(0);
            }
        }
    }
    async_wait_all();
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int st = tk.step0; st < tk.step1; ++st) {
        const hm_step S = steps[st];
        for (int w = threadIdx.x >> 5; w < S.e1 - S.e0; w += nw) {
            const int e = S.e0 + w;
            const hm_xfer X = ents[e];
            const A *c0 = L + (int64_t)(X.pad & 0xffff) * QC * r;
            const A *c1 = L + (int64_t)(X.pad >> 16) * QC * r;
            A *out = L + (int64_t)(e - e0) * QC * r;
            if (lane < r) {
                A acc[QC];
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) acc[qq] = 0;
                for (int mp = 0; mp < r; ++mp) {
                    const A a0 = Ts[mp * r + lane], a1 = Ts[r * r + mp * r + lane];
                    A v0[QC], v1[QC];
                    ld_vec<QC>(c0 + mp * QC, v0);
                    ld_vec<QC>(c1 + mp * QC, v1);
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq) acc[qq] += a0 * v0[qq] + a1 * v1[qq];
                }
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) {
                    out[lane * QC + qq] = acc[qq];
                    if (qq < qc) t[((int64_t)X.slot * k + q0 + qq) * r + lane] = acc[qq];
                }
            }
        }
        __syncthreads();
    }
}

template <typename A, int QC>
__global__ void xfer_down_task(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *s,
                               int r, int k, int early)
{
    extern __shared__ unsigned char smem_raw[];
    A *Ts = reinterpret_cast<A *>(smem_raw);
    A *L = Ts + 2 * HM_RMAX * HM_RMAX;
    const hm_task tk = tasks[blockIdx.x];
    const int e0 = steps[tk.step0].e0, e1 = steps[tk.step1 - 1].e1, nrec = e1 - e0;
    const int q0 = blockIdx.y * QC, qc = min(QC, k - q0);      // this CTA's right-hand sides
    if (early) pdl_trigger();
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) async_copy<sizeof(A)>(Ts + i, T + i);
    pdl_wait();                                                // far-field and parent coefficients are ready
    // children start from their far-field (m2l) coefficients; external parents as computed
    // warps take records, lanes coefficients
    for (int rec = threadIdx.x >> 5; rec < nrec; rec += blockDim.x >> 5) {
        const hm_xfer X = ents[e0 + rec];
        const int ln = threadIdx.x & 31;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            int lc, slot;
            if (c < 2) {
                lc = 2 * rec + c;
                slot = c ? X.c1 : X.c0;
            } else {
                lc = X.pad;
                slot = X.slot;
                if (lc < 2 * nrec) continue;              // a child of an earlier level of this task
            }
            if (ln >= r) continue;
            const A *src = s + ((int64_t)slot * k + q0) * r + ln;
            A *d = L + (int64_t)lc * QC * r + ln;
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) {
                if (qq < qc) async_copy<sizeof(A)>(d + qq * r, src + (int64_t)qq * r);
                else d[qq * r] = A(0);
            }
        }
    }
    async_wait_all();
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int st = tk.step0; st < tk.step1; ++st) {
        const hm_step S = steps[st];
        for (int w = threadIdx.x >> 5; w < S.e1 - S.e0; w += nw) {
            const int e = S.e0 + w;
            const hm_xfer X = ents[e];
            const A *p = L + (int64_t)X.pad * QC * r;
            A *o0 = L + (int64_t)(2 * (e - e0)) * QC * r;
            A *o1 = o0 + QC * r;
            if (lane < r) {
                A a0[QC], a1[QC];
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) { a0[qq] = 0; a1[qq] = 0; }
                for (int m = 0; m < r; ++m) {
                    const A t0 = Ts[lane * r + m], t1 = Ts[r * r + lane * r + m];
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq) {
                        const A v = p[qq * r + m];
                        a0[qq] += t0 * v;
                        a1[qq] += t1 * v;
                    }
                }
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) {
                    const A v0 = o0[qq * r + lane] + a0[qq], v1 = o1[qq * r + lane] + a1[qq];
                    o0[qq * r + lane] = v0;
                    o1[qq * r + lane] = v1;
                    if (qq < qc) {
                        s[((int64_t)X.c0 * k + q0 + qq) * r + lane] = v0;
                        s[((int64_t)X.c1 * k + q0 + qq) * r + lane] = v1;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// Far field: s[slot][m] = sum_e sum_n F_e[m + r n] t[yslot_e][n]
// (the F stage of src/algebra.jl:258-265, grouped by row cluster).  One warp
// per (row slot, chunk of up to QC right-hand sides).  The r x r blocks of the
// row and the column coefficients they multiply are double-buffered in
// shared memory with cp.async: block e + 1 is in flight while block e is
// used for every right-hand side of the chunk.  Lane m accumulates row m.
template <typename S, typename A, int QC>
__global__ void m2l(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const S *F, int fstride,
                    const A *t, A *s, int r, int k)
{
    extern __shared__ unsigned char smem_raw[];
    // per warp: two F blocks (fstride values of S) and two column-coefficient chunks (QC * HM_RMAX of A)
    const int wib = threadIdx.x >> 5;
    const size_t wbytes = 2 * (size_t)fstride * sizeof(S) + 2 * (size_t)QC * HM_RMAX * sizeof(A);
    S *Fb = reinterpret_cast<S *>(smem_raw + wib * wbytes);
    A *Tb = reinterpret_cast<A *>(Fb + 2 * fstride);
    const int lane = threadIdx.x & 31;
    const int nq = (k + QC - 1) / QC;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    pdl_trigger();
    pdl_wait();                                                // the upward pass's coefficients are ready
    if (w >= (int64_t)nrows * nq) return;
    const hm_m2l_row R = rows[w / nq];
    const int q0 = (int)(w % nq) * QC, qc = min(QC, k - q0);
    auto fetch = [&](int e, int buf) {
        const hm_m2l_ent E = ents[e];
        const char *src = reinterpret_cast<const char *>(F + E.foff);
        char *dst = reinterpret_cast<char *>(Fb + buf * fstride);
        for (int i = lane; i < (int)(fstride * sizeof(S) / 16); i += 32) async_copy16(dst + 16 * i, src + 16 * i);
        A *tb = Tb + buf * QC * HM_RMAX;
        if (lane < r) {
            const A *src = t + ((int64_t)E.yslot * k + q0) * r + lane;
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) {
                if (qq < qc) async_copy<sizeof(A)>(tb + qq * HM_RMAX + lane, src + (int64_t)qq * r);
                else tb[qq * HM_RMAX + lane] = A(0);
            }
        }
        async_commit();
    };
    A acc[QC];
#pragma unroll
    for (int qq = 0; qq < QC; ++qq) acc[qq] = 0;
    if (R.begin < R.end) fetch(R.begin, 0);
    for (int e = R.begin; e < R.end; ++e) {
        const int buf = (e - R.begin) & 1;
        if (e + 1 < R.end) {
            fetch(e + 1, buf ^ 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            async_wait_all();
        }
        __syncwarp();
        const S *fb = Fb + buf * fstride;
        const A *tb = Tb + buf * QC * HM_RMAX;
        if (lane < r) {
            for (int n = 0; n < r; ++n) {
                const A f = (A)fb[lane + r * n];
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) acc[qq] += f * tb[qq * HM_RMAX + n];
            }
        }
        __syncwarp();                         // buffer buf is refilled by the next fetch
    }
    if (lane < r) {
#pragma unroll
        for (int qq = 0; qq < QC; ++qq)
            if (qq < qc) s[((int64_t)R.slot * k + q0 + qq) * r + lane] = acc[qq];
    }
}

// Far field for many right-hand sides (k > QC): one CTA (4 warps) per row
// slot.  The row's r x r blocks are staged once in shared memory (up to
// kM2lBlocks at a time, cp.async); the warps then take chunks of QC
// right-hand sides in turn, double-buffering each block's column
// coefficients, lane m accumulating row m of the chunk.
constexpr int kM2lBlocks = 8;
template <typename S, typename A, int QC>
__global__ void m2l_k(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const S *F, int fstride,
                      const A *t, A *s, int r, int k)
{
    extern __shared__ unsigned char smem_raw[];
    S *Fb = reinterpret_cast<S *>(smem_raw);                                      // kM2lBlocks x fstride
    A *Tb = reinterpret_cast<A *>(Fb + kM2lBlocks * fstride) + (threadIdx.x >> 5) * 2 * QC * HM_RMAX;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    pdl_trigger();
    pdl_wait();
    if (blockIdx.x >= nrows) return;
    const hm_m2l_row R = rows[blockIdx.x];
    for (int e0 = R.begin; e0 < R.end || e0 == R.begin; e0 += kM2lBlocks) {
        const int nb = min(kM2lBlocks, R.end - e0);
        __syncthreads();                                                           // previous batch used
        for (int b = 0; b < nb; ++b) {
            const char *src = reinterpret_cast<const char *>(F + ents[e0 + b].foff);
            char *dst = reinterpret_cast<char *>(Fb + b * fstride);
            for (int i = threadIdx.x; i < (int)(fstride * sizeof(S) / 16); i += blockDim.x)
                async_copy16(dst + 16 * i, src + 16 * i);
        }
        async_commit();
        async_wait_all();
        __syncthreads();
        for (int q0 = warp * QC; q0 < k; q0 += nw * QC) {
            const int qc = min(QC, k - q0);
            auto fetch = [&](int b, int buf) {
                A *tb = Tb + buf * QC * HM_RMAX;
                if (lane < r) {
                    const A *src = t + ((int64_t)ents[e0 + b].yslot * k + q0) * r + lane;
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq) {
                        if (qq < qc) async_copy<sizeof(A)>(tb + qq * HM_RMAX + lane, src + (int64_t)qq * r);
                        else tb[qq * HM_RMAX + lane] = A(0);
                    }
                }
                async_commit();
            };
            A acc[QC];
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) acc[qq] = 0;
            if (nb > 0) fetch(0, 0);
            for (int b = 0; b < nb; ++b) {
                if (b + 1 < nb) {
                    fetch(b + 1, (b + 1) & 1);
                    asm volatile("cp.async.wait_group 1;" ::: "memory");
                } else {
                    async_wait_all();
                }
                __syncwarp();
                const S *fb = Fb + b * fstride;
                const A *tb = Tb + (b & 1) * QC * HM_RMAX;
                if (lane < r) {
                    for (int n = 0; n < r; ++n) {
                        const A f = (A)fb[lane + r * n];
#pragma unroll
                        for (int qq = 0; qq < QC; ++qq) acc[qq] += f * tb[qq * HM_RMAX + n];
                    }
                }
                __syncwarp();
            }
            if (lane < r) {
                A *sp = s + ((int64_t)R.slot * k + q0) * r + lane;
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) {
                    if (qq >= qc) break;
                    if (e0 == R.begin) sp[(int64_t)qq * r] = acc[qq];
                    else sp[(int64_t)qq * r] += acc[qq];
                }
            }
        }
        if (R.end <= R.begin) break;                                               // empty row: zeros written once
    }
}

// Downward transfers of one band: s[child_c][m'] += sum_m T_c[m', m] s[parent][m].
// Same task/step structure as xfer_up_band, topmost level first.
template <typename A, int QC>
__global__ void xfer_down_band(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *s,
                               int r, int k)
{
    extern __shared__ unsigned char smem_raw[];
    A *Ts = reinterpret_cast<A *>(smem_raw);
    A *ps = Ts + 2 * HM_RMAX * HM_RMAX + (threadIdx.x >> 5) * QC * HM_RMAX;   // [qq][m]
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) Ts[i] = T[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int nq = (k + QC - 1) / QC;
    const hm_task tk = tasks[blockIdx.x];
    for (int st = tk.step0; st < tk.step1; ++st) {
        const hm_step S = steps[st];
        for (int64_t w = threadIdx.x >> 5; w < (int64_t)(S.e1 - S.e0) * nq; w += nw) {
            const hm_xfer X = ents[S.e0 + w / nq];
            const int q0 = (int)(w % nq) * QC, qc = min(QC, k - q0);
            for (int i = lane; i < QC * r; i += 32) {
                const int qq = i / r, m = i % r;
                ps[qq * HM_RMAX + m] = qq < qc ? s[((int64_t)X.slot * k + q0 + qq) * r + m] : (A)0;
            }
            __syncwarp();
            if (lane < r) {
                A a0[QC], a1[QC];
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) { a0[qq] = 0; a1[qq] = 0; }
                for (int m = 0; m < r; ++m) {
                    const A t0 = Ts[lane * r + m], t1 = Ts[r * r + lane * r + m];
#pragma unroll
                    for (int qq = 0; qq < QC; ++qq) {
                        const A v = ps[qq * HM_RMAX + m];
                        a0[qq] += t0 * v;
                        a1[qq] += t1 * v;
                    }
                }
#pragma unroll
                for (int qq = 0; qq < QC; ++qq) {
                    if (qq < qc) {
                        s[((int64_t)X.c0 * k + q0 + qq) * r + lane] += a0[qq];
                        s[((int64_t)X.c1 * k + q0 + qq) * r + lane] += a1[qq];
                    }
                }
            }
            __syncwarp();
        }
        __syncthreads();
    }
}

// Row segments, up to KB right-hand sides: one warp per segment (<= 64 rows).
// FAR = false: the near-field dense columns, y (+)= D x (written with the
// caller's accumulate flag); FAR = true: the row-basis columns, y += U s.
// FP32: lanes 0-15 and 16-31 take alternate panel columns, each lane four
// consecutive rows through one 16-byte load per column; FP64: each lane two
// rows per 16-byte load.  The panel streams once from HBM whatever the
// number of right-hand sides; the gathered right-hand sides [s ; x pieces]
// are staged per warp in shared memory (g[c * KB + q]).  KB = 1 accumulates
// with compensated (TwoProd/TwoSum) sums, KB > 1 with FMA per piece folded
// in with TwoSum.
template <typename A, int KB>
struct SegAcc;
template <typename A>
struct SegAcc<A, 1> {
    Acc<A> a;
    __device__ __forceinline__ void zero() { a.zero(); }
    __device__ __forceinline__ void add(A p, const A *g) { a.add(p, g[0]); }
    __device__ __forceinline__ void fold() {}
    __device__ __forceinline__ A hi(int) const { return a.s_hi(); }
    __device__ __forceinline__ A lo(int) const { return a.s_lo(); }
    __device__ __forceinline__ A merged(int, A so, A co) const { return a.merged(so, co); }
};
template <typename A, int KB>
struct SegAcc {
    A part[KB], h[KB], l[KB];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int q = 0; q < KB; ++q) { part[q] = 0; h[q] = 0; l[q] = 0; }
    }
    __device__ __forceinline__ void add(A p, const A *g)
    {
#pragma unroll
        for (int q = 0; q < KB; ++q) part[q] = fma(p, g[q], part[q]);
    }
    __device__ __forceinline__ void fold()   // end of a piece: compensated fold of the partial sums
    {
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            const A t = h[q] + part[q];
            const A bp = t - h[q];
            l[q] += (h[q] - (t - bp)) + (part[q] - bp);
            h[q] = t;
            part[q] = 0;
        }
    }
    __device__ __forceinline__ A hi(int q) const { return h[q]; }
    __device__ __forceinline__ A lo(int q) const { return l[q]; }
    __device__ __forceinline__ A merged(int q, A so, A co) const
    {
        const A t = h[q] + so;
        const A bp = t - h[q];
        return t + (((h[q] - (t - bp)) + (so - bp)) + (l[q] + co));
    }
};

// Near field (FAR = false: y (+)= D x) or far field (FAR = true: U s) of one
// row segment per warp.  The far field goes to yfar (leading dimension ldf)
// when given, else it is added into y.
template <typename S, typename A, bool FAR, int KB>
__global__ void expand_part(MulArgs<S> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const S *P,
                            const A *s, const A *t, int r, int maxw, S *yfar, int64_t ldf)
{
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int seg = blockIdx.x * (blockDim.x >> 5) + wib;
    if constexpr (FAR) pdl_wait();                             // the downward pass's coefficients are ready
    if (seg >= nsegs) return;
    A *g = reinterpret_cast<A *>(smem_raw) + (int64_t)wib * maxw * KB;
    const hm_seg G = segs[seg];
    const int k = ma.k;
    // gather the right-hand sides of the columns this part uses; the part's
    // pieces are one contiguous column run [c0, c1) of the panel
    int c0 = -1, c1 = 0, col = 0;
    for (int pc = 0; pc < G.npieces; ++pc) {
        const hm_piece Q = pieces[G.piece0 + pc];
        const bool take = FAR ? (Q.kind != HM_PIECE_X) : (Q.kind == HM_PIECE_X);
        if (take) {
            if (c0 < 0) c0 = col;
            const A *coef = Q.kind == HM_PIECE_TCOEF ? t : s;
            // fire-and-forget copies into shared memory for every piece, one
            // wait after the loop (no load-to-store round trip per piece)
            const int n = Q.width * KB;
            for (int i = lane; i < n; i += 32) {
                const int c = i / KB, q = i % KB;
                A *d = g + (col + c) * KB + q;
                if (q >= k) {
                    *d = A(0);
                } else if constexpr (FAR) {
                    async_copy<sizeof(A)>(d, coef + ((int64_t)Q.src * k + q) * r + c);
                } else if constexpr (sizeof(S) == sizeof(A)) {
                    async_copy<sizeof(A)>(d, ma.x + (Q.src + c) * ma.incx + (int64_t)q * ma.ldx);
                } else {
                    *d = (A)ma.x[(Q.src + c) * ma.incx + (int64_t)q * ma.ldx];
                }
            }
            c1 = col + Q.width;
        }
        col += Q.width;
    }
    async_wait_all();
    if (c0 < 0) {
        if (FAR && !yfar) return;          // no far field on these rows
        c0 = c1 = 0;
    }
    __syncwarp();
    const S *Pg = P + G.poff;
    // FAR with yfar: write the far-field rows to yfar (added to y later);
    // FAR without: add into y; near field: y (+)= per the caller's flag
    const bool acc_y = FAR ? (yfar == nullptr) : (ma.accumulate != 0);
    constexpr int FOLD = 64;              // columns between compensated folds (KB > 1)
    if constexpr (sizeof(S) == 4 && KB >= 4) {
        // four or more right-hand sides: each value loaded feeds KB FMAs, so
        // two rows per lane (float2) and every column in turn, which halves
        // the accumulators of the four-row form (3 KB values per row) and lets
        // twice as many warps hide the loads' latency
        SegAcc<A, KB> a0, a1;
        a0.zero(); a1.zero();
        if (2 * lane < G.ld) {
            const float2 *base = reinterpret_cast<const float2 *>(Pg + 2 * lane);
            const int64_t ld2 = G.ld / 2;
            for (int cb = c0; cb < c1; cb += FOLD) {
                const int ce = min(c1, cb + FOLD);
                int c = cb;
                for (; c + 16 <= ce; c += 16) {      // 16 loads in flight per lane
                    float2 p[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) p[u] = __ldcs(base + ld2 * (c + u));
#pragma unroll
                    for (int u = 0; u < 16; ++u) { a0.add(p[u].x, g + (c + u) * KB); a1.add(p[u].y, g + (c + u) * KB); }
                }
                for (; c + 8 <= ce; c += 8) {
                    float2 p[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) p[u] = __ldcs(base + ld2 * (c + u));
#pragma unroll
                    for (int u = 0; u < 8; ++u) { a0.add(p[u].x, g + (c + u) * KB); a1.add(p[u].y, g + (c + u) * KB); }
                }
                for (; c + 4 <= ce; c += 4) {
                    float2 p[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) p[u] = __ldcs(base + ld2 * (c + u));
#pragma unroll
                    for (int u = 0; u < 4; ++u) { a0.add(p[u].x, g + (c + u) * KB); a1.add(p[u].y, g + (c + u) * KB); }
                }
                for (; c < ce; ++c) {
                    const float2 p0 = __ldcs(base + ld2 * c);
                    a0.add(p0.x, g + c * KB); a1.add(p0.y, g + c * KB);
                }
                a0.fold(); a1.fold();
            }
        }
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            if (q >= k) break;
            const A v2[2] = {a0.merged(q, 0, 0), a1.merged(q, 0, 0)};
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int row = 2 * lane + j;
                if (row < G.nrows) {
                    if (FAR && yfar) {
                        yfar[(G.row0 + row) + (int64_t)q * ldf] = (S)v2[j];
                    } else {
                        S *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)q * ma.ldy;
                        A v = v2[j];
                        if (acc_y) v += (A)(*yp);
                        *yp = (S)v;
                    }
                }
            }
        }
    } else if (sizeof(S) == 4) {
        const int rg = lane & 15, h = lane >> 4;
        SegAcc<A, KB> acc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j].zero();
        if (4 * rg < G.ld) {
            const float4 *base = reinterpret_cast<const float4 *>(Pg + 4 * rg);
            const int64_t ld4 = G.ld / 4;
            for (int cb = c0; cb < c1; cb += FOLD) {
                const int ce = min(c1, cb + FOLD);
                int c = cb + ((h - cb) & 1);             // this half's columns have parity h
                for (; c + 14 < ce; c += 16) {
                    float4 p[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) p[u] = __ldcs(base + ld4 * (c + 2 * u));
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const A *gu = g + (c + 2 * u) * KB;
                        acc[0].add(p[u].x, gu); acc[1].add(p[u].y, gu); acc[2].add(p[u].z, gu); acc[3].add(p[u].w, gu);
                    }
                }
                for (; c + 6 < ce; c += 8) {           // tails in batches: fewer dependent round trips
                    float4 p[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) p[u] = __ldcs(base + ld4 * (c + 2 * u));
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const A *gu = g + (c + 2 * u) * KB;
                        acc[0].add(p[u].x, gu); acc[1].add(p[u].y, gu); acc[2].add(p[u].z, gu); acc[3].add(p[u].w, gu);
                    }
                }
                for (; c + 2 < ce; c += 4) {
                    const float4 p0 = __ldcs(base + ld4 * c), p1 = __ldcs(base + ld4 * (c + 2));
                    const A *g0 = g + c * KB, *g1 = g + (c + 2) * KB;
                    acc[0].add(p0.x, g0); acc[1].add(p0.y, g0); acc[2].add(p0.z, g0); acc[3].add(p0.w, g0);
                    acc[0].add(p1.x, g1); acc[1].add(p1.y, g1); acc[2].add(p1.z, g1); acc[3].add(p1.w, g1);
                }
                for (; c < ce; c += 2) {
                    const float4 p0 = __ldcs(base + ld4 * c);
                    const A *g0 = g + c * KB;
                    acc[0].add(p0.x, g0); acc[1].add(p0.y, g0); acc[2].add(p0.z, g0); acc[3].add(p0.w, g0);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[j].fold();
            }
        }
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            if (q >= k) break;
            A val[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const A so = __shfl_xor_sync(0xffffffffu, acc[j].hi(q), 16);
                const A co = __shfl_xor_sync(0xffffffffu, acc[j].lo(q), 16);
                val[j] = acc[j].merged(q, so, co);
            }
            if (h == 0) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int row = 4 * rg + j;
                    if (row < G.nrows) {
                        if (FAR && yfar) {
                            yfar[(G.row0 + row) + (int64_t)q * ldf] = (S)val[j];
                        } else {
                            S *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)q * ma.ldy;
                            A v = val[j];
                            if (acc_y) v += (A)(*yp);
                            *yp = (S)v;
                        }
                    }
                }
            }
        }
    } else {
        SegAcc<A, KB> a0, a1;
        a0.zero(); a1.zero();
        if (2 * lane < G.ld) {
            const double2 *base = reinterpret_cast<const double2 *>(Pg + 2 * lane);
            const int64_t ld2 = G.ld / 2;
            for (int cb = c0; cb < c1; cb += FOLD) {
                const int ce = min(c1, cb + FOLD);
                int c = cb;
                for (; c + 8 <= ce; c += 8) {
                    double2 p[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) p[u] = __ldcs(base + ld2 * (c + u));
#pragma unroll
                    for (int u = 0; u < 8; ++u) { a0.add(p[u].x, g + (c + u) * KB); a1.add(p[u].y, g + (c + u) * KB); }
                }
                for (; c < ce; ++c) {
                    const double2 p0 = __ldcs(base + ld2 * c);
                    a0.add(p0.x, g + c * KB); a1.add(p0.y, g + c * KB);
                }
                a0.fold(); a1.fold();
            }
        }
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            if (q >= k) break;
            const A v2[2] = {a0.merged(q, 0, 0), a1.merged(q, 0, 0)};
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int row = 2 * lane + j;
                if (row < G.nrows) {
                    if (FAR && yfar) {
                        yfar[(G.row0 + row) + (int64_t)q * ldf] = (S)v2[j];
                    } else {
                        S *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)q * ma.ldy;
                        A v = v2[j];
                        if (acc_y) v += (A)(*yp);
                        *yp = (S)v;
                    }
                }
            }
        }
    }
}

// Far-field rows U s with one thread per row: four segments per CTA of 256
// threads, 64 threads per segment.  The segment's far-field coefficients (its
// non-X pieces, at most 64 columns, KB right-hand sides) are gathered once into
// shared memory; thread `row` then reads its row of the column-major basis
// columns (consecutive threads, consecutive rows: coalesced) and accumulates
// KB sums with FMA (at most 64 terms, as the warp kernels' folds do).  The
// rows go to yfar (leading dimension ldf) or, without it, are added into y.
template <typename S, typename A, int KB>
__global__ void __launch_bounds__(256)
    far_rows(MulArgs<S> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const S *P, const A *s,
             const A *t, int r, S *yfar, int64_t ldf)
{
    __shared__ A cs[4][64 * KB];                               // [segment][column][q]
    pdl_wait();                                                // the downward pass's coefficients are ready
    const int ls = threadIdx.x >> 6, row = threadIdx.x & 63;
    const int j = blockIdx.x * 4 + ls;
    const int k = ma.k;
    hm_seg G{};
    int nfar = 0;
    if (j < nsegs) {
        G = segs[j];
        nfar = G.nfar;
        // coefficients of the far columns: element e = (column c, q) with c = e / KB
        for (int e = row; e < nfar * KB; e += 64) {
            const int c = e / KB, q = e % KB;
            int pc = 0, pi = 0;
            hm_piece Q = pieces[G.piece0];
            while (c >= pc + Q.width) {
                pc += Q.width;
                Q = pieces[G.piece0 + ++pi];
            }
            A v = A(0);
            if (q < k) v = (Q.kind == HM_PIECE_TCOEF ? t : s)[((int64_t)Q.src * k + q) * r + (c - pc)];
            cs[ls][e] = v;
        }
    }
    __syncthreads();
    if (j >= nsegs || row >= G.nrows) return;
    if (nfar == 0 && !yfar) return;                            // y += 0
    A acc[KB];
#pragma unroll
    for (int q = 0; q < KB; ++q) acc[q] = A(0);
    const S *pr = P + G.poff + row;
    // eight columns' loads issued before their FMAs (eight loads in flight per
    // thread), the sums in column order as one column at a time
    constexpr int CU = 8;
    int c = 0;
    for (; c + CU <= nfar; c += CU) {
        A u[CU];
#pragma unroll
        for (int i = 0; i < CU; ++i) u[i] = (A)__ldcs(pr + (int64_t)(c + i) * G.ld);
#pragma unroll
        for (int i = 0; i < CU; ++i)
#pragma unroll
            for (int q = 0; q < KB; ++q) acc[q] = fma(u[i], cs[ls][(c + i) * KB + q], acc[q]);
    }
    for (; c < nfar; ++c) {
        const A u = (A)__ldcs(pr + (int64_t)c * G.ld);
#pragma unroll
        for (int q = 0; q < KB; ++q) acc[q] = fma(u, cs[ls][c * KB + q], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < KB; ++q) {
        if (q >= k) break;
        if (yfar) {
            yfar[(G.row0 + row) + (int64_t)q * ldf] = (S)acc[q];
        } else {
            S *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)q * ma.ldy;
            *yp = (S)((A)(*yp) + acc[q]);
        }
    }
}

// y[i*incy + q*ldy] += yfar[i + q*ldf]: adds the far-field rows computed on the
// side stream (after the join).
template <typename S>
__global__ void add_far(MulArgs<S> ma, int64_t n, const S *yfar, int64_t ldf)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * ma.k) return;
    const int64_t row = i % n, q = i / n;
    S *yp = ma.y + row * ma.incy + q * ma.ldy;
    S *dst = ma.yout ? ma.yout + row + q * n : yp;
    *dst = *yp + yfar[row + q * ldf];
}

// ------------------------------------------------------- streamed panels
//
// One persistent CTA of 256 threads per slot (two per SM).  CTA b owns the
// segments [cta_seg[b], cta_seg[b+1]), balanced by panel bytes on the host.
// Thread 0 streams the part's columns of those panels chunk by chunk (ld rows
// x cc columns, one contiguous run of the column-major panel) into a ring of
// nst shared-memory stages with cp.async.bulk; each stage's mbarrier
// completes when its bytes have landed.  All threads consume: thread
// (row = tid % 64, group = tid / 64) multiplies its row by a quarter of the
// chunk's columns with plain FMA and folds the chunk's partial into a
// compensated (TwoSum) pair.  The gathered right-hand sides of the next
// segment are fetched with cp.async while the current one streams.  Every
// wait is bounded: after wait_ns (the handle's HM_OPT_WAIT_LIMIT_NS) the CTA
// records HM_DEV_WAIT_TIMEOUT in *status, waits (bounded by kDrainLimitNs) for
// its copies in flight and returns.  stall != 0 (a test hook) makes the first
// wait of every CTA run out.


template <typename S, typename A, bool FAR, int KB>
__global__ void __launch_bounds__(kStreamThreads, KB >= 4 ? (sizeof(S) == 4 ? 2 : 1) : 3)   // registers of 4+ right-hand sides
    stream_part(MulArgs<S> ma, const hm_seg *segs, const int *cta_seg, const hm_piece *pieces, const S *P,
                const A *s, const A *t, int r, int nst, int gcap, int ngb, int dsegs, S *yfar, int *status,
                unsigned long long wait_ns, int stall)
{
    static_assert(sizeof(S) == sizeof(A), "right-hand sides are copied into shared memory as they are");
    // rows per thread: one 16-byte load; FP32 with 4+ right-hand sides takes 2
    // (8-byte loads) to keep its accumulators in registers
    constexpr bool kNarrow = sizeof(S) == 4 && KB >= 4;
    using V = typename std::conditional<sizeof(S) == 4, typename std::conditional<kNarrow, float2, float4>::type,
                                        double2>::type;
    constexpr int VEC = kNarrow ? 2 : 16 / (int)sizeof(S);
    constexpr int RQ = 64 / VEC;                               // row vectors of a 64-row segment
    constexpr int NG = kStreamThreads / RQ;                    // column groups
    constexpr int CC = kChunkBytes / (64 * (int)sizeof(S));   // columns per chunk
    constexpr int CPG = CC / NG;                               // columns per group per chunk
    constexpr int FOLDC = 4;                                   // chunks between compensated folds
    constexpr bool kFold = sizeof(A) == 4;                     // FP64 sums plainly
    static_assert(CPG * NG == CC && NG * RQ == kStreamThreads, "chunk geometry");
    extern __shared__ unsigned char stream_smem[];
    const int seg_lo = cta_seg[blockIdx.x], seg_hi = cta_seg[blockIdx.x + 1];
    if (seg_lo >= seg_hi) return;
    const int tid = threadIdx.x, rv = tid % RQ, grp = tid / RQ;
    const int lane = tid & 31, warp = tid >> 5;
    const int k = ma.k;
    unsigned char *ring = stream_smem;
    uint64_t *full = reinterpret_cast<uint64_t *>(stream_smem + (size_t)nst * kChunkBytes);
    uint64_t *never = full + nst;                              // nothing arrives on it (stall hook)
    A *gbuf = reinterpret_cast<A *>(full + nst + 1);
    A *red = gbuf + ngb * gcap * KB;                           // [warp][row][q][hi, lo]
    // the CTA's segment and piece records, staged once (records of one CTA
    // are consecutive in both arrays)
    hm_seg *sseg = reinterpret_cast<hm_seg *>(red + 8 * 64 * KB * 2);
    hm_piece *spc = reinterpret_cast<hm_piece *>(sseg + dsegs);
    {
        const int ns = seg_hi - seg_lo;
        const int p_lo = segs[seg_lo].piece0;
        const int np = segs[seg_hi - 1].piece0 + segs[seg_hi - 1].npieces - p_lo;
        const int64_t *gs = reinterpret_cast<const int64_t *>(segs + seg_lo);
        int64_t *ds = reinterpret_cast<int64_t *>(sseg);
        for (int i = tid; i < ns * (int)(sizeof(hm_seg) / 8); i += kStreamThreads) ds[i] = gs[i];
        const int64_t *gp = reinterpret_cast<const int64_t *>(pieces + p_lo);
        int64_t *dp = reinterpret_cast<int64_t *>(spc);
        for (int i = tid; i < np * (int)(sizeof(hm_piece) / 8); i += kStreamThreads) dp[i] = gp[i];
        __syncthreads();
        for (int i = tid; i < ns; i += kStreamThreads) sseg[i].piece0 -= p_lo;
        __syncthreads();
    }

    auto part_range = [&](const hm_seg &G, int &cb, int &ce) {
        cb = FAR ? 0 : G.nfar;
        ce = FAR ? G.nfar : G.width;
    };
    // right-hand side entries of segment j's part columns into dst (cp.async)
    auto gather = [&](int j, A *dst) {
        const hm_seg G = sseg[j - seg_lo];
        int col = 0;
        for (int pc = 0; pc < G.npieces; ++pc) {
            const hm_piece Q = spc[G.piece0 + pc];
            const bool take = FAR ? (Q.kind != HM_PIECE_X) : (Q.kind == HM_PIECE_X);
            if (!take) continue;
            for (int i = tid; i < Q.width * KB; i += kStreamThreads) {
                const int c = i / KB, q = i % KB;
                A *d = dst + (col + c) * KB + q;
                if (q < k) {
                    const void *src;
                    if (FAR)
                        src = (Q.kind == HM_PIECE_TCOEF ? t : s) + ((int64_t)Q.src * k + q) * r + c;
                    else
                        src = ma.x + (Q.src + c) * ma.incx + (int64_t)q * ma.ldx;
                    async_copy<sizeof(A)>(d, src);
                } else {
                    *d = A(0);
                }
            }
            col += Q.width;
        }
    };

    // producer state (thread 0): next chunk to issue
    int pj = seg_lo, pc = 0, pce = 0, pld = 0, issued = 0;
    int64_t pbase = 0;
    auto seek = [&](int j) {
        for (; j < seg_hi; ++j) {
            const hm_seg G = sseg[j - seg_lo];
            int cb, ce;
            part_range(G, cb, ce);
            if (ce > cb) {
                pc = cb; pce = ce; pld = G.ld; pbase = G.poff;
                break;
            }
        }
        pj = j;
    };
    auto issue = [&](int stage) {
        const int cols = min(CC, pce - pc);
        const uint32_t bytes = (uint32_t)(cols * pld) * (uint32_t)sizeof(S);
        bulk_load(ring + (size_t)stage * kChunkBytes, P + pbase + (int64_t)pc * pld, bytes, &full[stage]);
        ++issued;
        pc += CC;
        if (pc >= pce) seek(pj + 1);
    };

    if (tid == 0) {
        for (int i = 0; i <= nst; ++i) mbar_init(&full[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // right-hand sides run ngb - 1 segments ahead (one cp.async group per segment)
    for (int j = seg_lo; j < seg_lo + ngb - 1; ++j) {
        if (j < seg_hi) gather(j, gbuf + ((j - seg_lo) % ngb) * gcap * KB);
        async_commit();
    }
    __syncthreads();
    if (tid == 0) {
        seek(seg_lo);
        for (int i = 0; i < nst && pj < seg_hi; ++i) issue(i);
    }

    int stage = 0, consumed = 0;
    uint32_t phase = 0;
    bool abort = false;
    bool stall_first = stall != 0;
    for (int j = seg_lo; j < seg_hi && !abort; ++j) {
        async_wait_pending(ngb - 2);
        __syncthreads();                      // g of segment j visible; g and partials of j - 1 read
        {
            const int ja = j + ngb - 1;       // into the buffer segment j - 1 used
            if (ja < seg_hi) gather(ja, gbuf + ((ja - seg_lo) % ngb) * gcap * KB);
            async_commit();
        }
        const hm_seg G = sseg[j - seg_lo];
        int cb, ce;
        part_range(G, cb, ce);
        const A *g = gbuf + ((j - seg_lo) % ngb) * gcap * KB;
        const int row0 = VEC * rv;
        const bool live = row0 < G.nrows;
        const bool acc_y = FAR ? (yfar == nullptr && ce > cb) : (ma.accumulate != 0);
        A part[VEC][KB], hi[VEC][KB], lo[VEC][KB];
#pragma unroll
        for (int v = 0; v < VEC; ++v)
#pragma unroll
            for (int q = 0; q < KB; ++q) part[v][q] = hi[v][q] = lo[v][q] = A(0);
        // the final merge: thread t combines the partials of row t / 4 (the
        // four threads of a row sit in one warp); t % 4 == 0 writes the row
        const int mrow = tid >> 2, mpart = tid & 3;
        const bool writer = mpart == 0 && mrow < G.nrows;
        // y values the segment adds to, loaded now and used at its end
        S yold[KB];
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            yold[q] = S(0);
            if (acc_y && writer && q < k) yold[q] = ma.y[(G.row0 + mrow) * ma.incy + (int64_t)q * ma.ldy];
        }
        int nchunk = 0;
        for (int c0 = cb; c0 < ce; c0 += CC) {
            const int cols = min(CC, ce - c0);
            const bool ok = mbar_wait_first(&full[stage], phase, wait_ns, stall_first, never);
            if (ok && live) {
                const S *st = reinterpret_cast<const S *>(ring + (size_t)stage * kChunkBytes);
#pragma unroll
                for (int u = 0; u < CPG; ++u) {
                    const int c = grp * CPG + u;
                    if (c < cols) {
                        const V pv = *reinterpret_cast<const V *>(st + c * G.ld + row0);
                        const A *gc = g + (c0 - cb + c) * KB;
                        A pr[VEC];
                        if constexpr (VEC == 4) {
                            pr[0] = pv.x; pr[1] = pv.y; pr[2] = pv.z; pr[3] = pv.w;
                        } else {
                            pr[0] = pv.x; pr[1] = pv.y;
                        }
#pragma unroll
                        for (int q = 0; q < KB; ++q) {
                            const A gq = gc[q];
#pragma unroll
                            for (int v = 0; v < VEC; ++v) part[v][q] = fma(pr[v], gq, part[v][q]);
                        }
                    }
                }
                if (kFold && ++nchunk == FOLDC) {
                    nchunk = 0;
#pragma unroll
                    for (int v = 0; v < VEC; ++v)
#pragma unroll
                        for (int q = 0; q < KB; ++q) { fold(hi[v][q], lo[v][q], part[v][q]); part[v][q] = A(0); }
                }
            }
            if (__syncthreads_or(!ok)) {      // every thread leaves together
                abort = true;
                break;
            }
            ++consumed;
            if (tid == 0 && pj < seg_hi) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(stage);
            }
            if (++stage == nst) { stage = 0; phase ^= 1; }
        }
        if (abort) break;
#pragma unroll
        for (int v = 0; v < VEC; ++v)
#pragma unroll
            for (int q = 0; q < KB; ++q) fold(hi[v][q], lo[v][q], part[v][q]);
        // the column groups of a warp first (float: lanes l and l + 16 hold the same rows)
        if constexpr (RQ == 16) {
#pragma unroll
            for (int v = 0; v < VEC; ++v)
#pragma unroll
                for (int q = 0; q < KB; ++q) {
                    const A oh = __shfl_xor_sync(0xffffffffu, hi[v][q], 16);
                    const A ol = __shfl_xor_sync(0xffffffffu, lo[v][q], 16);
                    fold(hi[v][q], lo[v][q], oh);
                    lo[v][q] += ol;
                }
        }
        // every warp's partial to shared memory: red[warp][row][q][hi, lo]
        const bool holder = RQ == 16 ? lane < 16 : true;
        if (holder && live) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                A *rd = red + (warp * 64 + row0 + v) * KB * 2;
#pragma unroll
                for (int q = 0; q < KB; ++q) { rd[2 * q] = hi[v][q]; rd[2 * q + 1] = lo[v][q]; }
            }
        }
        __syncthreads();
        // fixed-order tree: warps (2p, 2p + 1) per thread, then lanes ^1, ^2
        if (mrow < 64) {
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                A h0 = A(0), l0 = A(0);
                if (mrow < G.nrows) {
                    const A *ra = red + ((2 * mpart) * 64 + mrow) * KB * 2;
                    const A *rb = red + ((2 * mpart + 1) * 64 + mrow) * KB * 2;
                    h0 = ra[2 * q];
                    l0 = ra[2 * q + 1];
                    fold(h0, l0, rb[2 * q]);
                    l0 += rb[2 * q + 1];
                }
#pragma unroll
                for (int o = 1; o <= 2; o <<= 1) {
                    const A oh = __shfl_xor_sync(0xffffffffu, h0, o);
                    const A ol = __shfl_xor_sync(0xffffffffu, l0, o);
                    fold(h0, l0, oh);
                    l0 += ol;
                }
                if (writer && q < k && !(FAR && !yfar && ce == cb)) {
                    const A val = h0 + l0;
                    if (FAR && yfar)
                        yfar[(G.row0 + mrow) + (int64_t)q * ma.ldy] = (S)val;
                    else {
                        S *yp = ma.y + (G.row0 + mrow) * ma.incy + (int64_t)q * ma.ldy;
                        *yp = acc_y ? (S)((A)yold[q] + val) : (S)val;
                    }
                }
            }
        }
    }
    if (abort) {
        async_wait_all();
        if (tid == 0) {
            atomicExch(status, HM_DEV_WAIT_TIMEOUT);
            for (int m = consumed; m < issued; ++m) mbar_wait(&full[m % nst], (m / nst) & 1, kDrainLimitNs);
        }
    }
}

// Row segments, several right-hand sides.  One CTA (128 threads) per
// segment: the whole column-major panel is staged once in shared memory
// (16-byte streaming loads), then right-hand sides are processed in chunks
// of QC: the gathered [s ; x pieces] chunk goes to shared memory and each
// thread accumulates an RB-row x QB-column register tile.  Each piece is
// summed in plain FMA and folded into the output with a compensated
// (TwoSum) addition.
template <typename A>
struct KTile;
template <> struct KTile<float> { static constexpr int RB = 4, QB = 4, RG = 16, QG = 8; };   // 64 rows x 32 rhs
template <> struct KTile<double> { static constexpr int RB = 2, QB = 4, RG = 32, QG = 4; };  // 64 rows x 16 rhs

// n consecutive shared-memory values (16-byte aligned) converted to A.
template <typename S, typename A, int n>
__device__ __forceinline__ void load_vec(const S *p, A *out)
{
    if (sizeof(S) * n == 16) {
        if (sizeof(S) == 4) {
            const float4 v = *reinterpret_cast<const float4 *>(p);
            out[0] = (A)v.x; out[1] = (A)v.y; out[2] = (A)v.z; out[3] = (A)v.w;
        } else {
            const double2 v = *reinterpret_cast<const double2 *>(p);
            out[0] = (A)v.x; out[1] = (A)v.y;
        }
    } else if (sizeof(S) * n == 32 && sizeof(S) == 8) {
        const double2 v0 = *reinterpret_cast<const double2 *>(p), v1 = *reinterpret_cast<const double2 *>(p + 2);
        out[0] = (A)v0.x; out[1] = (A)v0.y; out[2] = (A)v1.x; out[3] = (A)v1.y;
    } else {
#pragma unroll
        for (int i = 0; i < n; ++i) out[i] = (A)p[i];
    }
}

template <typename A>
__device__ __forceinline__ void comp_add(A &hi, A &lo, A v)
{
    const A t = hi + v;
    const A bp = t - hi;
    lo += (hi - (t - bp)) + (v - bp);
    hi = t;
}

template <typename S, typename A>
__global__ void expand_k(MulArgs<S> ma, const hm_seg *segs, const hm_piece *pieces, const S *P, const A *s,
                         const A *t, int r, int maxw)
{
    constexpr int RB = KTile<A>::RB, QB = KTile<A>::QB, RG = KTile<A>::RG, QG = KTile<A>::QG;
    constexpr int QC = QB * QG;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const hm_seg G = segs[blockIdx.x];
    S *Ps = reinterpret_cast<S *>(smem_raw);                              // ld x width
    A *Gs = reinterpret_cast<A *>(smem_raw + (((size_t)64 * maxw * sizeof(S) + 31) / 32) * 32);  // QC x width
    {
        // the whole panel in flight at once
        const int n16 = (int)((int64_t)G.ld * G.width * sizeof(S) / 16);
        const char *src = reinterpret_cast<const char *>(P + G.poff);
        char *dst = reinterpret_cast<char *>(Ps);
        for (int i = threadIdx.x; i < n16; i += blockDim.x) async_copy16(dst + 16 * i, src + 16 * i);
    }
    const int W = G.width;
    const int rg = threadIdx.x % RG, qg = threadIdx.x / RG;
    for (int q0 = 0; q0 < ma.k; q0 += QC) {
        const int qc = min(QC, ma.k - q0);
        __syncthreads();                      // the previous chunk's Gs is consumed
        // gathered [s ; x pieces] chunk, right-hand side major: Gs[qq * W + c];
        // consecutive threads take consecutive entries of one right-hand side
        int col = 0;
        for (int pc = 0; pc < G.npieces; ++pc) {
            const hm_piece Q = pieces[G.piece0 + pc];
            for (int idx = threadIdx.x; idx < Q.width * QC; idx += blockDim.x) {
                const int qq = idx / Q.width, c = idx - qq * Q.width;
                A *d = Gs + qq * W + col + c;
                if (qq < qc) {
                    if (Q.kind == HM_PIECE_X)
                        async_copy<sizeof(A)>(d, ma.x + (Q.src + c) * ma.incx + (int64_t)(q0 + qq) * ma.ldx);
                    else
                        async_copy<sizeof(A)>(d, (Q.kind == HM_PIECE_TCOEF ? t : s) +
                                                     ((int64_t)Q.src * ma.k + q0 + qq) * r + c);
                } else {
                    *d = A(0);
                }
            }
            col += Q.width;
        }
        async_wait_all();
        __syncthreads();
        A hi[RB][QB], lo[RB][QB];
#pragma unroll
        for (int i = 0; i < RB; ++i)
#pragma unroll
            for (int j = 0; j < QB; ++j) { hi[i][j] = 0; lo[i][j] = 0; }
        if (rg * RB < G.ld) {
            int c = 0;
            for (int pc = 0; pc < G.npieces; ++pc) {
                const int cend = c + pieces[G.piece0 + pc].width;
                A part[RB][QB];
#pragma unroll
                for (int i = 0; i < RB; ++i)
#pragma unroll
                    for (int j = 0; j < QB; ++j) part[i][j] = 0;
                for (; c < cend; ++c) {
                    A pv[RB], gv[QB];
                    load_vec<S, A, RB>(Ps + (int64_t)c * G.ld + rg * RB, pv);
#pragma unroll
                    for (int j = 0; j < QB; ++j) gv[j] = Gs[(qg * QB + j) * W + c];
#pragma unroll
                    for (int i = 0; i < RB; ++i)
#pragma unroll
                        for (int j = 0; j < QB; ++j) part[i][j] = fma(pv[i], gv[j], part[i][j]);
                }
#pragma unroll
                for (int i = 0; i < RB; ++i)
#pragma unroll
                    for (int j = 0; j < QB; ++j) comp_add(hi[i][j], lo[i][j], part[i][j]);
            }
        }
#pragma unroll
        for (int i = 0; i < RB; ++i) {
            const int row = rg * RB + i;
            if (row >= G.nrows) continue;
#pragma unroll
            for (int j = 0; j < QB; ++j) {
                const int q = qg * QB + j;
                if (q >= qc) continue;
                S *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)(q0 + q) * ma.ldy;
                A v = hi[i][j] + lo[i][j];
                if (ma.accumulate) v += (A)(*yp);
                *yp = (S)v;
            }
        }
    }
}

#define HM_INST_PART(S, A, KB)                                                                       \
    template __global__ void expand_part<S, A, false, KB>(MulArgs<S>, const hm_seg *, int, const hm_piece *, \
                                                          const S *, const A *, const A *, int, int, S *, \
                                                          int64_t);                                     \
    template __global__ void expand_part<S, A, true, KB>(MulArgs<S>, const hm_seg *, int, const hm_piece *,  \
                                                         const S *, const A *, const A *, int, int, S *,  \
                                                         int64_t);
#define HM_INST_STREAM(S, A, KB)                                                                      \
    template __global__ void stream_part<S, A, false, KB>(MulArgs<S>, const hm_seg *, const int *,       \
                                                          const hm_piece *, const S *, const A *, const A *, \
                                                          int, int, int, int, int, S *, int *,          \
                                                          unsigned long long, int);                     \
    template __global__ void stream_part<S, A, true, KB>(MulArgs<S>, const hm_seg *, const int *,        \
                                                         const hm_piece *, const S *, const A *, const A *,  \
                                                         int, int, int, int, int, S *, int *,           \
                                                         unsigned long long, int);
#define HM_INST_FAR(S, A, KB)                                                                        \
    template __global__ void far_rows<S, A, KB>(MulArgs<S>, const hm_seg *, int, const hm_piece *, const S *, \
                                                const A *, const A *, int, S *, int64_t);
HM_INST_FAR(float, float, 4) HM_INST_FAR(float, float, 8) HM_INST_FAR(double, double, 4)
HM_INST_FAR(double, double, 8)
#define HM_INST_MV(S, A)                                                                             \
    template __global__ void leaf_up<S, A, 1>(MulArgs<S>, const hm_vpanel *, int, const S *, A *, int, int, int); \
    template __global__ void leaf_up<S, A, 8>(MulArgs<S>, const hm_vpanel *, int, const S *, A *, int, int, int); \
    template __global__ void m2l<S, A, 1>(const hm_m2l_row *, int, const hm_m2l_ent *, const S *, int,    \
                                          const A *, A *, int, int);                                    \
    template __global__ void m2l<S, A, 8>(const hm_m2l_row *, int, const hm_m2l_ent *, const S *, int,    \
                                          const A *, A *, int, int);                                    \
    template __global__ void m2l_k<S, A, 8>(const hm_m2l_row *, int, const hm_m2l_ent *, const S *, int,  \
                                            const A *, A *, int, int);                                  \
    HM_INST_PART(S, A, 1) HM_INST_PART(S, A, 2) HM_INST_PART(S, A, 4) HM_INST_PART(S, A, 8)               \
    HM_INST_STREAM(S, A, 1) HM_INST_STREAM(S, A, 2) HM_INST_STREAM(S, A, 4) HM_INST_STREAM(S, A, 8)       \
    template __global__ void expand_k<S, A>(MulArgs<S>, const hm_seg *, const hm_piece *, const S *,  \
                                            const A *, const A *, int, int);                            \
    template __global__ void xfer_up_band<A, 1>(const hm_task *, const hm_step *, const hm_xfer *, const A *, \
                                                A *, int, int);                                         \
    template __global__ void xfer_up_band<A, 8>(const hm_task *, const hm_step *, const hm_xfer *, const A *, \
                                                A *, int, int);                                         \
    template __global__ void xfer_down_band<A, 1>(const hm_task *, const hm_step *, const hm_xfer *,        \
                                                  const A *, A *, int, int);                            \
    template __global__ void xfer_down_band<A, 8>(const hm_task *, const hm_step *, const hm_xfer *,        \
                                                  const A *, A *, int, int);                            \
    template __global__ void xfer_up_task<A, 1>(const hm_task *, const hm_step *, const hm_xfer *, const A *, \
                                                A *, int, int, int);                                    \
    template __global__ void xfer_up_task<A, 8>(const hm_task *, const hm_step *, const hm_xfer *, const A *, \
                                                A *, int, int, int);                                    \
    template __global__ void xfer_down_task<A, 1>(const hm_task *, const hm_step *, const hm_xfer *,        \
                                                  const A *, A *, int, int, int);                       \
    template __global__ void xfer_down_task<A, 8>(const hm_task *, const hm_step *, const hm_xfer *,        \
                                                  const A *, A *, int, int, int);
HM_INST_MV(double, double)
HM_INST_MV(float, float)
template __global__ void add_far<double>(MulArgs<double>, int64_t, const double *, int64_t);
template __global__ void add_far<float>(MulArgs<float>, int64_t, const float *, int64_t);

// ============================================================== direct sums

// out[q] = sum_j f(x[rows[q]], y[j]) b[j] in FP64 with double-double
// accumulation; one CTA per row.  An exact-as-possible dense evaluation used
// to state the error of the compressed product.
__global__ void direct_rows(int kid, const double *x, int64_t nx, const double *y, int64_t ny,
                           const double *b, const int64_t *rows, int64_t nrows, double *out)
{
    __shared__ double hs[32], ls[32];
    const int64_t q = blockIdx.x;
    if (q >= nrows) return;
    const int64_t row = rows[q];
    if (row < 0 || row >= nx) {           // invalid row index: report NaN
        if (threadIdx.x == 0) out[q] = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    const double xi = x[row];
    double s = 0.0, c = 0.0;
    for (int64_t j = threadIdx.x; j < ny; j += blockDim.x) {
        const double f = kernel_eval(kid, xi, y[j]);
        const double p = __dmul_rn(f, b[j]);
        const double pe = fma(f, b[j], -p);
        const double t = __dadd_rn(s, p);
        const double bp = __dsub_rn(t, s);
        const double se = __dadd_rn(__dsub_rn(s, __dsub_rn(t, bp)), __dsub_rn(p, bp));
        s = t;
        c = __dadd_rn(c, __dadd_rn(se, pe));
    }
    // combine (s, c) pairs across the block
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o; o >>= 1) {
        const double s2 = __shfl_down_sync(0xffffffffu, s, o);
        const double c2 = __shfl_down_sync(0xffffffffu, c, o);
        const double t = __dadd_rn(s, s2);
        const double bp = __dsub_rn(t, s);
        const double se = __dadd_rn(__dsub_rn(s, __dsub_rn(t, bp)), __dsub_rn(s2, bp));
        s = t;
        c = __dadd_rn(__dadd_rn(c, c2), se);
    }
    if (lane == 0) { hs[wid] = s; ls[wid] = c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            const double t = __dadd_rn(S, hs[k]);
            const double bp = __dsub_rn(t, S);
            const double se = __dadd_rn(__dsub_rn(S, __dsub_rn(t, bp)), __dsub_rn(hs[k], bp));
            S = t;
            C = __dadd_rn(__dadd_rn(C, ls[k]), se);
        }
        out[q] = __dadd_rn(S, C);
    }
}

}  // namespace hm
