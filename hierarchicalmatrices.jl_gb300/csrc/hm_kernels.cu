// CUDA kernels: batched compression (fill) and the hierarchical matvec.
#include "hm_kernels.cuh"

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
__global__ void fill_f(FillArgs fa, const hm_fill_f *ff, int nblocks, S *F)
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
    S *Fe = F + (int64_t)e * r * r;
    for (int idx = threadIdx.x; idx < r * r; idx += blockDim.x) {
        const int m = idx % r, n = idx / r;
        Fe[idx] = (S)kernel_eval(fa.kernel, xh[m], yh[n]);
    }
}

// Segment panels: the first basis_w columns hold the row basis U[i, m] of the
// segment's deepest row box (src/BarycentricMatrix.jl:256-267), the rest the
// near-field dense blocks f(x_i, y_j) (src/KernelMatrix.jl:57-60).  Column-major
// with leading dimension ld.  One CTA per segment.
template <typename S>
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
#pragma unroll
            for (int m = 0; m < HM_RMAX; ++m)
                if (m < r) Pg[i + (int64_t)G.ld * m] = (S)(w[m] / sum);
        }
        col = Fi.basis_w;
    }
    for (int pc = (Fi.has_basis ? 1 : 0); pc < G.npieces; ++pc) {
        const hm_piece Q = pieces[G.piece0 + pc];
        const int64_t tot = (int64_t)Q.width * G.nrows;
        for (int64_t idx = threadIdx.x; idx < tot; idx += blockDim.x) {
            const int i = (int)(idx % G.nrows), j = (int)(idx / G.nrows);
            Pg[i + (int64_t)G.ld * (col + j)] =
                (S)kernel_eval(fa.kernel, fa.x[G.row0 + i], fa.y[Q.src + j]);
        }
        col += Q.width;
    }
}

template __global__ void fill_vpanels<double>(FillArgs, const hm_vpanel *, const hm_fill_vpanel *, int, double *);
template __global__ void fill_vpanels<float>(FillArgs, const hm_vpanel *, const hm_fill_vpanel *, int, float *);
template __global__ void fill_f<double>(FillArgs, const hm_fill_f *, int, double *);
template __global__ void fill_f<float>(FillArgs, const hm_fill_f *, int, float *);
template __global__ void fill_segments<double>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, double *);
template __global__ void fill_segments<float>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, float *);

// ============================================================== matvec kernels
//
// Coefficients of slot `sl` for right-hand side q live at coef[(sl*k + q)*r + m].

// t[slot] = V^T x over an explicit basis panel.  One warp per (panel, rhs);
// lane m owns basis column m, so the row-major panel is read coalesced and no
// cross-lane reduction is needed.
template <typename S, typename A>
__global__ void leaf_up(MulArgs<S> ma, const hm_vpanel *vp, int npanels, const S *V, A *t, int r)
{
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (int64_t)npanels * ma.k) return;
    const int p = (int)(w / ma.k), q = (int)(w % ma.k);
    const hm_vpanel P = vp[p];
    const S *xq = ma.x + (int64_t)q * ma.ldx;
    Acc<A> acc;
    acc.zero();
    if (lane < r) {
        const S *col = V + P.off + lane;
        int j = 0;
        for (; j + 4 <= P.nrows; j += 4) {
            A x0 = (A)xq[(P.row0 + j) * ma.incx], x1 = (A)xq[(P.row0 + j + 1) * ma.incx];
            A x2 = (A)xq[(P.row0 + j + 2) * ma.incx], x3 = (A)xq[(P.row0 + j + 3) * ma.incx];
            A v0 = (A)col[(int64_t)j * P.ld], v1 = (A)col[(int64_t)(j + 1) * P.ld];
            A v2 = (A)col[(int64_t)(j + 2) * P.ld], v3 = (A)col[(int64_t)(j + 3) * P.ld];
            acc.add(v0, x0); acc.add(v1, x1); acc.add(v2, x2); acc.add(v3, x3);
        }
        for (; j < P.nrows; ++j) acc.add((A)col[(int64_t)j * P.ld], (A)xq[(P.row0 + j) * ma.incx]);
        t[((int64_t)P.slot * ma.k + q) * r + lane] = acc.value();
    }
}

// Upward transfer: t[parent][m] = sum_c sum_m' T_c[m', m] t[child_c][m'].
// T holds T_0 then T_1, each r x r with T_c[m' * r + m].
template <typename A>
__global__ void xfer_up(const hm_xfer *xf, int nx, const A *T, A *t, int r, int k)
{
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (int64_t)nx * k) return;
    const hm_xfer X = xf[w / k];
    const int q = (int)(w % k);
    if (lane >= r) return;
    const A *t0 = t + ((int64_t)X.c0 * k + q) * r;
    const A *t1 = t + ((int64_t)X.c1 * k + q) * r;
    A acc = 0;
    for (int mp = 0; mp < r; ++mp) {
        acc += T[mp * r + lane] * t0[mp];
        acc += T[r * r + mp * r + lane] * t1[mp];
    }
    t[((int64_t)X.slot * k + q) * r + lane] = acc;
}

// Far field: s[slot][m] = sum_e sum_n F_e[m + r n] t[yslot_e][n]
// (the F stage of src/algebra.jl:258-265, per row cluster).
template <typename S, typename A>
__global__ void m2l(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const S *F,
                    const A *t, A *s, int r, int k)
{
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (int64_t)nrows * k) return;
    const hm_m2l_row R = rows[w / k];
    const int q = (int)(w % k);
    if (lane >= r) return;
    Acc<A> acc;
    acc.zero();
    for (int e = R.begin; e < R.end; ++e) {
        const hm_m2l_ent E = ents[e];
        const S *Fe = F + E.foff + lane;
        const A *te = t + ((int64_t)E.yslot * k + q) * r;
        for (int n = 0; n < r; ++n) acc.add((A)Fe[n * r], te[n]);
    }
    s[((int64_t)R.slot * k + q) * r + lane] = acc.value();
}

// Downward transfer: s[child_c][m'] += sum_m T_c[m', m] s[parent][m].
template <typename A>
__global__ void xfer_down(const hm_xfer *xf, int nx, const A *T, A *s, int r, int k)
{
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (int64_t)nx * k) return;
    const hm_xfer X = xf[w / k];
    const int q = (int)(w % k);
    if (lane >= r) return;
    const A *sp = s + ((int64_t)X.slot * k + q) * r;
    A a0 = 0, a1 = 0;
    for (int m = 0; m < r; ++m) {
        const A v = sp[m];
        a0 += T[lane * r + m] * v;
        a1 += T[r * r + lane * r + m] * v;
    }
    s[((int64_t)X.c0 * k + q) * r + lane] += a0;
    s[((int64_t)X.c1 * k + q) * r + lane] += a1;
}

// Row segments: y[rows] (+)= panel * [s coefficients ; x segments].
// One CTA per segment, one thread per row; the gathered right-hand side is
// staged in shared memory, KT right-hand sides at a time.
template <typename S, typename A, int KT>
__global__ void expand(MulArgs<S> ma, const hm_seg *segs, const hm_piece *pieces, const S *P,
                       const A *s, int r)
{
    extern __shared__ unsigned char smem_raw[];
    A *g = reinterpret_cast<A *>(smem_raw);
    const hm_seg G = segs[blockIdx.x];
    const S *Pg = P + G.poff;
    for (int q0 = 0; q0 < ma.k; q0 += KT) {
        const int kt = min(KT, ma.k - q0);
        int col = 0;
        for (int pc = 0; pc < G.npieces; ++pc) {
            const hm_piece Q = pieces[G.piece0 + pc];
            for (int idx = threadIdx.x; idx < Q.width * KT; idx += blockDim.x) {
                const int c = idx / KT, qq = idx % KT;
                A v = 0;
                if (qq < kt) {
                    if (Q.kind == HM_PIECE_COEF)
                        v = s[((int64_t)Q.src * ma.k + q0 + qq) * r + c];
                    else
                        v = (A)ma.x[(Q.src + c) * ma.incx + (int64_t)(q0 + qq) * ma.ldx];
                }
                g[(col + c) * KT + qq] = v;
            }
            col += Q.width;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < G.nrows; i += blockDim.x) {
            Acc<A> acc[KT];
#pragma unroll
            for (int qq = 0; qq < KT; ++qq) acc[qq].zero();
            const S *pr = Pg + i;
            int c = 0;
            for (; c + 4 <= G.width; c += 4) {
                A p0 = (A)pr[(int64_t)G.ld * c], p1 = (A)pr[(int64_t)G.ld * (c + 1)];
                A p2 = (A)pr[(int64_t)G.ld * (c + 2)], p3 = (A)pr[(int64_t)G.ld * (c + 3)];
#pragma unroll
                for (int qq = 0; qq < KT; ++qq) {
                    acc[qq].add(p0, g[c * KT + qq]);
                    acc[qq].add(p1, g[(c + 1) * KT + qq]);
                    acc[qq].add(p2, g[(c + 2) * KT + qq]);
                    acc[qq].add(p3, g[(c + 3) * KT + qq]);
                }
            }
            for (; c < G.width; ++c) {
                A p0 = (A)pr[(int64_t)G.ld * c];
#pragma unroll
                for (int qq = 0; qq < KT; ++qq) acc[qq].add(p0, g[c * KT + qq]);
            }
#pragma unroll
            for (int qq = 0; qq < KT; ++qq) {
                if (qq < kt) {
                    S *yp = ma.y + (G.row0 + i) * ma.incy + (int64_t)(q0 + qq) * ma.ldy;
                    A v = acc[qq].value();
                    if (ma.accumulate) v += (A)(*yp);
                    *yp = (S)v;
                }
            }
        }
        __syncthreads();
    }
}

#define HM_INST_MV(S, A)                                                                        \
    template __global__ void leaf_up<S, A>(MulArgs<S>, const hm_vpanel *, int, const S *, A *, int); \
    template __global__ void m2l<S, A>(const hm_m2l_row *, int, const hm_m2l_ent *, const S *,   \
                                       const A *, A *, int, int);                               \
    template __global__ void expand<S, A, 1>(MulArgs<S>, const hm_seg *, const hm_piece *,       \
                                             const S *, const A *, int);                        \
    template __global__ void expand<S, A, 4>(MulArgs<S>, const hm_seg *, const hm_piece *,       \
                                             const S *, const A *, int);                        \
    template __global__ void expand<S, A, 8>(MulArgs<S>, const hm_seg *, const hm_piece *,       \
                                             const S *, const A *, int);
HM_INST_MV(double, double)
HM_INST_MV(float, float)
template __global__ void xfer_up<double>(const hm_xfer *, int, const double *, double *, int, int);
template __global__ void xfer_up<float>(const hm_xfer *, int, const float *, float *, int, int);
template __global__ void xfer_down<double>(const hm_xfer *, int, const double *, double *, int, int);
template __global__ void xfer_down<float>(const hm_xfer *, int, const float *, float *, int, int);

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
