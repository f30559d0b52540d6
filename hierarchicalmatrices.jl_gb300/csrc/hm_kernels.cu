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
template __global__ void fill_f<double>(FillArgs, const hm_fill_f *, const hm_m2l_ent *, int, double *);
template __global__ void fill_f<float>(FillArgs, const hm_fill_f *, const hm_m2l_ent *, int, float *);
template __global__ void fill_segments<double>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, double *);
template __global__ void fill_segments<float>(FillArgs, const hm_seg *, const hm_piece *, const hm_fill_seg *, int, float *);

// ============================================================== matvec kernels
//
// Coefficients of slot `sl` for right-hand side q live at coef[(sl*k + q)*r + m].
// A product is three launches: up_pass, down_pass, then expand1/expand.

// Upward pass in one launch.  One warp per explicit column basis panel:
// t[leaf] = V^T x (lane m owns basis column m of the row-major panel, so
// loads are coalesced and need no cross-lane reduction), then the warp
// climbs the column tree: at each parent the second child to arrive (an
// atomic counter) computes t[parent] = sum_c T_c^T t[child_c] and climbs on,
// the first simply stops.  Nothing waits, so the launch always completes.
// The second arrival resets the counter, leaving it zero for the next call.
template <typename S, typename A>
__global__ void up_pass(MulArgs<S> ma, const hm_vpanel *vp, int npanels, const S *V, const hm_xfer *up,
                        const int32_t *yparent, const A *T, A *t, int *cnt, int r)
{
    extern __shared__ unsigned char smem_raw[];
    A *Ts = reinterpret_cast<A *>(smem_raw);
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) Ts[i] = T[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= npanels) return;
    const hm_vpanel P = vp[w];
    const int k = ma.k;
    for (int q = 0; q < k; ++q) {
        const S *xq = ma.x + (int64_t)q * ma.ldx + P.row0 * ma.incx;
        Acc<A> acc;
        acc.zero();
        if (lane < r) {
            const S *col = V + P.off + lane;
            int j = 0;
            for (; j + 4 <= P.nrows; j += 4) {
                const A x0 = (A)xq[(int64_t)j * ma.incx], x1 = (A)xq[(int64_t)(j + 1) * ma.incx];
                const A x2 = (A)xq[(int64_t)(j + 2) * ma.incx], x3 = (A)xq[(int64_t)(j + 3) * ma.incx];
                const A v0 = (A)col[(int64_t)j * P.ld], v1 = (A)col[(int64_t)(j + 1) * P.ld];
                const A v2 = (A)col[(int64_t)(j + 2) * P.ld], v3 = (A)col[(int64_t)(j + 3) * P.ld];
                acc.add(v0, x0); acc.add(v1, x1); acc.add(v2, x2); acc.add(v3, x3);
            }
            for (; j < P.nrows; ++j) acc.add((A)col[(int64_t)j * P.ld], (A)xq[(int64_t)j * ma.incx]);
            t[((int64_t)P.slot * k + q) * r + lane] = acc.value();
        }
    }
    int slot = P.slot;
    for (;;) {
        const int p = yparent[slot];
        if (p < 0) break;
        __syncwarp();
        int old = 0;
        if (lane == 0) {
            __threadfence();
            old = atomicAdd(&cnt[p], 1);
        }
        old = __shfl_sync(0xffffffffu, old, 0);
        if (old == 0) break;                    // first child here: the sibling climbs on
        if (lane == 0) cnt[p] = 0;
        __threadfence();
        const hm_xfer X = up[p];
        for (int q = 0; q < k; ++q) {
            if (lane < r) {
                const A *t0 = t + ((int64_t)X.c0 * k + q) * r;
                const A *t1 = t + ((int64_t)X.c1 * k + q) * r;
                A a = 0;
                for (int mp = 0; mp < r; ++mp) {
                    a += Ts[mp * r + lane] * __ldcg(t0 + mp);
                    a += Ts[r * r + mp * r + lane] * __ldcg(t1 + mp);
                }
                t[((int64_t)X.slot * k + q) * r + lane] = a;
            }
        }
        slot = X.slot;
    }
}

// Far field and downward pass in one launch.  Warps take row slots in
// level order from a ticket counter.  For its slot a warp forms
//   s[slot] = sum_e F_e t[yslot_e]            (the F stage of src/algebra.jl:258-265)
// staging each r x r block in shared memory with 16-byte loads, then waits
// for its parent slot's flag and adds T_c s[parent] (the downward transfer),
// and publishes its own flag.  A parent always holds a lower ticket than its
// children, so it was taken by a running warp: every wait ends.  Waits are
// still bounded; on the bound the warp records an error in err[0] and goes on.
#define HM_SPIN_LIMIT (1 << 22)
template <typename S, typename A>
__global__ void down_pass(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const S *F, int fstride,
                          const int32_t *xparent, const A *T, const A *t, A *s, int *flags, int *ticket,
                          int *err, int r, int k)
{
    extern __shared__ unsigned char smem_raw[];
    A *Ts = reinterpret_cast<A *>(smem_raw);
    S *Fb = reinterpret_cast<S *>(smem_raw + sizeof(A) * 2 * r * r) + (threadIdx.x >> 5) * fstride;
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) Ts[i] = T[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    constexpr int QC = 8;
    constexpr int VE = 16 / sizeof(S);         // elements per 16-byte load
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(ticket, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nrows) break;
        const hm_m2l_row R = rows[item];
        const int slot = R.slot;
        for (int q0 = 0; q0 < k; q0 += QC) {
            const int qc = min(QC, k - q0);
            A acc[QC];
#pragma unroll
            for (int qq = 0; qq < QC; ++qq) acc[qq] = 0;
            for (int e = R.begin; e < R.end; ++e) {
                const hm_m2l_ent E = ents[e];
                const float4 *src = reinterpret_cast<const float4 *>(F + E.foff);
                float4 *dst = reinterpret_cast<float4 *>(Fb);
                for (int i = lane; i < fstride / VE; i += 32) dst[i] = __ldg(src + i);
                __syncwarp();
                if (lane < r) {
                    const A *te = t + ((int64_t)E.yslot * k + q0) * r;
                    for (int n = 0; n < r; ++n) {
                        const A f = (A)Fb[lane + r * n];
#pragma unroll
                        for (int qq = 0; qq < QC; ++qq)
                            if (qq < qc) acc[qq] += f * te[qq * r + n];
                    }
                }
                __syncwarp();
            }
            if (lane < r) {
#pragma unroll
                for (int qq = 0; qq < QC; ++qq)
                    if (qq < qc) s[((int64_t)slot * k + q0 + qq) * r + lane] = acc[qq];
            }
        }
        const int pp = xparent[slot];
        if (pp >= 0) {
            const int ps = pp >> 1, c = pp & 1;
            if (lane == 0) {
                int it = 0;
                while (*(volatile int *)(flags + ps) == 0) {
                    if (++it > HM_SPIN_LIMIT) { atomicExch(err, 1); break; }
                    __nanosleep(64);
                }
            }
            __syncwarp();
            __threadfence();
            if (lane < r) {
                const A *Tc = Ts + c * r * r + lane * r;
                for (int q = 0; q < k; ++q) {
                    const A *sp = s + ((int64_t)ps * k + q) * r;
                    A a = 0;
                    for (int m = 0; m < r; ++m) a += Tc[m] * __ldcg(sp + m);
                    s[((int64_t)slot * k + q) * r + lane] += a;
                }
            }
        }
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            atomicExch(flags + slot, 1);
        }
    }
}

// Clears the flags and the ticket of down_pass so the next call starts from
// zero (runs in the launch that follows down_pass).
__device__ __forceinline__ void clear_sync(int *flags, int nflags, int *ticket)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < nflags; i += nth) flags[i] = 0;
    if (tid == 0 && ticket) *ticket = 0;
}

// Row segments, one right-hand side: one warp per segment (<= 64 rows).
// FP32: lanes 0-15 and 16-31 take alternate panel columns, each lane four
// consecutive rows through one 16-byte load per column; FP64: each lane two
// rows per 16-byte load.  The gathered right-hand side [s ; x pieces] is
// staged per warp in shared memory.  FP32 products accumulate with
// compensated (TwoProd/TwoSum) sums.
template <typename S, typename A>
__global__ void expand1(MulArgs<S> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const S *P,
                        const A *s, int r, int maxw, int *flags, int nflags, int *ticket)
{
    extern __shared__ unsigned char smem_raw[];
    clear_sync(flags, nflags, ticket);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int seg = blockIdx.x * (blockDim.x >> 5) + wib;
    if (seg >= nsegs) return;
    A *g = reinterpret_cast<A *>(smem_raw) + (int64_t)wib * maxw;
    const hm_seg G = segs[seg];
    int col = 0;
    for (int pc = 0; pc < G.npieces; ++pc) {
        const hm_piece Q = pieces[G.piece0 + pc];
        for (int c = lane; c < Q.width; c += 32)
            g[col + c] = (Q.kind == HM_PIECE_COEF) ? s[Q.src * r + c] : (A)ma.x[(Q.src + c) * ma.incx];
        col += Q.width;
    }
    __syncwarp();
    const S *Pg = P + G.poff;
    if (sizeof(S) == 4) {
        const int rg = lane & 15, h = lane >> 4;
        Acc<A> acc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j].zero();
        if (4 * rg < G.ld) {
            const float4 *base = reinterpret_cast<const float4 *>(Pg + 4 * rg);
            const int64_t ld4 = G.ld / 4;
            int c = h;
            for (; c + 6 < G.width; c += 8) {
                const float4 p0 = __ldcs(base + ld4 * c), p1 = __ldcs(base + ld4 * (c + 2));
                const float4 p2 = __ldcs(base + ld4 * (c + 4)), p3 = __ldcs(base + ld4 * (c + 6));
                const A g0 = g[c], g1 = g[c + 2], g2 = g[c + 4], g3 = g[c + 6];
                acc[0].add(p0.x, g0); acc[1].add(p0.y, g0); acc[2].add(p0.z, g0); acc[3].add(p0.w, g0);
                acc[0].add(p1.x, g1); acc[1].add(p1.y, g1); acc[2].add(p1.z, g1); acc[3].add(p1.w, g1);
                acc[0].add(p2.x, g2); acc[1].add(p2.y, g2); acc[2].add(p2.z, g2); acc[3].add(p2.w, g2);
                acc[0].add(p3.x, g3); acc[1].add(p3.y, g3); acc[2].add(p3.z, g3); acc[3].add(p3.w, g3);
            }
            for (; c < G.width; c += 2) {
                const float4 p0 = __ldcs(base + ld4 * c);
                const A g0 = g[c];
                acc[0].add(p0.x, g0); acc[1].add(p0.y, g0); acc[2].add(p0.z, g0); acc[3].add(p0.w, g0);
            }
        }
        // fold the two column halves: (s, c) pairs combined with TwoSum
        A val[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const A so = __shfl_xor_sync(0xffffffffu, acc[j].s_hi(), 16);
            const A co = __shfl_xor_sync(0xffffffffu, acc[j].s_lo(), 16);
            val[j] = acc[j].merged(so, co);
        }
        if (h == 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int row = 4 * rg + j;
                if (row < G.nrows) {
                    S *yp = ma.y + (G.row0 + row) * ma.incy;
                    A v = val[j];
                    if (ma.accumulate) v += (A)(*yp);
                    *yp = (S)v;
                }
            }
        }
    } else {
        Acc<A> a0, a1;
        a0.zero(); a1.zero();
        if (2 * lane < G.ld) {
            const double2 *base = reinterpret_cast<const double2 *>(Pg + 2 * lane);
            const int64_t ld2 = G.ld / 2;
            int c = 0;
            for (; c + 4 <= G.width; c += 4) {
                const double2 p0 = __ldcs(base + ld2 * c), p1 = __ldcs(base + ld2 * (c + 1));
                const double2 p2 = __ldcs(base + ld2 * (c + 2)), p3 = __ldcs(base + ld2 * (c + 3));
                a0.add(p0.x, g[c]); a1.add(p0.y, g[c]);
                a0.add(p1.x, g[c + 1]); a1.add(p1.y, g[c + 1]);
                a0.add(p2.x, g[c + 2]); a1.add(p2.y, g[c + 2]);
                a0.add(p3.x, g[c + 3]); a1.add(p3.y, g[c + 3]);
            }
            for (; c < G.width; ++c) {
                const double2 p0 = __ldcs(base + ld2 * c);
                a0.add(p0.x, g[c]); a1.add(p0.y, g[c]);
            }
        }
        const A v2[2] = {a0.value(), a1.value()};
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int row = 2 * lane + j;
            if (row < G.nrows) {
                S *yp = ma.y + (G.row0 + row) * ma.incy;
                A v = v2[j];
                if (ma.accumulate) v += (A)(*yp);
                *yp = (S)v;
            }
        }
    }
}

// Row segments, several right-hand sides: one CTA per segment, one thread per
// row; the gathered right-hand sides are staged in shared memory, KT at a time.
template <typename S, typename A, int KT>
__global__ void expand(MulArgs<S> ma, const hm_seg *segs, const hm_piece *pieces, const S *P,
                       const A *s, int r, int *flags, int nflags, int *ticket)
{
    extern __shared__ unsigned char smem_raw[];
    A *g = reinterpret_cast<A *>(smem_raw);
    clear_sync(flags, nflags, ticket);
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

#define HM_INST_MV(S, A)                                                                             \
    template __global__ void up_pass<S, A>(MulArgs<S>, const hm_vpanel *, int, const S *, const hm_xfer *, \
                                           const int32_t *, const A *, A *, int *, int);                \
    template __global__ void down_pass<S, A>(const hm_m2l_row *, int, const hm_m2l_ent *, const S *, int, \
                                             const int32_t *, const A *, const A *, A *, int *, int *,  \
                                             int *, int, int);                                          \
    template __global__ void expand1<S, A>(MulArgs<S>, const hm_seg *, int, const hm_piece *, const S *, \
                                           const A *, int, int, int *, int, int *);                     \
    template __global__ void expand<S, A, 4>(MulArgs<S>, const hm_seg *, const hm_piece *,            \
                                             const S *, const A *, int, int *, int, int *);             \
    template __global__ void expand<S, A, 8>(MulArgs<S>, const hm_seg *, const hm_piece *,            \
                                             const S *, const A *, int, int *, int, int *);
HM_INST_MV(double, double)
HM_INST_MV(float, float)

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
