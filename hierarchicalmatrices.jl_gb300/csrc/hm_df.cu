// Double-float row-segment panels: the FP64 product's near-field and
// far-field panels stored as pairs of FP32 values and multiplied on the FP32
// pipes.  Written for sm_103a.
//
// GB300 issues FP64 FMAs at about 1/56 of its FP32 rate, so the FP64
// product's panel stage is bound by the FP64 pipe rather than by HBM.  With
// HM_DF64 storage every panel value v (computed in FP64 at build) is kept as
// the pair (h, l) = (fl32(v), fl32(v - h)), the same 8 bytes, which
// represents v to about 2^-48 relative.  A product term p * g (p a panel pair,
// g the right-hand-side entry split the same way when it is gathered) is
//     h = ph * gh,  e = fma(ph, gh, -h) + ph * gl + pl * gh   (Dekker's
// product, the exact error of ph * gh from one FMA, plus the cross terms),
// and is added to the running double-float sum (sh, sl) by Knuth's TwoSum of
// sh and h, the low parts added to its error, and a Fast2Sum renormalisation
// (the "sloppy" double-word addition analysed by Joldes, Muller and Popescu,
// ACM TOMS 44(2), 2017): 15 FP32 operations per term, all rounded to nearest
// (no contraction: the error-free transformations need exact roundings).
// Row results are formed in FP64 as sh + sl.  The column bases V and the
// far-field blocks F are stored the same way and their products (leaf_up_df,
// m2l_df) and the transfers between tree levels (xfer_df, with the transfer
// matrices as pairs) run in the same arithmetic; coefficients stay FP64 in
// memory.
#include "hm_kernels.cuh"
#include "hm_async.cuh"

namespace hm {

namespace {

__device__ __forceinline__ float2 df_split(double v)
{
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(__dsub_rn(v, (double)h)));
}

// (sh, sl) += (ph + pl) (gh + gl)
__device__ __forceinline__ void df_fma(float &sh, float &sl, float ph, float pl, float gh, float gl)
{
    const float h = __fmul_rn(ph, gh);
    float e = __fmaf_rn(ph, gh, -h);
    e = __fmaf_rn(ph, gl, e);
    e = __fmaf_rn(pl, gh, e);
    const float s = __fadd_rn(sh, h);
    const float bp = __fsub_rn(s, sh);
    float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bp)), __fsub_rn(h, bp));
    t = __fadd_rn(t, __fadd_rn(sl, e));
    sh = __fadd_rn(s, t);
    sl = __fsub_rn(t, __fsub_rn(sh, s));
}

}  // namespace

// In place: every FP64 value of P becomes its (h, l) pair; *bad is set when a
// value's magnitude is at or above 2^127, where the pair would overflow.
__global__ void panels_to_df(double *P, int64_t n, int *bad)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = P[i];
        if (!(fabs(v) < 0x1p127)) atomicOr(bad, 1);
        const float2 d = df_split(v);
        reinterpret_cast<float2 *>(P)[i] = d;
    }
}

// One warp per row segment, lane l rows 2l and 2l + 1 (one 16-byte load of
// two (h, l) pairs per column), up to KB right-hand sides q0 .. q0 + KB - 1.
// PART 0: the near-field (X) columns, y (+)= D x per the caller's flag;
// PART 1: the far-field columns, U s into yfar (leading dimension ldf) or,
// without yfar, added into y; PART 2: every column, y (+)= per the caller's
// flag.  The right-hand-side entries of the part are gathered once per
// segment into shared memory as (h, l) pairs (maxw * KB per warp).
template <int PART, int KB>
__global__ void expand_df(MulArgs<double> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const float2 *P,
                          const double *s, const double *t, int r, int maxw, double *yfar, int64_t ldf, int q0)
{
    extern __shared__ float2 df_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int seg = blockIdx.x * (blockDim.x >> 5) + wib;
    if constexpr (PART == 1) pdl_wait();                       // the downward pass's coefficients are ready
    if (seg >= nsegs) return;
    float2 *g = df_smem + (int64_t)wib * maxw * KB;
    const hm_seg G = segs[seg];
    const int k = ma.k;
    int c0 = -1, c1 = 0, col = 0;
    for (int pc = 0; pc < G.npieces; ++pc) {
        const hm_piece Q = pieces[G.piece0 + pc];
        const bool take = PART == 2 ? true : PART == 1 ? (Q.kind != HM_PIECE_X) : (Q.kind == HM_PIECE_X);
        if (take) {
            if (c0 < 0) c0 = col;
            for (int i = lane; i < Q.width * KB; i += 32) {
                const int c = i / KB, q = q0 + i % KB;
                double v = 0.0;
                if (q < k) {
                    if (Q.kind == HM_PIECE_X) v = ma.x[(Q.src + c) * ma.incx + (int64_t)q * ma.ldx];
                    else v = (Q.kind == HM_PIECE_TCOEF ? t : s)[((int64_t)Q.src * k + q) * r + c];
                }
                g[(col + c) * KB + i % KB] = df_split(v);
            }
            c1 = col + Q.width;
        }
        col += Q.width;
    }
    if (c0 < 0) {
        if (PART == 1 && !yfar) return;                        // no far field on these rows
        c0 = c1 = 0;
    }
    __syncwarp();
    float sh[2][KB], sl[2][KB];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int q = 0; q < KB; ++q) sh[j][q] = sl[j][q] = 0.f;
    if (2 * lane < G.ld) {
        const float4 *base = reinterpret_cast<const float4 *>(P + G.poff + 2 * lane);
        const int64_t ld2 = G.ld / 2;                         // float4 (two pairs) per column step
        constexpr int U = KB <= 2 ? 16 : 8;                    // loads in flight per lane
        int c = c0;
        auto use = [&](const float4 &p, int cc) {
            const float2 *gc = g + cc * KB;
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                const float2 gq = gc[q];
                df_fma(sh[0][q], sl[0][q], p.x, p.y, gq.x, gq.y);
                df_fma(sh[1][q], sl[1][q], p.z, p.w, gq.x, gq.y);
            }
        };
        for (; c + U <= c1; c += U) {
            float4 p[U];
#pragma unroll
            for (int u = 0; u < U; ++u) p[u] = __ldcs(base + ld2 * (c + u));
#pragma unroll
            for (int u = 0; u < U; ++u) use(p[u], c + u);
        }
        for (; c < c1; ++c) use(__ldcs(base + ld2 * c), c);
    }
    const bool acc_y = PART == 1 ? (yfar == nullptr) : (ma.accumulate != 0);
#pragma unroll
    for (int q = 0; q < KB; ++q) {
        if (q0 + q >= k) break;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int row = 2 * lane + j;
            if (row < G.nrows) {
                const double v = __dadd_rn((double)sh[j][q], (double)sl[j][q]);
                if (PART == 1 && yfar) {
                    yfar[(G.row0 + row) + (int64_t)(q0 + q) * ldf] = v;
                } else {
                    double *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)(q0 + q) * ma.ldy;
                    *yp = acc_y ? *yp + v : v;
                }
            }
        }
    }
}

// Explicit column bases with HM_DF64 storage (V as (h, l) pairs, row-major,
// ld == width <= 32): t[slot][q][col0 + m] = sum_j V[j][m] x[row0 + j][q] in
// double-float arithmetic on the FP32 pipes, one warp per panel, lane m one
// basis column; the panel's right-hand-side rows are split into pairs once
// per right-hand side in shared memory (cap pairs per warp).  With ma.xin
// (a page-locked host source) the rows are read there and stored into x for
// the kernels after this one, as leaf_up does.
__global__ void leaf_up_df(MulArgs<double> ma, const hm_vpanel *vp, int npanels, const float2 *V, double *t, int r,
                           int cap)
{
    extern __shared__ float2 leaf_df_smem[];
    pdl_trigger();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    if (w >= (int64_t)npanels) return;
    const hm_vpanel P = vp[w];
    float2 *xs = leaf_df_smem + (size_t)wib * cap;
    const float2 *Vp = V + P.off;
    const double *xsrc = ma.xin ? ma.xin : ma.x;
    double *xcopy = ma.xin ? const_cast<double *>(ma.x) : nullptr;
    const int nr = min((int)P.nrows, cap);
    for (int q = 0; q < ma.k; ++q) {
        for (int j = lane; j < P.nrows; j += 32) {
            const int64_t e = (P.row0 + j) * ma.incx + (int64_t)q * ma.ldx;
            const double v = xsrc[e];
            if (xcopy) xcopy[e] = v;
            if (j < nr) xs[j] = df_split(v);
        }
        __syncwarp();
        if (lane < P.width) {
            float sh = 0.f, sl = 0.f;
            int j = 0;
            for (; j + 8 <= nr; j += 8) {
                float2 v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = Vp[(int64_t)(j + u) * P.ld + lane];
#pragma unroll
                for (int u = 0; u < 8; ++u) df_fma(sh, sl, v[u].x, v[u].y, xs[j + u].x, xs[j + u].y);
            }
            for (; j < nr; ++j) {
                const float2 v = Vp[(int64_t)j * P.ld + lane];
                df_fma(sh, sl, v.x, v.y, xs[j].x, xs[j].y);
            }
            // rows past the staged ones (panels longer than cap) straight from x
            for (j = nr; j < P.nrows; ++j) {
                const float2 v = Vp[(int64_t)j * P.ld + lane];
                const float2 xv = df_split(xsrc[(P.row0 + j) * ma.incx + (int64_t)q * ma.ldx]);
                df_fma(sh, sl, v.x, v.y, xv.x, xv.y);
            }
            t[((int64_t)P.slot * ma.k + q) * r + P.col0 + lane] = __dadd_rn((double)sh, (double)sl);
        }
        __syncwarp();
    }
}

// Far-field blocks with HM_DF64 storage (F as (h, l) pairs, r x r column-major
// with fstride pairs between blocks): s[slot][q][m] = sum_e sum_n F_e[m + r n]
// t[yslot_e][q][n], one warp per row slot, lane m one coefficient; each
// block's column coefficients are split into pairs in shared memory (lane n
// splits coefficient n) and the next block's pairs of F are loaded while the
// current block is multiplied.
namespace {
// rank 20: the next block's pairs of F (and its column coefficients) are
// loaded into registers while the current block is multiplied
__device__ __forceinline__ void m2l_df_r20(const hm_m2l_row &R, const hm_m2l_ent *ents, const float2 *F,
                                           const double *t, double *s, int k, int lane, float2 *ts)
{
    constexpr int R20 = 20;
    for (int q = 0; q < k; ++q) {
        float sh = 0.f, sl = 0.f;
        float2 fc[R20];
        double tc = 0.0;
        if (R.begin < R.end && lane < R20) {
            const hm_m2l_ent E = ents[R.begin];
#pragma unroll
            for (int n = 0; n < R20; ++n) fc[n] = F[E.foff + lane + (int64_t)R20 * n];
            tc = t[((int64_t)E.yslot * k + q) * R20 + lane];
        }
        for (int e = R.begin; e < R.end; ++e) {
            if (lane < R20) ts[lane] = df_split(tc);
            __syncwarp();
            float2 fn[R20];
            if (e + 1 < R.end && lane < R20) {
                const hm_m2l_ent E = ents[e + 1];
#pragma unroll
                for (int n = 0; n < R20; ++n) fn[n] = F[E.foff + lane + (int64_t)R20 * n];
                tc = t[((int64_t)E.yslot * k + q) * R20 + lane];
            }
            if (lane < R20) {
#pragma unroll
                for (int n = 0; n < R20; ++n) df_fma(sh, sl, fc[n].x, fc[n].y, ts[n].x, ts[n].y);
            }
            __syncwarp();
#pragma unroll
            for (int n = 0; n < R20; ++n) fc[n] = fn[n];
        }
        if (lane < R20) s[((int64_t)R.slot * k + q) * R20 + lane] = __dadd_rn((double)sh, (double)sl);
    }
}
}  // namespace

// Rank 20 with a per-warp ring of kM2lDfStages blocks of F in shared memory
// filled by cp.async: a warp keeps two blocks (6.4 KB) in flight instead of
// one in registers, and without the 40 registers of the register copy more
// warps fit on an SM (four per CTA, 38.4 KB of ring per CTA).
template <int NS>
__global__ void __launch_bounds__(kM2lDfWarps * 32)
    m2l_df_ring(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const float2 *F, const double *t,
                double *s, int k)
{
    extern __shared__ __align__(16) unsigned char m2l_smem[];
    __shared__ float2 tsh[kM2lDfWarps][32];
    constexpr int R20 = 20, BLK = R20 * R20;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * kM2lDfWarps + wib;
    pdl_trigger();
    pdl_wait();                                                // the upward pass's coefficients are ready
    if (w >= (int64_t)nrows) return;
    float2 *ring = reinterpret_cast<float2 *>(m2l_smem) + (size_t)wib * NS * BLK;
    float2 *ts = tsh[wib];
    const hm_m2l_row R = rows[w];
    const int ne = R.end - R.begin;
    auto issue = [&](int i, int stage) {
        const hm_m2l_ent E = ents[R.begin + i];
        float2 *dst = ring + stage * BLK;
        const float2 *src = F + E.foff;
        if ((E.foff & 1) == 0) {
            for (int c = lane; c < BLK / 2; c += 32) async_copy16(dst + 2 * c, src + 2 * c);
        } else {
            for (int c = lane; c < BLK; c += 32) async_copy<8>(dst + c, src + c);
        }
    };
    for (int q = 0; q < k; ++q) {
        float sh = 0.f, sl = 0.f;
        double tc = 0.0;
        if (ne > 0 && lane < R20) tc = t[((int64_t)ents[R.begin].yslot * k + q) * R20 + lane];
#pragma unroll
        for (int i = 0; i < NS - 1; ++i) {
            if (i < ne) issue(i, i);
            async_commit();
        }
        for (int e = 0; e < ne; ++e) {
            const int ei = e + NS - 1;
            if (ei < ne) issue(ei, ei % NS);
            async_commit();
            asm volatile("cp.async.wait_group %0;" ::"n"(NS - 1) : "memory");
            if (lane < R20) ts[lane] = df_split(tc);
            __syncwarp();                                      // block e and the coefficients visible
            double tn = 0.0;
            if (e + 1 < ne && lane < R20) tn = t[((int64_t)ents[R.begin + e + 1].yslot * k + q) * R20 + lane];
            if (lane < R20) {
                const float2 *f = ring + (e % NS) * BLK + lane;
#pragma unroll
                for (int n = 0; n < R20; ++n) {
                    const float2 v = f[R20 * n];
                    df_fma(sh, sl, v.x, v.y, ts[n].x, ts[n].y);
                }
            }
            __syncwarp();                                      // the stage and ts are free again
            tc = tn;
        }
        async_wait_all();
        __syncwarp();
        if (lane < R20) s[((int64_t)R.slot * k + q) * R20 + lane] = __dadd_rn((double)sh, (double)sl);
    }
}
template __global__ void m2l_df_ring<kM2lDfStages>(const hm_m2l_row *, int, const hm_m2l_ent *, const float2 *,
                                                   const double *, double *, int);

__global__ void m2l_df(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const float2 *F, int fstride,
                       const double *t, double *s, int r, int k)
{
    __shared__ float2 ts[8][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    pdl_trigger();
    pdl_wait();                                                // the upward pass's coefficients are ready
    if (w >= (int64_t)nrows) return;
    const hm_m2l_row R = rows[w];
    if (r == 20) {
        m2l_df_r20(R, ents, F, t, s, k, lane, ts[wib]);
        return;
    }
    for (int q = 0; q < k; ++q) {
        float sh = 0.f, sl = 0.f;
        for (int e = R.begin; e < R.end; ++e) {
            const hm_m2l_ent E = ents[e];
            if (lane < r) ts[wib][lane] = df_split(t[((int64_t)E.yslot * k + q) * r + lane]);
            __syncwarp();
            if (lane < r) {
                const float2 *Fe = F + E.foff + lane;
                int n = 0;
                for (; n + 4 <= r; n += 4) {
                    float2 f[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) f[u] = Fe[(int64_t)r * (n + u)];
#pragma unroll
                    for (int u = 0; u < 4; ++u) df_fma(sh, sl, f[u].x, f[u].y, ts[wib][n + u].x, ts[wib][n + u].y);
                }
                for (; n < r; ++n) {
                    const float2 f = Fe[(int64_t)r * n];
                    df_fma(sh, sl, f.x, f.y, ts[wib][n].x, ts[wib][n].y);
                }
            }
            __syncwarp();
        }
        if (lane < r) s[((int64_t)R.slot * k + q) * r + lane] = __dadd_rn((double)sh, (double)sl);
    }
}

// Transfer bands with HM_DF64 storage (the transfer matrices T_0, T_1 as
// (h, l) pairs, T_c[m' r + m]): the task structure of xfer_up_task /
// xfer_down_task with one right-hand side per CTA (grid: tasks x k), local
// coefficient vectors as pairs in shared memory, products in double-float
// arithmetic; the coefficients in global memory stay FP64 (split when read,
// h + l when written).
//   upward:   t[parent][m] = sum_c sum_m' T_c[m', m] t[child_c][m']
//   downward: s[child_c][m'] += sum_m T_c[m', m] s[parent][m]
template <bool UP>
__global__ void xfer_df(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const float2 *T,
                        double *coef, int r, int k, int early)
{
    extern __shared__ float2 xfer_df_smem[];
    float2 *Ts = xfer_df_smem;                                 // 2 r r pairs
    float2 *L = Ts + 2 * HM_RMAX * HM_RMAX;                    // r pairs per local
    const hm_task tk = tasks[blockIdx.x];
    const int e0 = steps[tk.step0].e0, e1 = steps[tk.step1 - 1].e1, nrec = e1 - e0;
    const int q = blockIdx.y;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (early) pdl_trigger();
    for (int i = threadIdx.x; i < 2 * r * r; i += blockDim.x) Ts[i] = T[i];
    pdl_wait();                                                // inputs of the band are ready
    for (int rec = warp; rec < nrec; rec += nw) {
        const hm_xfer X = ents[e0 + rec];
        if (lane >= r) continue;
#pragma unroll
        for (int c = 0; c < (UP ? 2 : 3); ++c) {
            int lc, slot;
            if (UP) {
                lc = c ? (X.pad >> 16) : (X.pad & 0xffff);
                slot = c ? X.c1 : X.c0;
                if (lc < nrec) continue;                       // produced by an earlier level of this task
            } else if (c < 2) {
                lc = 2 * rec + c;                              // children start from their far-field values
                slot = c ? X.c1 : X.c0;
            } else {
                lc = X.pad;
                slot = X.slot;
                if (lc < 2 * nrec) continue;                   // a child of an earlier level of this task
            }
            L[lc * r + lane] = df_split(coef[((int64_t)slot * k + q) * r + lane]);
        }
    }
    __syncthreads();
    for (int st = tk.step0; st < tk.step1; ++st) {
        const hm_step S = steps[st];
        for (int w = warp; w < S.e1 - S.e0; w += nw) {
            const int e = S.e0 + w;
            const hm_xfer X = ents[e];
            if (lane >= r) continue;
            if (UP) {
                const float2 *c0 = L + (X.pad & 0xffff) * r, *c1 = L + (X.pad >> 16) * r;
                float sh = 0.f, sl = 0.f;
                for (int mp = 0; mp < r; ++mp) {
                    const float2 a0 = Ts[mp * r + lane], a1 = Ts[r * r + mp * r + lane];
                    df_fma(sh, sl, a0.x, a0.y, c0[mp].x, c0[mp].y);
                    df_fma(sh, sl, a1.x, a1.y, c1[mp].x, c1[mp].y);
                }
                L[(e - e0) * r + lane] = make_float2(sh, sl);
                coef[((int64_t)X.slot * k + q) * r + lane] = __dadd_rn((double)sh, (double)sl);
            } else {
                const float2 *p = L + X.pad * r;
                float2 *o0 = L + (2 * (e - e0)) * r, *o1 = o0 + r;
                float h0 = o0[lane].x, l0 = o0[lane].y, h1 = o1[lane].x, l1 = o1[lane].y;
                for (int m = 0; m < r; ++m) {
                    const float2 t0 = Ts[lane * r + m], t1 = Ts[r * r + lane * r + m];
                    df_fma(h0, l0, t0.x, t0.y, p[m].x, p[m].y);
                    df_fma(h1, l1, t1.x, t1.y, p[m].x, p[m].y);
                }
                o0[lane] = make_float2(h0, l0);
                o1[lane] = make_float2(h1, l1);
                coef[((int64_t)X.c0 * k + q) * r + lane] = __dadd_rn((double)h0, (double)l0);
                coef[((int64_t)X.c1 * k + q) * r + lane] = __dadd_rn((double)h1, (double)l1);
            }
        }
        __syncthreads();
    }
}
template __global__ void xfer_df<true>(const hm_task *, const hm_step *, const hm_xfer *, const float2 *, double *,
                                       int, int, int);
template __global__ void xfer_df<false>(const hm_task *, const hm_step *, const hm_xfer *, const float2 *, double *,
                                        int, int, int);

// Far-field rows with HM_DF64 storage, one thread per row (four segments of at
// most 64 rows per CTA of 256 threads): y_far[row] = sum_c U[row][c] s[c] over
// the segment's far columns (at most 64), the coefficients split into pairs
// once per segment in shared memory, the row's pairs read column by column
// (consecutive threads, consecutive rows), double-float accumulation; one
// right-hand side q0.  Rows go to yfar or, without it, are added into y.
__global__ void __launch_bounds__(256)
    far_rows_df(MulArgs<double> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const float2 *P,
                const double *s, const double *t, int r, double *yfar, int64_t ldf, int q0)
{
    __shared__ float2 cs[4][64];
    pdl_wait();                                                // the downward pass's coefficients are ready
    const int ls = threadIdx.x >> 6, row = threadIdx.x & 63;
    const int j = blockIdx.x * 4 + ls;
    const int k = ma.k;
    hm_seg G{};
    int nfar = 0;
    if (j < nsegs) {
        G = segs[j];
        nfar = G.nfar;
        if (row < nfar) {
            int pc = 0, pi = 0;
            hm_piece Q = pieces[G.piece0];
            while (row >= pc + Q.width) {
                pc += Q.width;
                Q = pieces[G.piece0 + ++pi];
            }
            cs[ls][row] = df_split((Q.kind == HM_PIECE_TCOEF ? t : s)[((int64_t)Q.src * k + q0) * r + (row - pc)]);
        }
    }
    __syncthreads();
    if (j >= nsegs || row >= G.nrows) return;
    if (nfar == 0 && !yfar) return;                            // y += 0
    float sh = 0.f, sl = 0.f;
    const float2 *pr = P + G.poff + row;
    int c = 0;
    for (; c + 4 <= nfar; c += 4) {
        float2 u[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) u[i] = pr[(int64_t)(c + i) * G.ld];
#pragma unroll
        for (int i = 0; i < 4; ++i) df_fma(sh, sl, u[i].x, u[i].y, cs[ls][c + i].x, cs[ls][c + i].y);
    }
    for (; c < nfar; ++c) {
        const float2 u = pr[(int64_t)c * G.ld];
        df_fma(sh, sl, u.x, u.y, cs[ls][c].x, cs[ls][c].y);
    }
    const double v = __dadd_rn((double)sh, (double)sl);
    if (yfar) {
        yfar[(G.row0 + row) + (int64_t)q0 * ldf] = v;
    } else {
        double *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)q0 * ma.ldy;
        *yp = *yp + v;
    }
}

#define HM_INST_DF(PART)                                                                                        \
    template __global__ void expand_df<PART, 1>(MulArgs<double>, const hm_seg *, int, const hm_piece *,          \
                                                const float2 *, const double *, const double *, int, int,        \
                                                double *, int64_t, int);                                         \
    template __global__ void expand_df<PART, 2>(MulArgs<double>, const hm_seg *, int, const hm_piece *,          \
                                                const float2 *, const double *, const double *, int, int,        \
                                                double *, int64_t, int);                                         \
    template __global__ void expand_df<PART, 4>(MulArgs<double>, const hm_seg *, int, const hm_piece *,          \
                                                const float2 *, const double *, const double *, int, int,        \
                                                double *, int64_t, int);                                         \
    template __global__ void expand_df<PART, 8>(MulArgs<double>, const hm_seg *, int, const hm_piece *,          \
                                                const float2 *, const double *, const double *, int, int,        \
                                                double *, int64_t, int);
HM_INST_DF(0)
HM_INST_DF(1)
HM_INST_DF(2)

}  // namespace hm
