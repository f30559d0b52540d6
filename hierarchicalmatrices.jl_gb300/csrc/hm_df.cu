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
// Row results are formed in FP64 as sh + sl.  The tree passes (bases,
// transfers, far-field blocks) stay in FP64.
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
