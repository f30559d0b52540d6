// Tree passes for 32 and more right-hand sides: lane q of a warp owns
// right-hand side q of a chunk of 32 and accumulates all R coefficients of it
// in registers.  Written for sm_103a.
//
// With the basis width R (= rank, 20) on the lanes, as the kernels for up to 8
// right-hand sides have it, 12 of 32 lanes idle and every FMA needs its own
// shared-memory read of the right-hand side.  Here the small dense operand of
// a step (an R x R far-field block F, a transfer matrix, or R-value rows of a
// basis panel) is read from shared memory as 16-byte broadcasts and the
// right-hand side's own values as one 16-byte read per four, so about four of
// five FMA-or-load steps are FMAs; in FP32 each two adjacent FMAs go out as
// one packed FP32x2 FMA.  All are small GEMMs:
//   m2l_w:       s[slot][q][:] = sum_e F_e t[yslot_e][q][:]         (R x R times R)
//   leaf_up_w:   t[slot][q][:] = V^T x[rows][q]                      (R x nrows times nrows)
//   xfer_task_w: t[parent] = sum_c T_c^T t[child_c], s[child_c] += T_c s[parent]
// Shared memory: m2l_w two stages per warp of (one F block, the column slot's
// 32 x R coefficients), cp.async with 16-byte copies; leaf_up_w per warp the
// panel (nrows x R) and the 32 right-hand sides' rows, [q][j] with a row
// stride of 4 mod 8 words (conflict-free 16-byte reads by eight lanes);
// xfer_task_w per CTA the two transfer matrices and the task's local vectors.
#include "hm_kernels.cuh"
#include "hm_async.cuh"

namespace hm {

namespace {

// four consecutive values from 16-byte aligned shared memory
__device__ __forceinline__ void ld4(const float *p, float *v)
{
    const float4 a = *reinterpret_cast<const float4 *>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const double *p, double *v)
{
    const double2 a = *reinterpret_cast<const double2 *>(p);
    const double2 b = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
// acc[i] = fma(f[i], x, acc[i]) for i < 4.  FP32 runs it as two packed
// FP32x2 FMAs (__ffma2_rn, each half rounded as fmaf: the same sums in half
// the FMA instructions).
__device__ __forceinline__ void axpy4(const float *f, float x, float *acc)
{
    const float2 xx = make_float2(x, x);
    const float2 a = __ffma2_rn(make_float2(f[0], f[1]), xx, make_float2(acc[0], acc[1]));
    const float2 b = __ffma2_rn(make_float2(f[2], f[3]), xx, make_float2(acc[2], acc[3]));
    acc[0] = a.x; acc[1] = a.y; acc[2] = b.x; acc[3] = b.y;
}
__device__ __forceinline__ void axpy4(const double *f, double x, double *acc)
{
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] = fma(f[i], x, acc[i]);
}
template <typename A>
__device__ __forceinline__ void st4(A *p, const A *v);
template <>
__device__ __forceinline__ void st4<float>(float *p, const float *v)
{
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void st4<double>(double *p, const double *v)
{
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
}

// 16-byte copies of `bytes` (a multiple of 16) from global to shared memory by the warp
__device__ __forceinline__ void warp_copy16(void *dst, const void *src, int bytes, int lane)
{
    const char *s = static_cast<const char *>(src);
    char *d = static_cast<char *>(dst);
    for (int i = lane * 16; i < bytes; i += 32 * 16) async_copy16(d + i, s + i);
}

// the same by the QL lanes of a group (ql its lane within the group)
__device__ __forceinline__ void group_copy16(void *dst, const void *src, int bytes, int ql, int QL)
{
    const char *s = static_cast<const char *>(src);
    char *d = static_cast<char *>(dst);
    for (int i = ql * 16; i < bytes; i += QL * 16) async_copy16(d + i, s + i);
}

// lanes of group g of QL lanes
__device__ __forceinline__ unsigned group_mask(int g, int QL)
{
    return QL == 32 ? 0xffffffffu : (((1u << QL) - 1u) << (g * QL));
}

}  // namespace

// A warp holds G groups of QL = 32 / G lanes; each group takes one (row
// slot, chunk of QL QPL right-hand sides), lane l of a group right-hand sides
// l + QL p, p < QPL (two per lane halve the shared-memory reads per FMA; four
// groups of 8 serve up to 8 right-hand sides with every lane busy).  F blocks
// are R x R column-major (F[m + R n]) with fstride values between blocks;
// coefficients coef[(slot * k + q) * R + m].  Needs R % 4 == 0 and
// fstride % 4 == 0.  Groups synchronise only among their own lanes.
template <typename A, int R, int QPL, int G>
__global__ void __launch_bounds__(kWideWarps * 32)
    m2l_w(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const A *F, int fstride, const A *t, A *s,
          int k)
{
    extern __shared__ __align__(16) unsigned char wide_smem[];
    constexpr int QL = 32 / G, QW = QL * QPL;                  // lanes and right-hand sides of a group
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int g = lane / QL, ql = lane % QL;
    const unsigned gmask = group_mask(g, QL);
    const int nq = (k + QW - 1) / QW;
    const int64_t w = ((int64_t)blockIdx.x * kWideWarps + wib) * G + g;
    pdl_trigger();
    pdl_wait();                                                // the upward pass's coefficients are ready
    if (w >= (int64_t)nrows * nq) return;
    const hm_m2l_row Rw = rows[w / nq];
    const int q0 = (int)(w % nq) * QW, qc = min(QW, k - q0);
    const int stage_vals = fstride + QW * R;
    A *buf = reinterpret_cast<A *>(wide_smem) +
             ((size_t)wib * G + g) * m2l_w_group_vals(fstride, QW, R, (int)sizeof(A));
    auto fetch = [&](int e, int b) {
        const hm_m2l_ent E = ents[e];
        A *fb = buf + b * stage_vals;
        group_copy16(fb, F + E.foff, R * R * (int)sizeof(A), ql, QL);
        group_copy16(fb + fstride, t + ((int64_t)E.yslot * k + q0) * R, qc * R * (int)sizeof(A), ql, QL);
        async_commit();
    };
    A acc[QPL][R];
#pragma unroll
    for (int p = 0; p < QPL; ++p)
#pragma unroll
        for (int m = 0; m < R; ++m) acc[p][m] = A(0);
    if (Rw.begin < Rw.end) fetch(Rw.begin, 0);
    for (int e = Rw.begin; e < Rw.end; ++e) {
        const int b = (e - Rw.begin) & 1;
        if (e + 1 < Rw.end) {
            fetch(e + 1, b ^ 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            async_wait_all();
        }
        __syncwarp(gmask);
        const A *fb = buf + b * stage_vals;
        const A *tq = fb + fstride + ql * R;                   // this lane's right-hand sides (rows past qc unused)
#pragma unroll
        for (int n = 0; n < R; n += 4) {
            A tv[QPL][4];
#pragma unroll
            for (int p = 0; p < QPL; ++p) ld4(tq + p * QL * R + n, tv[p]);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const A *col = fb + (n + u) * R;
#pragma unroll
                for (int m = 0; m < R; m += 4) {
                    A f[4];
                    ld4(col + m, f);
#pragma unroll
                    for (int p = 0; p < QPL; ++p) axpy4(f, tv[p][u], acc[p] + m);
                }
            }
        }
        __syncwarp(gmask);                                     // stage b is refilled by the next fetch
    }
#pragma unroll
    for (int p = 0; p < QPL; ++p) {
        if (ql + QL * p < qc) {
            A *sp = s + ((int64_t)Rw.slot * k + q0 + ql + QL * p) * R;
#pragma unroll
            for (int m = 0; m < R; m += 4) st4<A>(sp + m, acc[p] + m);
        }
    }
}

// Groups as in m2l_w: each group takes one (explicit basis panel, chunk of
// QL QPL right-hand sides), lane l of a group right-hand sides l + QL p:
// t[slot][q][col0 + m] = sum_j V[j][m] x[row0 + j][q], the panel row-major
// (V[j * R + m], ld == width == R), at most cap rows (a multiple of 8).  With
// one group the panel is staged in shared memory; with several, each group
// reads its panel's rows straight from global memory (16-byte loads all lanes
// of the group share).
template <typename A, int R, int QPL, int G>
__global__ void __launch_bounds__(kWideWarps * 32)
    leaf_up_w(MulArgs<A> ma, const hm_vpanel *vp, int npanels, const A *V, A *t, int cap)
{
    extern __shared__ __align__(16) unsigned char wide_smem[];
    constexpr int QL = 32 / G, QW = QL * QPL;
    constexpr bool kStageV = G == 1;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int g = lane / QL, ql = lane % QL;
    const unsigned gmask = group_mask(g, QL);
    const int k = ma.k, nq = (k + QW - 1) / QW;
    const int64_t w = ((int64_t)blockIdx.x * kWideWarps + wib) * G + g;
    pdl_trigger();
    if (w >= (int64_t)npanels * nq) return;
    const hm_vpanel Pn = vp[w / nq];
    const int q0 = (int)(w % nq) * QW, qc = min(QW, k - q0);
    const int xs_stride = cap + 4;                             // 4 mod 8 words
    A *Xs = reinterpret_cast<A *>(wide_smem) +
            ((size_t)wib * G + g) * ((kStageV ? cap * R : 0) + QW * xs_stride);
    const A *Vr = V + Pn.off;                                  // the panel's rows (global, or staged below)
    const int nr = Pn.nrows;
    if constexpr (kStageV) {
        A *Vs = Xs;
        Xs += cap * R;
        group_copy16(Vs, V + Pn.off, nr * R * (int)sizeof(A), ql, QL);
        Vr = Vs;
    }
    // the right-hand sides: lanes walk rows (coalesced), right-hand side by
    // right-hand side, every copy in flight at once (cp.async); rows up to a
    // multiple of 4 and right-hand sides past the chunk are zero-filled
    const int nr4 = (nr + 3) & ~3;
    constexpr int VW = 16 / sizeof(A);                         // values per 16-byte copy
    if (ma.incx == 1 && Pn.row0 % VW == 0 && ma.ldx % VW == 0 && nr % VW == 0) {
        // rows of every right-hand side start on a 16-byte boundary: 16-byte copies,
        // lane (q, piece) over the QW x nr / VW pieces
        const int per_q = nr / VW;
        for (int i = ql; i < QW * per_q; i += QL) {
            const int q = i / per_q, v = i - q * per_q;
            A *d = Xs + q * xs_stride + v * VW;
            if (q < qc) async_copy16(d, ma.x + Pn.row0 + (int64_t)(q0 + q) * ma.ldx + v * VW);
            else for (int u = 0; u < VW; ++u) d[u] = A(0);
        }
        for (int i = ql; i < QW * (nr4 - nr); i += QL) Xs[(i / (nr4 - nr)) * xs_stride + nr + i % (nr4 - nr)] = A(0);
    } else {
        for (int q = 0; q < QW; ++q) {
            const A *xq = ma.x + Pn.row0 * ma.incx + (int64_t)(q0 + q) * ma.ldx;
            for (int j = ql; j < nr4; j += QL) {
                A *d = Xs + q * xs_stride + j;
                if (q < qc && j < nr) async_copy<sizeof(A)>(d, xq + (int64_t)j * ma.incx);
                else *d = A(0);
            }
        }
    }
    async_commit();
    async_wait_all();
    __syncwarp(gmask);
    A acc[QPL][R];
#pragma unroll
    for (int p = 0; p < QPL; ++p)
#pragma unroll
        for (int m = 0; m < R; ++m) acc[p][m] = A(0);
    const A *xr = Xs + ql * xs_stride;
    for (int j = 0; j < nr4; j += 4) {
        A xv[QPL][4];
#pragma unroll
        for (int p = 0; p < QPL; ++p) ld4(xr + p * QL * xs_stride + j, xv[p]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (j + u >= nr) break;
            const A *row = Vr + (j + u) * R;
#pragma unroll
            for (int m = 0; m < R; m += 4) {
                A v[4];
                ld4(row + m, v);
#pragma unroll
                for (int p = 0; p < QPL; ++p) axpy4(v, xv[p][u], acc[p] + m);
            }
        }
    }
#pragma unroll
    for (int p = 0; p < QPL; ++p) {
        if (ql + QL * p < qc) {
            A *tp = t + ((int64_t)Pn.slot * k + q0 + ql + QL * p) * R + Pn.col0;
#pragma unroll
            for (int m = 0; m < R; m += 4) st4<A>(tp + m, acc[p] + m);
        }
    }
}

// Transfer band tasks (the task-local numbering of xfer_up_task /
// xfer_down_task), one CTA per (task, chunk of 32 right-hand sides), warps
// taking the records of a level, lane q the chunk's right-hand side q.  Local
// coefficient vectors L[local][q][0 .. R) in shared memory, after the two
// transfer matrices (upward: as stored, T_c[m' R + m]; downward: transposed,
// so that both read R contiguous values per step).  Needs R % 4 == 0.
//   upward:   t[parent][m] = sum_c sum_m' T_c[m', m] t[child_c][m']
//   downward: s[child_c][m'] += sum_m T_c[m', m] s[parent][m]
template <typename A, int R, bool UP, int G>
__global__ void __launch_bounds__(kWideTaskThreads)
    xfer_task_w(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *coef, int k,
                int early)
{
    extern __shared__ __align__(16) unsigned char wide_smem[];
    constexpr int QL = 32 / G;                                 // lanes of a group = right-hand sides of the CTA
    A *Ts = reinterpret_cast<A *>(wide_smem);
    A *L = Ts + 2 * R * R;
    constexpr int LV = QL * R;                                 // values of one local vector
    const hm_task tk = tasks[blockIdx.x];
    const int e0 = steps[tk.step0].e0, e1 = steps[tk.step1 - 1].e1, nrec = e1 - e0;
    const int q0 = blockIdx.y * QL, qc = min(QL, k - q0);
    const int lane0 = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // group (warp, g) of QL lanes takes records warp * G + g, + nw * G, ...
    const int g = lane0 / QL, lane = lane0 % QL, gw = warp * G + g, nw = (blockDim.x >> 5) * G;
    if (early) pdl_trigger();
    if (UP) {
        for (int i = threadIdx.x; i < 2 * R * R; i += blockDim.x) async_copy<sizeof(A)>(Ts + i, T + i);
    } else {
        // T_c transposed: Ts[c][m][m'] = T_c[m', m]
        for (int i = threadIdx.x; i < 2 * R * R; i += blockDim.x) {
            const int c = i / (R * R), mm = i % (R * R), m = mm / R, mp = mm % R;
            async_copy<sizeof(A)>(Ts + i, T + c * R * R + mp * R + m);
        }
    }
    pdl_wait();                                                // inputs of the band are ready
    // external inputs: groups take records, a group copies a QL x R block
    for (int rec = gw; rec < nrec; rec += nw) {
        const hm_xfer X = ents[e0 + rec];
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
            group_copy16(L + (int64_t)lc * LV, coef + ((int64_t)slot * k + q0) * R, qc * R * (int)sizeof(A), lane,
                         QL);
        }
    }
    async_wait_all();
    __syncthreads();
    for (int st = tk.step0; st < tk.step1; ++st) {
        const hm_step S = steps[st];
        for (int w = gw; w < S.e1 - S.e0; w += nw) {
            const int e = S.e0 + w;
            const hm_xfer X = ents[e];
            if (UP) {
                const A *c0 = L + (int64_t)(X.pad & 0xffff) * LV + lane * R;
                const A *c1 = L + (int64_t)(X.pad >> 16) * LV + lane * R;
                A acc[R];
#pragma unroll
                for (int m = 0; m < R; ++m) acc[m] = A(0);
#pragma unroll
                for (int mp = 0; mp < R; mp += 4) {
                    A a[4], b[4];
                    ld4(c0 + mp, a);
                    ld4(c1 + mp, b);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
#pragma unroll
                        for (int m = 0; m < R; m += 4) {
                            A t0[4], t1[4];
                            ld4(Ts + (mp + u) * R + m, t0);
                            ld4(Ts + R * R + (mp + u) * R + m, t1);
                            axpy4(t0, a[u], acc + m);
                            axpy4(t1, b[u], acc + m);
                        }
                    }
                }
                A *out = L + (int64_t)(e - e0) * LV + lane * R;
#pragma unroll
                for (int m = 0; m < R; m += 4) st4<A>(out + m, acc + m);
                if (lane < qc) {
                    A *g = coef + ((int64_t)X.slot * k + q0 + lane) * R;
#pragma unroll
                    for (int m = 0; m < R; m += 4) st4<A>(g + m, acc + m);
                }
            } else {
                const A *p = L + (int64_t)X.pad * LV + lane * R;
                A *o0 = L + (int64_t)(2 * (e - e0)) * LV + lane * R;
                A *o1 = o0 + LV;
                A a0[R], a1[R];
#pragma unroll
                for (int m = 0; m < R; m += 4) {
                    ld4(o0 + m, a0 + m);
                    ld4(o1 + m, a1 + m);
                }
#pragma unroll
                for (int m = 0; m < R; m += 4) {
                    A pv[4];
                    ld4(p + m, pv);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
#pragma unroll
                        for (int mq = 0; mq < R; mq += 4) {
                            A t0[4], t1[4];
                            ld4(Ts + (m + u) * R + mq, t0);
                            ld4(Ts + R * R + (m + u) * R + mq, t1);
                            axpy4(t0, pv[u], a0 + mq);
                            axpy4(t1, pv[u], a1 + mq);
                        }
                    }
                }
#pragma unroll
                for (int m = 0; m < R; m += 4) {
                    st4<A>(o0 + m, a0 + m);
                    st4<A>(o1 + m, a1 + m);
                }
                if (lane < qc) {
                    A *g0 = coef + ((int64_t)X.c0 * k + q0 + lane) * R;
                    A *g1 = coef + ((int64_t)X.c1 * k + q0 + lane) * R;
#pragma unroll
                    for (int m = 0; m < R; m += 4) {
                        st4<A>(g0 + m, a0 + m);
                        st4<A>(g1 + m, a1 + m);
                    }
                }
            }
        }
        __syncthreads();
    }
}

#define HM_INST_WIDE(A, QPL, G)                                                                             \
    template __global__ void m2l_w<A, 20, QPL, G>(const hm_m2l_row *, int, const hm_m2l_ent *, const A *, int,  \
                                                  const A *, A *, int);                                         \
    template __global__ void leaf_up_w<A, 20, QPL, G>(MulArgs<A>, const hm_vpanel *, int, const A *, A *, int);
#define HM_INST_XFER(A, G)                                                                                     \
    template __global__ void xfer_task_w<A, 20, true, G>(const hm_task *, const hm_step *, const hm_xfer *,     \
                                                         const A *, A *, int, int);                             \
    template __global__ void xfer_task_w<A, 20, false, G>(const hm_task *, const hm_step *, const hm_xfer *,    \
                                                          const A *, A *, int, int);
HM_INST_WIDE(float, 1, 1) HM_INST_WIDE(float, 2, 1) HM_INST_WIDE(float, 1, 2) HM_INST_WIDE(float, 1, 4)
HM_INST_WIDE(double, 1, 1) HM_INST_WIDE(double, 2, 1) HM_INST_WIDE(double, 1, 2) HM_INST_WIDE(double, 1, 4)
HM_INST_XFER(float, 1) HM_INST_XFER(float, 2) HM_INST_XFER(float, 4)
HM_INST_XFER(double, 1) HM_INST_XFER(double, 2) HM_INST_XFER(double, 4)

}  // namespace hm
