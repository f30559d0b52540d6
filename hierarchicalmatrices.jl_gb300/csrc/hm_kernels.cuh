// CUDA kernels of the KernelMatrix compression and matrix-vector product.
// Written for sm_103a.  All kernels are launched from hm_api.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hm_types.h"

#define HM_RMAX 32

namespace hm {

// The calling thread's error message behind hm_last_error (hm_api.cu).
void set_last_error(const char *fmt, ...);
void clear_last_error();

// Every device allocation of the library goes through these (hm_api.cu), so
// that the test hook hm_debug_fail_alloc can make one of them fail with
// cudaErrorMemoryAllocation without calling CUDA.  stream == nullptr in
// device_malloc_async means the legacy default stream, as in CUDA.
cudaError_t device_malloc(void **p, size_t bytes);
cudaError_t device_malloc_async(void **p, size_t bytes, cudaStream_t stream);
// From the library's own stream-ordered pool, which keeps freed memory for
// reuse instead of returning it to the driver at synchronisations.
cudaError_t device_malloc_pooled(void **p, size_t bytes, cudaStream_t stream);

// ---------------------------------------------------------------- numerics

// Kernels of examples/Kernel.jl:34-37, evaluated in FP64 with every operation
// separately rounded (no contraction), as Julia evaluates them.
__device__ __forceinline__ double kernel_eval(int kid, double x, double y)
{
    double d = __dsub_rn(x, y);
    switch (kid) {
    case 0: return 1.0 / d;
    case 1: return 1.0 / __dmul_rn(d, d);
    case 2: return 1.0 / __dmul_rn(__dmul_rn(d, d), d);
    default: return log(fabs(d));
    }
}

// Chebyshev node m mapped to the box [a, b]  (src/BarycentricMatrix.jl:156-164)
__device__ __forceinline__ double box_node(double a, double b, double cheb)
{
    double ab2 = __dmul_rn(0.5, __dadd_rn(a, b));
    double ba2 = __dmul_rn(0.5, __dsub_rn(b, a));
    return __dadd_rn(ab2, __dmul_rn(ba2, cheb));
}

// Error-free transformations for the compensated FP32 dot products.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    float bp = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

template <typename A>
struct Acc;   // accumulator: plain FMA for FP64, compensated (Dot2) for FP32

template <>
struct Acc<double> {
    double s;
    __device__ __forceinline__ void zero() { s = 0.0; }
    __device__ __forceinline__ void add(double p, double g) { s = fma(p, g, s); }
    __device__ __forceinline__ double value() const { return s; }
    __device__ __forceinline__ double s_hi() const { return s; }
    __device__ __forceinline__ double s_lo() const { return 0.0; }
    __device__ __forceinline__ double merged(double so, double) const { return s + so; }
};

template <>
struct Acc<float> {
    float s, c;
    __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float p, float g)
    {
        float h = __fmul_rn(p, g);
        float l = __fmaf_rn(p, g, -h);      // exact product error
        float t, e;
        two_sum(s, h, t, e);
        s = t;
        c = __fadd_rn(c, __fadd_rn(e, l));
    }
    __device__ __forceinline__ float value() const { return __fadd_rn(s, c); }
    __device__ __forceinline__ float s_hi() const { return s; }
    __device__ __forceinline__ float s_lo() const { return c; }
    // value of this accumulator plus another (so, co) one
    __device__ __forceinline__ float merged(float so, float co) const
    {
        float t, e;
        two_sum(s, so, t, e);
        return __fadd_rn(t, __fadd_rn(e, __fadd_rn(c, co)));
    }
};

template <typename A>
struct PlainAcc {   // plain FMA accumulation (multi-RHS paths)
    A s;
    __device__ __forceinline__ void zero() { s = 0; }
    __device__ __forceinline__ void add(A p, A g) { s = fma(p, g, s); }
    __device__ __forceinline__ A value() const { return s; }
};

struct FillArgs {
    const double *x, *y;     // device copies of the points
    const double *cheb, *lam;
    int r, kernel;
    int swap;                // 1: entries are f(col point, row point) (the transposed matrix)
};

__device__ __forceinline__ double fill_kernel(const FillArgs &fa, double row_pt, double col_pt)
{
    return fa.swap ? kernel_eval(fa.kernel, col_pt, row_pt) : kernel_eval(fa.kernel, row_pt, col_pt);
}

// d/dx of the example kernels f(x, y) = phi(x - y), in FP64.
__device__ __forceinline__ double kernel_dx(int kid, double x, double y)
{
    const double d = __dsub_rn(x, y);
    switch (kid) {
    case 0: return -1.0 / __dmul_rn(d, d);
    case 1: return -2.0 / __dmul_rn(__dmul_rn(d, d), d);
    case 2: return -3.0 / __dmul_rn(__dmul_rn(d, d), __dmul_rn(d, d));
    default: return 1.0 / d;
    }
}

// Derivative of a matrix entry with respect to its row point.  For the
// transposed matrix (swap) the entry is f(col, row) and d/d(row) = -phi'.
__device__ __forceinline__ double fill_kernel_drow(const FillArgs &fa, double row_pt, double col_pt)
{
    return fa.swap ? -kernel_dx(fa.kernel, col_pt, row_pt) : kernel_dx(fa.kernel, row_pt, col_pt);
}

template <typename S>
struct MulArgs {
    const S *x;      // x[(j * incx) + q * ldx]
    S *y;            // y[(i * incy) + q * ldy]
    int64_t incx, ldx, incy, ldy;
    int k;           // right-hand sides
    int accumulate;  // 1: y += H x (the reference's mul!), 0: y = H x
    // when set, the final combination of near and far fields (add_far) writes
    // the result here (ld = the row count, e.g. a caller's page-locked host
    // buffer) instead of back into y
    S *yout = nullptr;
    // when set, leaf_up reads the right-hand sides here (e.g. a caller's
    // page-locked host buffer, same layout as x) and stores them into x for
    // the kernels after it; only when the leaf panels cover every row of x once
    const S *xin = nullptr;
};

// ---------------------------------------------------------------- fill (build)

template <typename S>
__global__ void fill_vpanels(FillArgs fa, const hm_vpanel *vp, const hm_fill_vpanel *vf, int npanels, S *V);

template <typename S>
__global__ void fill_f(FillArgs fa, const hm_fill_f *ff, const hm_m2l_ent *ents, int nblocks, S *F);

template <typename S, bool DROW>
__global__ void fill_segments(FillArgs fa, const hm_seg *segs, const hm_piece *pieces,
                              const hm_fill_seg *sf, int nsegs, S *P);

// ---------------------------------------------------------------- matvec

template <typename S, typename A, int QC>
__global__ void leaf_up(MulArgs<S> ma, const hm_vpanel *vp, int npanels, const S *V, A *t, int r, int cap, int wcap);

// Shared memory of one leaf_up warp: a panel of cap x wcap values of S and two
// x chunks of cap x QC values of A (16-byte multiples: cap is a multiple of 32).
template <typename S, typename A, int QC>
__host__ __device__ constexpr size_t leaf_up_warp_bytes(int cap, int wcap)
{
    return ((size_t)cap * wcap * sizeof(S) + 15) / 16 * 16 + 2 * (size_t)cap * QC * sizeof(A);
}

template <typename A, int QC>
__global__ void xfer_up_task(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *t,
                             int r, int k, int early);
template <typename A, int QC>
__global__ void xfer_down_task(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *s,
                               int r, int k, int early);
template <typename A, int QC>
__global__ void xfer_up_band(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *t,
                             int r, int k);

template <typename S, typename A, int QC>
__global__ void m2l(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const S *F, int fstride,
                    const A *t, A *s, int r, int k);

template <typename S, typename A, int QC>
__global__ void m2l_k(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const S *F, int fstride,
                      const A *t, A *s, int r, int k);
template <typename A, int QC>
__global__ void xfer_down_band(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *s,
                               int r, int k);

template <typename S, typename A, bool FAR, int KB>
__global__ void expand_part(MulArgs<S> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const S *P,
                            const A *s, const A *t, int r, int maxw, S *yfar, int64_t ldf);

template <typename S>
__global__ void add_far(MulArgs<S> ma, int64_t n, const S *yfar, int64_t ldf);

// Far-field rows U s, one thread per row (four segments of at most 64 rows per
// CTA of 256 threads); segments' far columns first and at most 64 of them.
template <typename S, typename A, int KB>
__global__ void far_rows(MulArgs<S> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const S *P,
                         const A *s, const A *t, int r, S *yfar, int64_t ldf);

// Persistent panel streaming (cp.async.bulk into a ring of shared-memory
// stages).  CTA b owns segments [cta_seg[b], cta_seg[b+1]); FAR selects the
// columns [0, nfar) of each panel, otherwise [nfar, width).  Shared memory:
// stream_smem_bytes(nst, gcap, KB, sizeof(A)).
constexpr int kStreamThreads = 256;
constexpr int kChunkBytes = 8192;
constexpr int HM_DEV_WAIT_TIMEOUT = 1;    // *status: a stage copy did not complete in time
// Shared memory of stream_part: the stage ring, its mbarriers (and one that
// nothing arrives on, for the stall hook), ngb (2..4)
// gathered right-hand-side buffers, the column-group partials and the CTA's segment
// and piece records (at most dsegs and dpieces of them).
__host__ __device__ constexpr size_t stream_smem_bytes(int nst, int gcap, int ngb, int kb, int asize, int dsegs,
                                                       int dpieces)
{
    return (size_t)nst * kChunkBytes + (size_t)(nst + 1) * 8 + (size_t)ngb * gcap * kb * asize +
           (size_t)8 * 64 * kb * 2 * asize + (size_t)dsegs * sizeof(hm_seg) + (size_t)dpieces * sizeof(hm_piece);
}
template <typename S, typename A, bool FAR, int KB>
__global__ void stream_part(MulArgs<S> ma, const hm_seg *segs, const int *cta_seg, const hm_piece *pieces,
                            const S *P, const A *s, const A *t, int r, int nst, int gcap, int ngb, int dsegs,
                            S *yfar, int *status, unsigned long long wait_ns, int stall);

// Per-warp rings (hm_ring.cu), FP32 storage, KB = 4 or 8 right-hand sides:
// warp w of the grid owns segments [w * nsegs / W, (w + 1) * nsegs / W) and
// streams their part's columns (FAR: the far-field pieces, else the X
// pieces; each part one contiguous column run) through NS stages of
// ring_stage_floats(KB, PF) floats; segments of at most 64 rows, ld % 4 == 0,
// poff % 4 == 0.  Grid: a whole number of CTAs of kRingWarps warps, shared
// memory ring_smem_bytes(KB, PF, NS).
constexpr int kRingWarps = 2;
constexpr int kRingSegsPerWarp = 24;      // segments per warp (the launch's grid follows from it)
constexpr int kRingCols = 32;              // columns per chunk at most (lane c gathers column c)
// The compiled tiles: panel values per stage (at most) and stages.
struct RingTile { int pf, ns; };
constexpr int kRingTiles = 3;
constexpr RingTile kRingTile[kRingTiles] = {{768, 3}, {512, 4}, {1024, 3}};
__host__ __device__ constexpr int ring_stage_floats(int kb, int pf) { return pf + kRingCols * kb; }
__host__ __device__ constexpr size_t ring_smem_bytes(int kb, int pf, int ns)
{
    return (size_t)kRingWarps * ns * ring_stage_floats(kb, pf) * sizeof(float);
}
template <int KB, bool FAR, int PF, int NS>
__global__ void ring_part(MulArgs<float> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const float *P,
                          const float *s, const float *t, int r, float *yfar, int64_t ldf);

// Tree passes for 32 and more right-hand sides (hm_wide.cu): lane q of a
// warp's group of QL = 32 / G lanes owns right-hand sides q + QL p (p < QPL)
// of a chunk of QL QPL; R (the rank) a multiple of 4.  m2l_w: a group per
// (row slot, chunk), shared memory kWideWarps * G * m2l_w_group_vals(...)
// values; leaf_up_w: a group per (panel, chunk), panels row-major with ld ==
// width == R and at most cap rows (a multiple of 8), shared memory
// kWideWarps * G * ((G == 1 ? cap R : 0) + QL QPL (cap + 4)) values;
// xfer_task_w: one chunk of QL per CTA, groups taking records;
// xfer_task_w: one CTA of kWideTaskThreads per (task, chunk), shared memory
// (2 R^2 + locals * QL R) values.
constexpr int kWideWarps = 4;
constexpr int kWideTaskThreads = 256;
// Values of one m2l_w group's buffer: two stages of (an F block, the chunk's
// qw x r coefficients), then 16 bytes of padding.  Without the padding the
// groups of a warp (2 x 560 floats apart for 8 right-hand sides, rank 20)
// start on the same shared-memory bank, and their simultaneous 16-byte reads
// of different F blocks would conflict.
__host__ __device__ constexpr int m2l_w_group_vals(int fstride, int qw, int r, int esize)
{
    return 2 * (fstride + qw * r) + 16 / esize;
}
template <typename A, int R, int QPL, int G>
__global__ void m2l_w(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const A *F, int fstride, const A *t,
                      A *s, int k);
template <typename A, int R, int QPL, int G>
__global__ void leaf_up_w(MulArgs<A> ma, const hm_vpanel *vp, int npanels, const A *V, A *t, int cap);
template <typename A, int R, bool UP, int G>
__global__ void xfer_task_w(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const A *T, A *coef, int k,
                            int early);

// Double-float panels (hm_df.cu, HM_DF64 storage): panels_to_df turns FP64
// panel values into (h, l) FP32 pairs in place; expand_df multiplies them on
// the FP32 pipes, one warp per row segment (PART 0 near-field columns, 1
// far-field columns, 2 all), right-hand sides q0 .. q0 + KB - 1 of k;
// shared memory kWarpsPerCta * maxw * KB * 8 bytes per CTA.
__global__ void panels_to_df(double *P, int64_t n, int *bad);
// leaf_up_df: one warp per basis panel, shared memory cap pairs per warp;
// m2l_df: one warp per row slot, 256 threads per CTA (8 warps).
__global__ void leaf_up_df(MulArgs<double> ma, const hm_vpanel *vp, int npanels, const float2 *V, double *t, int r,
                           int cap);
__global__ void m2l_df(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const float2 *F, int fstride,
                       const double *t, double *s, int r, int k);
// m2l_df_ring: rank 20, kM2lDfWarps warps per CTA (one per row slot), each with
// a ring of NS blocks of F in shared memory (NS * 3.2 KB per warp).
constexpr int kM2lDfWarps = 4, kM2lDfStages = 3;
template <int NS>
__global__ void m2l_df_ring(const hm_m2l_row *rows, int nrows, const hm_m2l_ent *ents, const float2 *F, const double *t,
                            double *s, int k);
// far_rows_df: far-field rows of right-hand side q0, one thread per row, four
// segments of at most 64 rows per CTA of 256 threads (at most 64 far columns).
__global__ void far_rows_df(MulArgs<double> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces,
                            const float2 *P, const double *s, const double *t, int r, double *yfar, int64_t ldf,
                            int q0);
// xfer_df: one CTA per (band task, right-hand side), shared memory
// (2 HM_RMAX^2 + locals r) pairs.
template <bool UP>
__global__ void xfer_df(const hm_task *tasks, const hm_step *steps, const hm_xfer *ents, const float2 *T,
                        double *coef, int r, int k, int early);
template <int PART, int KB>
__global__ void expand_df(MulArgs<double> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const float2 *P,
                          const double *s, const double *t, int r, int maxw, double *yfar, int64_t ldf, int q0);

// Tensor-core panels for many right-hand sides (FP32 storage): grid
// (ceil(k / 128), segments), 256 threads, expand_tc_smem_bytes(maxw) of shared
// memory; needs segments of <= 64 rows, ld % 4 == 0, poff % 32 == 0.
// Waits on the tensor core give up after wait_ns (HM_DEV_WAIT_TIMEOUT in
// *status); stall != 0 makes each CTA's first wait run out (test hook).
size_t expand_tc_smem_bytes(int maxw);
__global__ void expand_tc(MulArgs<float> ma, const hm_seg *segs, const hm_piece *pieces, const float *P,
                          const float *s, const float *t, int r, int maxw, int *status, unsigned long long wait_ns,
                          int stall);

template <typename S, typename A>
__global__ void expand_k(MulArgs<S> ma, const hm_seg *segs, const hm_piece *pieces, const S *P, const A *s,
                         const A *t, int r, int maxw);

// ---------------------------------------------------------------- block-level (hm_blocks.cu)

template <typename T>
__global__ void gemv_n(const T *A, int64_t m, int64_t n, int64_t lda, const T *x, int64_t incx, T *y, int64_t incy);
template <typename T>
__global__ void gemv_t(const T *A, int64_t m, int64_t n, int64_t lda, const T *x, int64_t incx, T *y, int64_t incy);
template <typename T>
__global__ void lr_project(const T *W, int64_t rows, int64_t ldw, int64_t r, const T *x, int64_t incx, T *t);
template <typename T>
__global__ void lr_expand(const T *W, int64_t rows, int64_t ldw, int64_t r, const T *core, int core_diag,
                          int core_trans, const T *t, T *y, int64_t incy);
template <typename T>
__global__ void bary_factors(int kernel, int r, double a, double b, double c, double d, const double *cheb,
                             const double *lam, const double *x, int64_t nx, const double *y, int64_t ny, T *U, T *F,
                             T *V);

// ---------------------------------------------------------------- direct sums

__global__ void direct_rows(int kid, const double *x, int64_t nx, const double *y, int64_t ny,
                           const double *b, const int64_t *rows, int64_t nrows, double *out);

}  // namespace hm
