// Tensor-core (tcgen05) row-segment panels for many right-hand sides, FP32
// storage.  Written for sm_103a.
//
// For one row segment (nrows <= 64 rows, panel P of nrows x width, column-
// major with leading dimension ld) and a chunk of up to 128 right-hand sides,
// a CTA of 256 threads computes
//     Y[row][q] (+)= sum_c P[row][c] G[q][c],
// where G holds the gathered [s ; x pieces] entries of the chunk.  The MMA is
// D = A B with A = G (M = 128 right-hand sides x K) and B = P^T (K x N = 64
// rows), both stored K-major in shared memory, D (128 x 64, FP32) in tensor
// memory.  FP32 accuracy comes from splitting every FP32 value exactly into
// three BF16 pieces, v = v_h + v_m + v_l (round-to-nearest at each step;
// 3 x 8 significant bits cover FP32's 24), and summing the six products
//     G_h P_h + G_h P_m + G_m P_h + G_m P_m + G_h P_l + G_l P_h
// with FP32 accumulation (the dropped terms are below 2^-24 relative).  The
// G_h P_h products accumulate in one tensor-memory block and the five
// correction products in a second, added at the end: the tensor core rounds
// each accumulation relative to the running sum, so the corrections (2^-8 of
// it) must not ride on the large sum.
//
// K runs in chunks of 32 columns through a two-stage pipeline: every thread
// loads its share of chunk c + 1 (right-hand-side pairs and panel pairs) from
// global memory into registers while it splits chunk c into one of two
// operand buffers, and thread 0 issues chunk c's MMAs as soon as the buffer
// is written; a buffer is refilled only after the MMAs that read it (chunk
// c - 2) have completed (tcgen05.commit to that buffer's mbarrier), so the
// split of chunk c overlaps the MMAs of chunk c - 1.
//
// Operand layout (SWIZZLE_NONE, K-major, 16-bit): 8-row x 16-byte core
// matrices; element (row, k) of a 32-column chunk sits at byte
//     (row / 8) * 512 + (k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2,
// so core matrices adjacent in K are 128 bytes apart (leading byte offset)
// and 8-row groups 512 bytes apart (stride byte offset).
#include "hm_kernels.cuh"
#include "hm_async.cuh"

#include <cuda_bf16.h>

namespace hm {

namespace {

constexpr int TC_M = 128;          // right-hand sides per CTA (MMA M)
constexpr int TC_N = 64;           // rows per segment (MMA N)
constexpr int TC_KC = 32;          // columns per K chunk
constexpr int TC_THREADS = 256;
constexpr int TC_GI = TC_M * TC_KC / 2 / TC_THREADS;   // right-hand-side pairs per thread and chunk (8)
constexpr int TC_PI = TC_N * TC_KC / 2 / TC_THREADS;   // panel pairs per thread and chunk (4)

struct TcSmem {
    uint32_t G3[2][3][TC_M * TC_KC / 2];   // two buffers of the BF16 pieces h, m, l of G (K-major core matrices)
    uint32_t P3[2][3][TC_N * TC_KC / 2];   // two buffers of the BF16 pieces of P^T
    uint64_t mma_bar[2];                   // completion of the MMAs that read buffer 0 / 1
    uint64_t never_bar;                    // nothing arrives on it (stall hook)
    uint32_t tmem_base;
};
static_assert(sizeof(TcSmem::G3) >= sizeof(float) * TC_M * 65, "epilogue stage fits the operand buffers");
// followed in shared memory by the segment's column table: for each panel
// column, the source of its first right-hand side and the element step
// between right-hand sides (maxw entries of each)

// 32-bit word of the BF16 pair (row, k), (row, k + 1), k even
__device__ __forceinline__ int kmajor_pair_word(int row, int k)
{
    return (row >> 3) * 128 + (k >> 3) * 32 + (row & 7) * 4 + ((k & 7) >> 1);
}

// (a, b) = h + m + l exactly, each a BF16 pair (round to nearest at every
// step); the pairs are packed as stored: a in the low half.
__device__ __forceinline__ void split3x2(float a, float b, uint32_t &h, uint32_t &m, uint32_t &l)
{
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h2);
    const float ra = a - hf.x, rb = b - hf.y;
    const __nv_bfloat162 m2 = __floats2bfloat162_rn(ra, rb);
    const float2 mf = __bfloat1622float2(m2);
    const __nv_bfloat162 l2 = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
    h = *reinterpret_cast<const uint32_t *>(&h2);
    m = *reinterpret_cast<const uint32_t *>(&m2);
    l = *reinterpret_cast<const uint32_t *>(&l2);
}

// Shared-memory matrix descriptor, SWIZZLE_NONE, descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc(const void *p, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((smem_addr(p) & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor (kind::f16): D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace

size_t expand_tc_smem_bytes(int maxw)
{
    return (sizeof(TcSmem) + 15) / 16 * 16 + (size_t)maxw * (sizeof(const float *) + sizeof(int64_t));
}

__global__ void __launch_bounds__(TC_THREADS, 2)
    expand_tc(MulArgs<float> ma, const hm_seg *segs, const hm_piece *pieces, const float *P, const float *s,
              const float *t, int r, int maxw, int *status, unsigned long long wait_ns, int stall)
{
    extern __shared__ __align__(128) unsigned char tc_smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(tc_smem_raw);
    const float **colbase = reinterpret_cast<const float **>(tc_smem_raw + (sizeof(TcSmem) + 15) / 16 * 16);
    int64_t *colstride = reinterpret_cast<int64_t *>(colbase + maxw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const hm_seg G = segs[blockIdx.y];
    const int q0 = blockIdx.x * TC_M;
    const int qc = min(TC_M, ma.k - q0);
    const int W = G.width;
    const int nch = (W + TC_KC - 1) / TC_KC;

    // tensor memory: two blocks of 64 FP32 columns x 128 lanes (h h products, corrections)
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem_base)),
                     "r"(2 * TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&S.mma_bar[0], 1);
        mbar_init(&S.mma_bar[1], 1);
        mbar_init(&S.never_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    // column table of the whole segment (pieces read once; W <= maxw)
    for (int c = tid; c < W; c += TC_THREADS) {
        const float *base = nullptr;
        int64_t step = 0;
        int pc0 = 0;
        for (int pi = 0; pi < G.npieces; ++pi) {
            const hm_piece Q = pieces[G.piece0 + pi];
            if (c < pc0 + Q.width) {
                const int pcol = c - pc0;
                if (Q.kind == HM_PIECE_X) {
                    base = ma.x + (Q.src + pcol) * ma.incx + (int64_t)q0 * ma.ldx;
                    step = ma.ldx;
                } else {
                    base = (Q.kind == HM_PIECE_TCOEF ? t : s) + ((int64_t)Q.src * ma.k + q0) * r + pcol;
                    step = r;
                }
                break;
            }
            pc0 += Q.width;
        }
        colbase[c] = base;
        colstride[c] = step;
    }
    // 8-row groups of A that hold live right-hand sides; the others stay zero in both buffers
    const int live_groups = (qc + 7) >> 3;
    for (int b = 0; b < 2; ++b)
        for (int p = 0; p < 3; ++p)
            for (int w = live_groups * 128 + tid; w < TC_M * TC_KC / 2; w += TC_THREADS) S.G3[b][p][w] = 0u;
    __syncthreads();

    // This thread's pairs of a chunk.  Pair j of the right-hand sides is
    // (q, columns c, c + 1) with q = qb + 16 j, and pair j of the panel is
    // (row, columns c, c + 1) with row = rb + 16 j: a warp covers 8 right-hand
    // sides (rows) x 4 column pairs, the thread's columns are the same for all
    // j, so that only the q / row offsets change from pair to pair.
    const int gq0 = (warp >> 2) * 8 + (lane >> 2), gc = ((warp & 3) * 4 + (lane & 3)) * 2;
    const int pr0 = (warp >> 2) * 8 + (lane & 7), pcol = ((warp & 3) * 4 + (lane >> 3)) * 2;
    // output words: kmajor_pair_word(q, c) advances by 256 words per 16 rows
    const int gw0 = kmajor_pair_word(gq0, gc), pw0 = kmajor_pair_word(pr0, pcol);
    // global loads of chunk ch into registers (zeros outside the live block)
    auto load = [&](int ch, float2 *gv, float2 *pv) {
        const int c0 = ch * TC_KC, cols = min(TC_KC, W - c0);
        const bool l0 = gc < cols, l1 = gc + 1 < cols;
        const float *b0 = l0 ? colbase[c0 + gc] : nullptr, *b1 = l1 ? colbase[c0 + gc + 1] : nullptr;
        const int64_t s0 = l0 ? colstride[c0 + gc] : 0, s1 = l1 ? colstride[c0 + gc + 1] : 0;
#pragma unroll
        for (int j = 0; j < TC_GI; ++j) {
            const int q = gq0 + 16 * j;
            float2 v = make_float2(0.f, 0.f);
            if (q < qc) {
                if (l0) v.x = b0[q * s0];
                if (l1) v.y = b1[q * s1];
            }
            gv[j] = v;
        }
        const bool m0 = pcol < cols, m1 = pcol + 1 < cols;
        const float *pb = P + G.poff + (int64_t)(c0 + pcol) * G.ld;
#pragma unroll
        for (int j = 0; j < TC_PI; ++j) {
            const int row = pr0 + 16 * j;
            float2 v = make_float2(0.f, 0.f);
            if (row < G.ld) {
                if (m0) v.x = __ldcs(pb + row);
                if (m1) v.y = __ldcs(pb + G.ld + row);
            }
            pv[j] = v;
        }
    };
    // split the registers into operand buffer b
    auto split = [&](int b, const float2 *gv, const float2 *pv) {
#pragma unroll
        for (int j = 0; j < TC_GI; ++j) {
            if (gq0 + 16 * j < live_groups * 8) {
                const int w = gw0 + 256 * j;
                split3x2(gv[j].x, gv[j].y, S.G3[b][0][w], S.G3[b][1][w], S.G3[b][2][w]);
            }
        }
#pragma unroll
        for (int j = 0; j < TC_PI; ++j) {
            const int w = pw0 + 256 * j;
            split3x2(pv[j].x, pv[j].y, S.P3[b][0][w], S.P3[b][1][w], S.P3[b][2][w]);
        }
    };

    const uint32_t idesc = umma_idesc_bf16(TC_M, TC_N);
    bool ok = true;
    bool stall_first = stall != 0;
    int committed = -1;                                         // last chunk whose MMAs were committed
    float2 gv[2][TC_GI], pv[2][TC_PI];
    if (nch > 0) load(0, gv[0], pv[0]);
    // two chunks per trip, so that the register sets are indexed statically
    for (int ch = 0; ch < nch && ok; ch += 2) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int cc = ch + h;
            if (cc >= nch) break;
            if (cc + 1 < nch) load(cc + 1, gv[h ^ 1], pv[h ^ 1]);
            // buffer h was read by the MMAs of chunk cc - 2
            if (cc >= 2 && !mbar_wait_first(&S.mma_bar[h], ((cc - 2) >> 1) & 1, wait_ns, stall_first, &S.never_bar))
                ok = false;
            if (__syncthreads_or(!ok)) {
                ok = false;
                break;
            }
            tc_fence_after();
            split(h, gv[h], pv[h]);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // operands visible to the tensor core
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                // (G piece, P piece) of the six products, the largest first
                constexpr int pa[6] = {0, 0, 1, 1, 0, 2}, pb[6] = {0, 1, 0, 1, 2, 0};
#pragma unroll
                for (int ks = 0; ks < TC_KC / 16; ++ks) {
                    const uint32_t off = ks * 256;              // two core matrices of K per step
#pragma unroll
                    for (int j = 0; j < 6; ++j) {
                        const uint64_t ad = umma_desc(reinterpret_cast<const char *>(S.G3[h][pa[j]]) + off, 128, 512);
                        const uint64_t bd = umma_desc(reinterpret_cast<const char *>(S.P3[h][pb[j]]) + off, 128, 512);
                        const uint32_t dt = j == 0 ? tmem : tmem + TC_N;
                        umma_bf16(dt, ad, bd, idesc, (cc > 0 || ks > 0 || j > 1) ? 1 : 0);
                    }
                }
                umma_commit(&S.mma_bar[h]);
            }
            committed = cc;
        }
    }
    // all MMAs done before reading D (a commit tracks every earlier MMA of the thread)
    if (ok && committed >= 0 &&
        !mbar_wait_first(&S.mma_bar[committed & 1], (committed >> 1) & 1, wait_ns, stall_first, &S.never_bar))
        ok = false;
    if (__syncthreads_or(!ok)) {
        if (tid == 0) {
            atomicExch(status, HM_DEV_WAIT_TIMEOUT);
            if (committed >= 0) mbar_wait(&S.mma_bar[committed & 1], (committed >> 1) & 1, kDrainLimitNs);
        }
    } else if (nch == 0) {                                      // no columns: the rows are zero
        for (int i = tid; i < qc * G.nrows; i += TC_THREADS) {
            const int qq = i / G.nrows, row = i - qq * G.nrows;
            float *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)(q0 + qq) * ma.ldy;
            if (!ma.accumulate) *yp = 0.f;
        }
    } else {
        tc_fence_after();
        // D row q (lane) x column row: this warp's 32 right-hand sides, all 64 rows,
        // staged through shared memory (the operand buffers, no longer read) for
        // row-contiguous stores
        float *Ys = reinterpret_cast<float *>(&S.G3[0][0][0]);  // [q][row], stride 65
        // warp w reads tensor-memory lanes 32 (w % 4) .. + 31, columns 32 (w / 4) .. + 31
        const int q = (warp & 3) * 32 + lane;
        const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll
        for (int c0 = (warp >> 2) * 32; c0 < (warp >> 2) * 32 + 32; c0 += 16) {
            float v[16], w[16];
            tmem_ld16(tmem + lane_off + (uint32_t)c0, v);
            tmem_ld16(tmem + lane_off + (uint32_t)(TC_N + c0), w);
#pragma unroll
            for (int i = 0; i < 16; ++i) Ys[q * 65 + c0 + i] = v[i] + w[i];
        }
        __syncthreads();
        for (int i = tid; i < qc * G.nrows; i += TC_THREADS) {
            const int qq = i / G.nrows, row = i - qq * G.nrows;
            float *yp = ma.y + (G.row0 + row) * ma.incy + (int64_t)(q0 + qq) * ma.ldy;
            const float v = Ys[qq * 65 + row];
            *yp = ma.accumulate ? *yp + v : v;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_N) : "memory");
}

}  // namespace hm
