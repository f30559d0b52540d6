// Row-segment panels streamed through per-warp shared-memory rings, FP32
// storage, 3 to 8 right-hand sides.  Written for sm_103a.
//
// Each warp owns a contiguous run of row segments and walks their panel
// columns (the near-field X pieces, or the far-field coefficient pieces) as
// one stream of chunks: a chunk is up to kRingCols consecutive columns of one
// segment's column-major panel (at most kRingPanelFloats values, one
// contiguous run in HBM) together with the chunk's right-hand-side entries
// g[c][q].  Chunks go through a ring of kRingStages shared-memory stages with
// cp.async: while chunk j is multiplied, chunks j+1 .. j+kRingStages-1 are in
// flight, across segment boundaries, so a warp keeps several KB of HBM reads
// outstanding without holding them in registers.  The stage size and count
// (the tile: PF panel values x NS stages) are template parameters; the
// autotuner picks among the compiled tiles (kRingTile).  Lane l owns rows 2l and
// 2l+1 of the current segment (8-byte reads of the staged columns) and
// accumulates KB right-hand sides with FMA, folding the partial sums into
// compensated (TwoSum) pairs at most every 64 columns, as the per-segment warp
// kernel does.  Only cp.async groups of the warp's own lanes are waited on
// (cp.async.wait_group, then __syncwarp): no barrier spans warps or kernels.
#include "hm_kernels.cuh"
#include "hm_async.cuh"

namespace hm {

namespace {

template <int KB>
struct RingAcc {     // two rows x KB right-hand sides: FMA partials folded into (hi, lo) pairs
    float part[2][KB], hi[2][KB], lo[2][KB];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int q = 0; q < KB; ++q) part[i][q] = hi[i][q] = lo[i][q] = 0.f;
    }
    __device__ __forceinline__ void fold()
    {
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                hm::fold(hi[i][q], lo[i][q], part[i][q]);
                part[i][q] = 0.f;
            }
    }
};

// cp.async of 4 bytes that bypasses nothing (right-hand-side entries are
// re-read by the other segments of their block column: keep them in L1/L2)
__device__ __forceinline__ void copy4(float *dst, const float *src) { async_copy<4>(dst, src); }

}  // namespace

template <int KB, bool FAR, int PF, int NS>
__global__ void __launch_bounds__(kRingWarps * 32)
    ring_part(MulArgs<float> ma, const hm_seg *segs, int nsegs, const hm_piece *pieces, const float *P,
              const float *s, const float *t, int r, float *yfar, int64_t ldf)
{
    extern __shared__ __align__(16) unsigned char ring_smem[];
    constexpr int kRingStages = NS, kRingPanelFloats = PF;
    constexpr int SF = ring_stage_floats(KB, PF);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if constexpr (FAR) pdl_wait();                             // the downward pass's coefficients are ready
    const int64_t gw = (int64_t)blockIdx.x * kRingWarps + wib;
    const int64_t nw = (int64_t)gridDim.x * kRingWarps;
    const int s0 = (int)(gw * nsegs / nw), s1 = (int)((gw + 1) * nsegs / nw);
    if (s0 >= s1) return;
    float *ring = reinterpret_cast<float *>(ring_smem) + (size_t)wib * kRingStages * SF;
    const int k = ma.k;
    const bool acc_y = FAR ? (yfar == nullptr) : (ma.accumulate != 0);

    auto part_range = [](const hm_seg &G, int &cb, int &ce) {
        cb = FAR ? 0 : G.nfar;
        ce = FAR ? G.nfar : G.width;
    };
    auto chunk_cols = [](int ld) { return min(kRingCols, kRingPanelFloats / max(ld, 4)); };

    // ---- producer: the next chunk to issue (warp-uniform), and each lane's
    // piece cursor for its column (lane c of a chunk gathers column c)
    int pj = s0, pc = 0, pce = 0, pld = 4, pcc = 1, ppiece0 = 0, pnp = 0;
    int64_t ppoff = 0;
    int ppi = -1, ppstart = 0, ppw = 0, ppkind = 0;
    int64_t ppsrc = 0;
    auto pseek = [&](int j) {
        for (; j < s1; ++j) {
            const hm_seg G = segs[j];
            int cb, ce;
            part_range(G, cb, ce);
            if (ce > cb) {
                pc = cb; pce = ce; pld = G.ld; pcc = chunk_cols(G.ld); ppoff = G.poff;
                ppiece0 = G.piece0; pnp = G.npieces;
                ppi = -1; ppstart = 0; ppw = 0;
                break;
            }
        }
        pj = j;
    };
    auto issue = [&](int stage) {
        float *sp = ring + stage * SF;
        float *sg = sp + kRingPanelFloats;
        const int cols = min(pcc, pce - pc);
        // the panel columns: one contiguous run of cols * ld values (16-byte copies)
        const float *src = P + ppoff + (int64_t)pc * pld;
        const int nvec = cols * pld / 4;
        for (int i = lane; i < nvec; i += 32) async_copy16(sp + 4 * i, src + 4 * i);
        // right-hand-side entries of column pc + lane
        if (lane < cols) {
            const int col = pc + lane;
            while (col >= ppstart + ppw && ppi + 1 < pnp) {
                ppstart += ppw;
                ++ppi;
                const hm_piece Q = pieces[ppiece0 + ppi];
                ppw = Q.width; ppkind = Q.kind; ppsrc = Q.src;
            }
            const int off = col - ppstart;
            const float *base;
            int64_t step;
            if (ppkind == HM_PIECE_X) {
                base = ma.x + (ppsrc + off) * ma.incx;
                step = ma.ldx;
            } else {
                base = (ppkind == HM_PIECE_TCOEF ? t : s) + (ppsrc * k) * r + off;
                step = r;
            }
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                if (q < k) copy4(sg + lane * KB + q, base + q * step);
                else sg[lane * KB + q] = 0.f;
            }
        }
        pc += cols;
        if (pc >= pce) pseek(pj + 1);
    };

    // ---- consumer: the chunk being multiplied
    int cj = s0, cc = 0, cce = 0, cld = 4, ccc = 1, cnrows = 0, nfold = 0;
    int64_t crow0 = 0;
    RingAcc<KB> acc;
    acc.zero();
    // rows of a segment whose part has no columns: the product's value there is 0
    auto write_zero = [&](const hm_seg &G) {
        if (FAR && !yfar) return;                               // y += 0
        if (!FAR && ma.accumulate) return;
        for (int q = 0; q < k && q < KB; ++q)
            for (int row = lane; row < G.nrows; row += 32) {
                if (FAR) yfar[(G.row0 + row) + (int64_t)q * ldf] = 0.f;
                else ma.y[(G.row0 + row) * ma.incy + (int64_t)q * ma.ldy] = 0.f;
            }
    };
    auto cseek = [&](int j) {
        for (; j < s1; ++j) {
            const hm_seg G = segs[j];
            int cb, ce;
            part_range(G, cb, ce);
            if (ce > cb) {
                cc = cb; cce = ce; cld = G.ld; ccc = chunk_cols(G.ld); cnrows = G.nrows; crow0 = G.row0;
                break;
            }
            write_zero(G);
        }
        cj = j;
    };
    auto finish = [&]() {
        acc.fold();
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            if (q >= k) break;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int row = 2 * lane + i;
                if (row < cnrows) {
                    const float v = acc.hi[i][q] + acc.lo[i][q];
                    if (FAR && yfar) {
                        yfar[(crow0 + row) + (int64_t)q * ldf] = v;
                    } else {
                        float *yp = ma.y + (crow0 + row) * ma.incy + (int64_t)q * ma.ldy;
                        *yp = acc_y ? *yp + v : v;
                    }
                }
            }
        }
        acc.zero();
        nfold = 0;
    };

    pseek(s0);
    cseek(s0);
    // prologue: kRingStages - 1 chunks in flight (one cp.async group each)
#pragma unroll
    for (int i = 0; i < kRingStages - 1; ++i) {
        if (pj < s1) issue(i);
        async_commit();
    }
    int stage = 0;
    while (cj < s1) {
        asm volatile("cp.async.wait_group %0;" ::"n"(kRingStages - 2) : "memory");
        __syncwarp();                                           // chunk visible; the previous stage is free
        {
            const int ist = stage == 0 ? kRingStages - 1 : stage - 1;
            if (pj < s1) issue(ist);
            async_commit();
        }
        const float *sp = ring + stage * SF;
        const float *sg = sp + kRingPanelFloats;
        const int cols = min(ccc, cce - cc);
        if (nfold + cols > 64) {                                // partial sums of at most 64 columns
            acc.fold();
            nfold = 0;
        }
        nfold += cols;
        if (2 * lane < cld) {
            const float *pr = sp + 2 * lane;
            const float4 *gr = reinterpret_cast<const float4 *>(sg);
            auto column = [&](const float *pc, const float4 *gc) {
                const float2 p = *reinterpret_cast<const float2 *>(pc);
                float g[KB];
#pragma unroll
                for (int v = 0; v < KB / 4; ++v) {
                    const float4 g4 = gc[v];
                    g[4 * v] = g4.x; g[4 * v + 1] = g4.y; g[4 * v + 2] = g4.z; g[4 * v + 3] = g4.w;
                }
#pragma unroll
                for (int q = 0; q < KB; ++q) {
                    acc.part[0][q] = fmaf(p.x, g[q], acc.part[0][q]);
                    acc.part[1][q] = fmaf(p.y, g[q], acc.part[1][q]);
                }
            };
            int u = 0;
            for (; u + 8 <= cols; u += 8) {
#pragma unroll
                for (int v = 0; v < 8; ++v) column(pr + (u + v) * cld, gr + (u + v) * (KB / 4));
            }
            for (; u < cols; ++u) column(pr + u * cld, gr + u * (KB / 4));
        }
        cc += cols;
        if (cc >= cce) {
            finish();
            cseek(cj + 1);
        }
        stage = stage + 1 == kRingStages ? 0 : stage + 1;
    }
    async_wait_all();                                           // empty groups: nothing lands after exit
}

#define HM_INST_RING(KB, PF, NS)                                                                             \
    template __global__ void ring_part<KB, false, PF, NS>(MulArgs<float>, const hm_seg *, int, const hm_piece *, \
                                                          const float *, const float *, const float *, int,     \
                                                          float *, int64_t);                                    \
    template __global__ void ring_part<KB, true, PF, NS>(MulArgs<float>, const hm_seg *, int, const hm_piece *,  \
                                                         const float *, const float *, const float *, int,      \
                                                         float *, int64_t);
HM_INST_RING(4, 768, 3) HM_INST_RING(4, 512, 4) HM_INST_RING(4, 1024, 3)
HM_INST_RING(8, 768, 3) HM_INST_RING(8, 512, 4) HM_INST_RING(8, 1024, 3)

}  // namespace hm
