// C ABI of libhmgpu.so: KernelMatrix build (host planner + GPU compression)
// and the hierarchical matvec.  See include/hmgpu.h for the contract.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <map>
#include <set>
#include <thread>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "hm_kernels.cuh"
#include "hm_plan.h"
#include "hmgpu.h"

using namespace hm;

namespace {

thread_local std::string g_last_error;

void set_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

}  // namespace

namespace hm {
void set_last_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}
void clear_last_error() { g_last_error.clear(); }

namespace {
// hm_debug_fail_alloc: allocations left to succeed before one fails, or -1
std::atomic<int64_t> g_fail_alloc{-1};
bool hook_fails()
{
    int64_t v = g_fail_alloc.load();
    while (v >= 0) {
        if (g_fail_alloc.compare_exchange_weak(v, v - 1)) return v == 0;   // 0 -> -1: this one fails
    }
    return false;
}
}  // namespace

cudaError_t device_malloc(void **p, size_t bytes)
{
    if (hook_fails()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaMalloc(p, bytes);
}
cudaError_t device_malloc_async(void **p, size_t bytes, cudaStream_t stream)
{
    if (hook_fails()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    return cudaMallocAsync(p, bytes, stream);
}

// The stream-ordered pool of the block-algebra calls, one per device.  Its
// release threshold is unbounded: the device's default pool hands freed
// memory back to the driver at every synchronisation, and mapping it again
// costs about 0.2 ms on the next allocation, longer than most of these calls.
cudaError_t device_malloc_pooled(void **p, size_t bytes, cudaStream_t stream)
{
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static cudaMemPool_t pools[kMaxDevices] = {};
    if (hook_fails()) { *p = nullptr; return cudaErrorMemoryAllocation; }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaMallocAsync(p, bytes, stream);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t np;
            e = cudaMemPoolCreate(&np, &props);
            if (e != cudaSuccess) return e;
            uint64_t keep = UINT64_MAX;
            e = cudaMemPoolSetAttribute(np, cudaMemPoolAttrReleaseThreshold, &keep);
            if (e != cudaSuccess) { cudaMemPoolDestroy(np); return e; }
            pools[dev] = np;
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}
}  // namespace hm

namespace {

int cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return HM_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? HM_ERR_ALLOC : HM_ERR_CUDA;
}

#define HM_CK(call)                                             \
    do {                                                        \
        int st_ = cuda_status((call), #call);                   \
        if (st_) return st_;                                    \
    } while (0)

#define HM_TRY(call)                                            \
    do {                                                        \
        int st_ = (call);                                       \
        if (st_) return st_;                                    \
    } while (0)

#define HM_CK_LAUNCH(what)                                      \
    do {                                                        \
        int st_ = cuda_status(cudaGetLastError(), what);        \
        if (st_) return st_;                                    \
    } while (0)

constexpr int kSegRows = 64;
#define HM_NSTAGES 5   // upward pass, far field + downward pass, near-field panels, far-field panels, whole product
constexpr int kWarpCta = 256;   // threads of the band-transfer CTAs

// sin(pi t) in extended precision, rounded once; t is formed in double like
// the reference's (n-2k+1)/2n.
double sinpi_ext(double t)
{
    const long double pi = 3.141592653589793238462643383279502884L;
    return (double)sinl(pi * (long double)t);
}

// chebyshevpoints(T, n) and chebyshevbarycentricweights(T, n), first kind
// (src/BarycentricMatrix.jl:92-136).
void chebyshev_first_kind(int n, std::vector<double> &x, std::vector<double> &w)
{
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const int nd2 = n / 2;
    for (int k = 1; k <= nd2; ++k) x[k - 1] = sinpi_ext(((double)(n - 2 * k) + 1.0) / (double)(2 * n));
    for (int k = 1; k <= nd2; ++k) x[n - k] = -x[k - 1];
    for (int k = 1; k <= nd2 + 1 && k <= n; ++k) w[k - 1] = sinpi_ext(((double)(2 * k) - 1.0) / (double)(2 * n));
    for (int k = 1; k <= nd2; ++k) w[n - k] = w[k - 1];
    for (int k = 2; k <= n; k += 2) w[k - 1] *= -1.0;
}

// Transfer matrices between a box and its two halves, in the box's
// normalised coordinate: T_c[m' * r + m] = L_m(u_m'), u = -1/2 + x_m'/2 for
// the first half and 1/2 + x_m'/2 for the second, L_m the barycentric Lagrange
// basis on the first-kind nodes.
void transfer_matrices(int r, const std::vector<double> &x, const std::vector<double> &w,
                       std::vector<double> &T)
{
    T.assign(2 * r * r, 0.0);
    for (int c = 0; c < 2; ++c) {
        for (int mp = 0; mp < r; ++mp) {
            const long double u = (c == 0 ? -0.5L : 0.5L) + 0.5L * (long double)x[mp];
            int hit = -1;
            for (int m = 0; m < r; ++m)
                if (u == (long double)x[m]) hit = m;
            long double vals[HM_RMAX];
            long double sum = 0.0L;
            for (int m = 0; m < r; ++m) {
                vals[m] = (hit >= 0) ? (m == hit ? 1.0L : 0.0L) : (long double)w[m] / (u - (long double)x[m]);
                sum += vals[m];
            }
            for (int m = 0; m < r; ++m) T[c * r * r + mp * r + m] = (double)(vals[m] / sum);
        }
    }
}

// The options one product runs with (hm_configure's HM_OPT_* values).
struct Sched {
    int overlap, near_kernel, near_stages, tensor_cores, pdl;
    int tile = 0;      // per-warp ring tile (kRingTile index) for 3-8 FP32 right-hand sides
    int wide = 1;      // tree passes on the lane-per-right-hand-side kernels: 0 never, 1 from 32, 2 from 2 RHS
};

// Right-hand-side buckets of the autotuned schedules: 1, 2, 3-4, 5-8, 9-16,
// 17-32, 33-64, 65-128, 129 and more.
constexpr int kSchedBuckets = 9;
inline int sched_bucket(int k)
{
    int b = 0;
    while (b + 1 < kSchedBuckets && (1 << b) < k) ++b;
    return b;
}

// Storage types whose vectors (right-hand sides, results, coefficients) are FP64.
inline bool f64_vectors(int storage) { return storage != HM_F32; }

}  // namespace

struct hm_handle {
    int kernel = 0, storage = HM_F64, r = 0;
    int device = -1;               // the device current when the handle was built
    int swap = 0;                  // 1: this handle holds the transpose of the kernel matrix
    int ninst = 1;                 // instances of a batched (block-diagonal) handle
    hm_fill_seg *d_seg_fill = nullptr;
    int64_t pstore_elems = 0;
    void *d_dP = nullptr;          // row-derivative panels, filled on the first hm_mul_drow
    std::mutex drow_mu;
    int64_t nx = 0, ny = 0;
    // host copies of the build inputs, for the lazily built transpose
    std::vector<double> hx, hy;
    double box[4] = {0, 0, 0, 0};
    int64_t blocksize = 0;
    hm_handle *trans = nullptr;    // H^T, built on the first hm_mul_t
    std::mutex trans_mu;
    PlanStats stats;
    int n_xslots = 0, n_yslots = 0, max_width = 0;
    std::vector<void *> allocs;
    int64_t device_bytes = 0;

    double *d_x = nullptr, *d_y = nullptr, *d_cheb = nullptr, *d_lam = nullptr;
    void *d_T = nullptr;               // transfer matrices in the storage type
    void *d_V = nullptr, *d_F = nullptr, *d_P = nullptr;
    hm_vpanel *d_vp = nullptr;
    int n_vp = 0;
    int vp_cap = 64, vp_wcap = HM_RMAX;   // leaf_up's shared-memory panel: rows (multiple of 32) x columns
    bool vp_covers_x = false;             // the leaf panels' rows partition [0, ny): leaf_up reads every x once
    bool vp_wide = false;                 // every leaf panel row-major with ld == width == 20 (leaf_up_w)
    int wide_tree = 1;                    // lane-per-RHS tree kernels: 0 never, 1 from 32 RHS, 2 from 2 (HM_OPT_WIDE_TREE)
    int ring_tile = 0;                    // per-warp ring tile (HM_OPT_RING_TILE)
    hm_xfer *d_up = nullptr;
    std::vector<int> up_ptr;
    hm_m2l_row *d_m2l_rows = nullptr;
    int n_m2l_rows = 0;
    hm_m2l_ent *d_m2l_ents = nullptr;
    hm_xfer *d_down = nullptr;
    std::vector<int> down_ptr;
    // banded transfers
    hm_xfer *d_up_ents = nullptr, *d_down_ents = nullptr;
    hm_step *d_up_steps = nullptr, *d_down_steps = nullptr;
    hm_task *d_up_tasks = nullptr, *d_down_tasks = nullptr;
    std::vector<int> up_band_ptr, down_band_ptr;
    int band_locals[2] = {0, 0};    // most task-local coefficient vectors of an upward / downward task
    int fstride = 0;
    hm_seg *d_segs = nullptr;
    int n_segs = 0;
    hm_piece *d_pieces = nullptr;
    // persistent panel streaming: CTA b of part p (0 near, 1 far) owns the
    // segments [d_cta_seg[p*(stream_ctas+1) + b], ... + b + 1)
    int *d_cta_seg = nullptr;
    int stream_ctas = 0;            // > 0: every segment's far and near parts are contiguous column runs
    int sms = 1;                    // multiprocessors of the device
    int part_width[2] = {0, 0};     // widest near / far column run of a segment
    int part_segs[2] = {0, 0};      // most segments of one CTA (near / far)
    int part_pieces[2] = {0, 0};    // most piece records of one CTA
    int *d_status = nullptr;        // device-side status word (HM_DEV_*), 0 when clean
    // bounded waits of the streamed and tensor-core panel kernels give up after
    // this long (HM_OPT_WAIT_LIMIT_NS); test_stall (HM_OPT_TEST_STALL) makes the
    // first wait of every CTA run out, to exercise the give-up path
    unsigned long long wait_ns = 2000000000ull;
    int test_stall = 0;
    bool tc_ok = false;             // segments fit the tensor-core panel kernel
    bool tensor_cores = true;       // use it for FP32 products with many right-hand sides

    std::mutex mu;
    // Per caller stream: coefficient scratch (grown stream-ordered), the side
    // stream of the tree passes and the fork/join events.
    struct StreamCtx {
        void *p = nullptr;
        size_t bytes = 0;
        cudaStream_t side = nullptr;
        cudaEvent_t fork = nullptr, join = nullptr;
        cudaEvent_t mid = nullptr;  // a point inside the tree passes where the near field may start
    };
    std::map<void *, StreamCtx> streams;
    void *d_stage = nullptr;
    size_t stage_bytes = 0;
    cudaStream_t host_stream = nullptr;
    // hm_mul_host replays the product's launches as one CUDA graph: captured
    // on the second call with the same right-hand-side count and accumulate
    // flag (the first one runs plainly and sets up scratch and attributes)
    struct HostGraph {
        int nrhs = -1, acc = -1;
        void *stage = nullptr;
        void *out = nullptr;          // page-locked destination written by the last kernel, or none
        const void *in = nullptr;     // page-locked source read by the leaf stage, or none
        bool warm = false;
        cudaGraphExec_t exec = nullptr;
    } host_graph;

    // Optional per-stage timing: CUDA events recorded on the launching stream
    // around each stage of hm_mul.
    unsigned profile_mask = 0;      // bit i: time stage i
    struct StageEvent { int stage; cudaEvent_t a, b; };
    std::vector<StageEvent> events;
    double stage_ms[HM_NSTAGES] = {0};
    int64_t stage_launches[HM_NSTAGES] = {0};
    int launches_per_mul = 0;
    // 0: every stage in order on the caller's stream; 1: tree passes on a side
    // stream from the start of the product, the near field beside them; 2 (the
    // default): the near field starts after the upward pass, whose streaming
    // leaf stage it would otherwise slow; 3: after the far-field (M2L) stage;
    // 4: after the leaf stage only
    int overlap = 2;
    int near_stages = 4;            // ring stages of the near-field streaming kernel
    int near_kernel = 0;            // 0 default (one warp per segment), 1 the same, 2 streamed CTAs
    // programmatic dependent launches along the tree passes: on for FP32
    // storage (measured 0.219 vs 0.231 ms at n = 2^20 with the near field after
    // the leaf stage), off for FP64, whose near field runs beside the tree
    // passes at the FP64 pipe's limit and lost more to CTAs scheduled early
    // (0.759 vs 0.702 ms); set at build from the storage type
    int pdl = -1;
    // hm_autotune's choice per right-hand-side bucket; a product whose bucket
    // has one runs with it instead of the options above
    Sched tuned[kSchedBuckets] = {};
    bool tuned_ok[kSchedBuckets] = {};

    template <typename T>
    int alloc(T **p, size_t count)
    {
        *p = nullptr;
        if (count == 0) return HM_OK;
        void *q = nullptr;
        HM_CK(device_malloc(&q, count * sizeof(T)));
        allocs.push_back(q);
        device_bytes += (int64_t)(count * sizeof(T));
        *p = static_cast<T *>(q);
        return HM_OK;
    }
    template <typename T>
    int upload(T **p, const std::vector<T> &v, cudaStream_t st)
    {
        int e = alloc(p, v.size());
        if (e) return e;
        if (!v.empty()) HM_CK(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        return HM_OK;
    }
};

namespace {

// Streaming kernel geometry: one CTA's chunk loop (wait, use, barrier,
// refill) paces its stream, so three CTAs share an SM, each with a short ring.
// CTAs own about kStreamCtaBytes of panels each rather than persisting for
// the whole product: CTAs that retire hand their SM slots to the tree passes
// running beside them (on the higher-priority side stream).
constexpr int kStreamCtasPerSm = 3;
constexpr double kStreamCtaBytes = 400.0 * 1024;

int check_points(const double *x, int64_t n, const char *name)
{
    for (int64_t i = 0; i < n; ++i) {
        if (std::isnan(x[i])) { set_error("%s[%lld] is NaN", name, (long long)i); return HM_ERR_NAN; }
        if (i > 0 && x[i] > x[i - 1]) {
            set_error("%s is not in non-increasing order at index %lld (KernelMatrix needs descending points)",
                      name, (long long)i);
            return HM_ERR_UNSORTED;
        }
    }
    return HM_OK;
}

// Per-segment part widths and the CTA ranges of the streaming kernels:
// kStreamCtasPerSm CTAs per SM, each owning a run of consecutive segments with about the same
// number of panel bytes (plus a fixed cost per segment).  Streaming needs
// the far-field pieces of every segment before its X pieces.
int prepare_streaming(hm_handle *h, const std::vector<hm_seg> &segs, const std::vector<hm_piece> &pieces,
                      cudaStream_t st)
{
    HM_TRY(h->alloc(&h->d_status, 1));
    HM_CK(cudaMemsetAsync(h->d_status, 0, sizeof(int), st));
    h->stream_ctas = 0;
    if (segs.empty()) return HM_OK;
    h->tc_ok = true;
    for (const hm_seg &g : segs)
        if (g.ld % 4 || g.poff % 32 || g.nrows > 64 || g.ld > 64) h->tc_ok = false;
    for (const hm_seg &g : segs) {
        int nfar = 0;
        bool seen_x = false;
        for (int i = 0; i < g.npieces; ++i) {
            const hm_piece &q = pieces[g.piece0 + i];
            if (q.kind == HM_PIECE_X) { seen_x = true; continue; }
            if (seen_x) return HM_OK;                 // not far-first: keep the per-warp kernels
            nfar += q.width;
        }
        if (nfar != g.nfar || g.ld % 4 || g.poff % 32 || g.nrows > 64) return HM_OK;
        if (&g != &segs[0] && g.piece0 != (&g)[-1].piece0 + (&g)[-1].npieces) return HM_OK;
        h->part_width[0] = std::max(h->part_width[0], g.width - g.nfar);
        h->part_width[1] = std::max(h->part_width[1], g.nfar);
    }
    int dev = 0, sms = 0;
    HM_CK(cudaGetDevice(&dev));
    HM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    h->sms = sms;
    double near_bytes = 0;
    for (const hm_seg &g : segs) near_bytes += (double)(g.width - g.nfar) * g.ld * 4.0;
    const int64_t want = std::max<int64_t>((int64_t)kStreamCtasPerSm * sms, (int64_t)(near_bytes / kStreamCtaBytes));
    const int G = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)segs.size()));
    std::vector<int> split(2 * (size_t)(G + 1));
    std::vector<double> pre(segs.size() + 1);
    for (int part = 0; part < 2; ++part) {
        pre[0] = 0;
        for (size_t j = 0; j < segs.size(); ++j) {
            const hm_seg &g = segs[j];
            const int cols = part == 0 ? g.width - g.nfar : g.nfar;
            pre[j + 1] = pre[j] + (double)cols * g.ld + 512.0;
        }
        int *sp = split.data() + (size_t)part * (G + 1);
        for (int b = 0; b <= G; ++b) {
            const double target = pre.back() * b / G;
            sp[b] = (int)(std::lower_bound(pre.begin(), pre.end(), target) - pre.begin());
            if (b == G) sp[b] = (int)segs.size();
            sp[b] = std::min<int>(sp[b], (int)segs.size());
            if (b > 0) sp[b] = std::max(sp[b], sp[b - 1]);
        }
        sp[0] = 0;
        h->part_segs[part] = h->part_pieces[part] = 0;
        for (int b = 0; b < G; ++b) {
            if (sp[b + 1] <= sp[b]) continue;
            const hm_seg &f = segs[sp[b]], &l = segs[sp[b + 1] - 1];
            h->part_segs[part] = std::max(h->part_segs[part], sp[b + 1] - sp[b]);
            h->part_pieces[part] = std::max(h->part_pieces[part], l.piece0 + l.npieces - f.piece0);
        }
    }
    HM_TRY(h->upload(&h->d_cta_seg, split, st));
    h->stream_ctas = G;
    return HM_OK;
}

// Most task-local coefficient vectors over the tasks of a band table (the
// numbering the planner stores in the records' pad).
int band_locals(const std::vector<hm_task> &tasks, const std::vector<hm_step> &steps,
                const std::vector<hm_xfer> &ents, bool upward)
{
    int most = 0;
    for (const hm_task &tk : tasks) {
        if (tk.step1 <= tk.step0) continue;
        const int e0 = steps[tk.step0].e0, e1 = steps[tk.step1 - 1].e1, nrec = e1 - e0;
        int n = upward ? nrec : 2 * nrec;
        for (int e = e0; e < e1; ++e) {
            if (upward) n = std::max(n, std::max(ents[e].pad & 0xffff, ents[e].pad >> 16) + 1);
            else n = std::max(n, ents[e].pad + 1);
        }
        most = std::max(most, n);
    }
    return most;
}

// leaf_up stages panels of up to vp_cap rows (the largest panel's rows rounded
// up to 32, at most 128: leaves of clustered or random points have up to
// BLOCKSIZE - 1 rows) and vp_wcap columns in shared memory.
void set_vp_caps(hm_handle *h, const std::vector<hm_vpanel> &vps)
{
    int rows = 1, width = 1;
    for (const hm_vpanel &p : vps) {
        rows = std::max(rows, (int)p.nrows);
        width = std::max(width, (int)p.width);
    }
    h->vp_cap = rows <= 128 ? (rows + 31) / 32 * 32 : 64;
    h->vp_wcap = std::min(width, HM_RMAX);
    h->vp_wide = !vps.empty() && rows <= 128;
    for (const hm_vpanel &p : vps)
        if (p.ld != 20 || p.width != 20 || p.off % 4) h->vp_wide = false;
    std::vector<std::pair<int64_t, int64_t>> runs;
    for (const hm_vpanel &p : vps) runs.push_back({p.row0, (int64_t)p.nrows});
    std::sort(runs.begin(), runs.end());
    int64_t cur = 0;
    bool ok = !runs.empty();
    for (const auto &rn : runs) {
        if (rn.first != cur) { ok = false; break; }
        cur += rn.second;
    }
    h->vp_covers_x = ok && cur == h->ny;
}

// HM_DF64 storage: the FP64 panel values become (h, l) FP32 pairs in place;
// a value too large for the pair is an error (HM_ERR_UNSUPPORTED).
int to_double_float(hm_handle *h, double *P, int64_t n, cudaStream_t st)
{
    if (!P || n == 0) return HM_OK;
    int *bad = nullptr;
    HM_TRY(h->alloc(&bad, 1));
    HM_CK(cudaMemsetAsync(bad, 0, sizeof(int), st));
    const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
    panels_to_df<<<grid, 256, 0, st>>>(P, n, bad);
    HM_CK_LAUNCH("panels_to_df");
    int hb = 0;
    HM_CK(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    HM_CK(cudaStreamSynchronize(st));
    if (hb) {
        set_error("a stored value's magnitude reaches 2^127: too large for double-float (HM_DF64) storage; "
                  "use HM_F64");
        return HM_ERR_UNSUPPORTED;
    }
    return HM_OK;
}

template <typename S>
int build_device(hm_handle *h, const Plan &P, const std::vector<double> &cheb, const std::vector<double> &lam,
                 const std::vector<double> &T, const double *x, const double *y, cudaStream_t st)
{
    HM_TRY(h->alloc(&h->d_x, (size_t)h->nx));
    HM_TRY(h->alloc(&h->d_y, (size_t)h->ny));
    HM_CK(cudaMemcpyAsync(h->d_x, x, sizeof(double) * h->nx, cudaMemcpyHostToDevice, st));
    HM_CK(cudaMemcpyAsync(h->d_y, y, sizeof(double) * h->ny, cudaMemcpyHostToDevice, st));
    HM_TRY(h->upload(&h->d_cheb, cheb, st));
    HM_TRY(h->upload(&h->d_lam, lam, st));
    std::vector<S> Ts(T.begin(), T.end());
    S *dT = nullptr;
    HM_TRY(h->upload(&dT, Ts, st));
    h->d_T = dT;

    hm_vpanel *vp = nullptr; hm_fill_vpanel *vpf = nullptr;
    HM_TRY(h->upload(&vp, P.vpanels, st));
    HM_TRY(h->upload(&vpf, P.vpanel_fill, st));
    h->d_vp = vp; h->n_vp = (int)P.vpanels.size();
    set_vp_caps(h, P.vpanels);
    HM_TRY(h->upload(&h->d_up, P.up, st));
    h->up_ptr = P.up_level_ptr;
    HM_TRY(h->upload(&h->d_m2l_rows, P.m2l_rows, st));
    h->n_m2l_rows = (int)P.m2l_rows.size();
    HM_TRY(h->upload(&h->d_m2l_ents, P.m2l_ents, st));
    hm_fill_f *ff = nullptr;
    HM_TRY(h->upload(&ff, P.f_fill, st));
    HM_TRY(h->upload(&h->d_down, P.down, st));
    h->down_ptr = P.down_level_ptr;
    HM_TRY(h->upload(&h->d_up_ents, P.up_ents, st));
    HM_TRY(h->upload(&h->d_up_steps, P.up_steps, st));
    HM_TRY(h->upload(&h->d_up_tasks, P.up_tasks, st));
    HM_TRY(h->upload(&h->d_down_ents, P.down_ents, st));
    HM_TRY(h->upload(&h->d_down_steps, P.down_steps, st));
    HM_TRY(h->upload(&h->d_down_tasks, P.down_tasks, st));
    h->up_band_ptr = P.up_band_ptr;
    h->down_band_ptr = P.down_band_ptr;
    h->band_locals[0] = band_locals(P.up_tasks, P.up_steps, P.up_ents, true);
    h->band_locals[1] = band_locals(P.down_tasks, P.down_steps, P.down_ents, false);
    h->fstride = P.fstride;
    HM_TRY(h->upload(&h->d_segs, P.segs, st));
    h->n_segs = (int)P.segs.size();
    HM_TRY(h->upload(&h->d_pieces, P.pieces, st));
    HM_TRY(prepare_streaming(h, P.segs, P.pieces, st));
    hm_fill_seg *sf = nullptr;
    HM_TRY(h->upload(&sf, P.seg_fill, st));
    h->d_seg_fill = sf;
    h->pstore_elems = P.pstore_elems;

    S *V = nullptr, *F = nullptr, *Pn = nullptr;
    HM_TRY(h->alloc(&V, (size_t)P.vstore_elems));
    HM_TRY(h->alloc(&F, (size_t)P.fstore_elems));
    HM_TRY(h->alloc(&Pn, (size_t)P.pstore_elems));
    if (Pn) HM_CK(cudaMemsetAsync(Pn, 0, sizeof(S) * P.pstore_elems, st));
    h->d_V = V; h->d_F = F; h->d_P = Pn;

    FillArgs fa;
    fa.x = h->d_x; fa.y = h->d_y; fa.cheb = h->d_cheb; fa.lam = h->d_lam; fa.r = h->r; fa.kernel = h->kernel;
    fa.swap = h->swap;
    if (h->n_vp) {
        fill_vpanels<S><<<h->n_vp, 128, 0, st>>>(fa, vp, vpf, h->n_vp, V);
        HM_CK_LAUNCH("fill_vpanels");
    }
    if (!P.f_fill.empty()) {
        fill_f<S><<<(unsigned)P.f_fill.size(), 128, 0, st>>>(fa, ff, h->d_m2l_ents, (int)P.f_fill.size(), F);
        HM_CK_LAUNCH("fill_f");
    }
    if (h->n_segs) {
        fill_segments<S, false><<<h->n_segs, 128, 0, st>>>(fa, h->d_segs, h->d_pieces, sf, h->n_segs, Pn);
        HM_CK_LAUNCH("fill_segments");
    }
    if constexpr (sizeof(S) == 8) {
        if (h->storage == HM_DF64) {
            // panels, column bases and far-field blocks as double-float pairs
            HM_TRY(to_double_float(h, reinterpret_cast<double *>(Pn), P.pstore_elems, st));
            HM_TRY(to_double_float(h, reinterpret_cast<double *>(V), P.vstore_elems, st));
            HM_TRY(to_double_float(h, reinterpret_cast<double *>(F), P.fstore_elems, st));
            HM_TRY(to_double_float(h, reinterpret_cast<double *>(h->d_T), (int64_t)T.size(), st));
        }
    }
    HM_CK(cudaStreamSynchronize(st));
    return HM_OK;
}

// Launches kernel on st.  With pdl the launch is a programmatic dependent of
// the kernel issued just before it on st: it may be scheduled while that
// kernel finishes, and the kernel itself waits (pdl_wait) before it reads the
// predecessor's results.  Only kernels that call pdl_wait get pdl = true.
template <typename... KArgs, typename... Args>
int launch_k(const char *what, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
             bool pdl, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cuda_status(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...), what);
}

struct StageTimer {
    hm_handle *h;
    int stage;
    cudaStream_t st;
    cudaEvent_t a = nullptr, b = nullptr;
    StageTimer(hm_handle *h_, int stage_, cudaStream_t st_) : h(h_), stage(stage_), st(st_)
    {
        if (stage < 0 || !(h->profile_mask & (1u << stage))) return;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, st);
    }
    ~StageTimer()
    {
        if (!a) return;
        cudaEventRecord(b, st);
        h->events.push_back({stage, a, b});
    }
};

// Uploads a flat plan (user-assembled HierarchicalMatrix) with its host-built
// stores; nothing is computed on the device at build time.
template <typename S>
int build_hier_device(hm_handle *h, const Plan &P, const std::vector<double> &vs, const std::vector<double> &fs,
                      const std::vector<double> &ps, cudaStream_t st)
{
    hm_vpanel *vp = nullptr;
    HM_TRY(h->upload(&vp, P.vpanels, st));
    h->d_vp = vp; h->n_vp = (int)P.vpanels.size();
    set_vp_caps(h, P.vpanels);
    HM_TRY(h->upload(&h->d_m2l_rows, P.m2l_rows, st));
    h->n_m2l_rows = (int)P.m2l_rows.size();
    HM_TRY(h->upload(&h->d_m2l_ents, P.m2l_ents, st));
    HM_TRY(h->upload(&h->d_segs, P.segs, st));
    h->n_segs = (int)P.segs.size();
    HM_TRY(h->upload(&h->d_pieces, P.pieces, st));
    HM_TRY(prepare_streaming(h, P.segs, P.pieces, st));
    h->up_band_ptr = P.up_band_ptr;
    h->down_band_ptr = P.down_band_ptr;
    h->fstride = P.fstride;
    h->pstore_elems = P.pstore_elems;
    std::vector<S> v(vs.begin(), vs.end()), f(fs.begin(), fs.end()), p(ps.begin(), ps.end());
    S *dv = nullptr, *df = nullptr, *dp = nullptr;
    HM_TRY(h->upload(&dv, v, st));
    HM_TRY(h->upload(&df, f, st));
    HM_TRY(h->upload(&dp, p, st));
    h->d_V = dv; h->d_F = df; h->d_P = dp;
    HM_CK(cudaStreamSynchronize(st));
    return HM_OK;
}

// Raises the dynamic shared-memory limit of `kernel` when `bytes` needs it.
// The limit set per kernel is remembered, so repeated products (and stream
// capture after a first product) make no further attribute calls.
std::mutex g_smem_mu;
std::map<std::pair<int, const void *>, size_t> g_smem_set;

template <typename K>
int ensure_smem(K kernel, size_t bytes)
{
    if (bytes <= 48 * 1024) return HM_OK;
    if (bytes > 227 * 1024) { set_error("kernel needs %zu bytes of shared memory", bytes); return HM_ERR_UNSUPPORTED; }
    int dev = 0;
    HM_CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_smem_mu);
    size_t &have = g_smem_set[{dev, reinterpret_cast<const void *>(kernel)}];
    if (have >= bytes) return HM_OK;
    HM_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    have = bytes;
    return HM_OK;
}

// The largest shared-memory carveout for a streaming panel kernel (set once
// per device and kernel, like ensure_smem): its blocks then fit by their
// registers, not by the default L1/shared split.
std::set<std::pair<int, const void *>> g_carveout_set;
template <typename K>
int prefer_shared(K kernel)
{
    int dev = 0;
    HM_CK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_smem_mu);
    if (!g_carveout_set.insert({dev, reinterpret_cast<const void *>(kernel)}).second) return HM_OK;
    HM_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared));
    return HM_OK;
}

// Per-call scratch: coefficients t (column slots) then s (row slots).
struct ScratchLayout {
    size_t t_off, s_off, yfar_off, bytes;
};

inline size_t align256(size_t v) { return (v + 255) / 256 * 256; }

template <typename A>
ScratchLayout scratch_layout(const hm_handle *h, int k)
{
    ScratchLayout L;
    L.t_off = 0;
    L.s_off = align256((size_t)h->n_yslots * k * h->r * sizeof(A));
    L.yfar_off = L.s_off + align256((size_t)h->n_xslots * k * h->r * sizeof(A));
    L.bytes = L.yfar_off;
    return L;
}

// Per-call scratch of hm_mul: the coefficients plus, for up to kPartMaxK
// right-hand sides with the side stream, the far-field rows (nx x k, type A).
template <typename A>
size_t stream_scratch_bytes(const hm_handle *h, int k)
{
    const ScratchLayout L = scratch_layout<A>(h, k);
    return L.yfar_off + (k <= 8 ? align256((size_t)h->nx * k * sizeof(A)) : 0);
}

// Scratch, side stream and fork/join events for products issued on stream st.
int stream_ctx(hm_handle *h, cudaStream_t st, size_t bytes, hm_handle::StreamCtx **out)
{
    std::lock_guard<std::mutex> lk(h->mu);
    auto &sc = h->streams[(void *)st];
    if (!sc.side) {
        int least = 0, greatest = 0;
        HM_CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        HM_CK(cudaStreamCreateWithPriority(&sc.side, cudaStreamNonBlocking, greatest));
        HM_CK(cudaEventCreateWithFlags(&sc.fork, cudaEventDisableTiming));
        HM_CK(cudaEventCreateWithFlags(&sc.join, cudaEventDisableTiming));
        HM_CK(cudaEventCreateWithFlags(&sc.mid, cudaEventDisableTiming));
    }
    if (sc.bytes < bytes) {
        if (sc.p) HM_CK(cudaFreeAsync(sc.p, st));
        sc.p = nullptr; sc.bytes = 0;
        HM_CK(device_malloc_async(&sc.p, bytes, st));
        sc.bytes = bytes;
    }
    *out = &sc;
    return HM_OK;
}

// The schedule of the product being issued by this host thread: set by
// run_mul (and hm_autotune) for the duration of one product's launches;
// launches issued outside them read the handle's configured options.
thread_local const Sched *t_sched = nullptr;

inline Sched configured_sched(const hm_handle *h)
{
    return Sched{h->overlap, h->near_kernel, h->near_stages, h->tensor_cores ? 1 : 0,
                 h->pdl >= 0 ? h->pdl : (h->storage != HM_F64 ? 1 : 0), h->ring_tile, h->wide_tree};
}
inline Sched cur_sched(const hm_handle *h) { return t_sched ? *t_sched : configured_sched(h); }
inline Sched sched_for(const hm_handle *h, int k)
{
    if (t_sched) return *t_sched;
    const int b = sched_bucket(k);
    return h->tuned_ok[b] ? h->tuned[b] : configured_sched(h);
}
struct SchedScope {
    const Sched *prev;
    explicit SchedScope(const Sched *s) : prev(t_sched) { t_sched = s; }
    ~SchedScope() { t_sched = prev; }
};

constexpr int kWarpsPerCta = 4;
constexpr int kPartMaxK = 8;    // right-hand sides handled by the streaming panel kernels

inline unsigned warp_ctas(int64_t warps) { return (unsigned)((warps + kWarpsPerCta - 1) / kWarpsPerCta); }

constexpr size_t kTaskSmemMax = 200 * 1024;     // shared memory of a band task kernel
constexpr int kWideMinK = 32;                    // right-hand sides from which the lane-per-RHS tree kernels run

// Index of the last non-empty band of a band pointer array, or -1.
inline int last_band(const std::vector<int> &ptr)
{
    int last = -1;
    for (size_t bd = 0; bd + 1 < ptr.size(); ++bd)
        if (ptr[bd + 1] > ptr[bd]) last = (int)bd;
    return last;
}

// Tree passes on stream st: leaf bases, upward transfers level by level, far
// field, downward transfers level by level.  QC right-hand sides per warp.
template <typename S, typename A, int QC>
int launch_tree_qc(hm_handle *h, const MulArgs<S> &ma, cudaStream_t st, A *t, A *s, bool timing, cudaEvent_t mid,
                   int mid_after, bool *ends_with_kernel)
{
    const int r = h->r, k = ma.k;
    // a launch may be a programmatic dependent while the previous operation on
    // st is one of this product's kernels (no event recorded since)
    // (timing events of the upward or downward stage would sit between the
    // chained kernels; the near-field and whole-product events do not)
    const bool pdl_on = cur_sched(h).pdl && !(h->profile_mask & 0x3u);
    bool chain = false;
    const int64_t nq = (k + QC - 1) / QC;
    const A *T = static_cast<const A *>(h->d_T);
    {
        StageTimer tm(h, timing ? 0 : -1, st);
        bool leaf_done = false;
        if constexpr (std::is_same<S, double>::value && std::is_same<A, double>::value) {
            if (h->n_vp && h->storage == HM_DF64) {
                // column bases as double-float pairs: every right-hand side in one launch
                const size_t smem = (size_t)kWarpsPerCta * h->vp_cap * sizeof(float2);
                HM_TRY(ensure_smem(leaf_up_df, smem));
                leaf_up_df<<<warp_ctas(h->n_vp), 32 * kWarpsPerCta, smem, st>>>(
                    ma, h->d_vp, h->n_vp, static_cast<const float2 *>(h->d_V), t, r, h->vp_cap);
                HM_CK_LAUNCH("leaf_up_df");
                chain = true;
                leaf_done = true;
            }
        }
        if (h->n_vp && !leaf_done) {
            const size_t smem = (size_t)kWarpsPerCta * leaf_up_warp_bytes<S, A, QC>(h->vp_cap, h->vp_wcap);
            HM_TRY(ensure_smem(leaf_up<S, A, QC>, smem));
            leaf_up<S, A, QC><<<warp_ctas(h->n_vp), 32 * kWarpsPerCta, smem, st>>>(
                ma, h->d_vp, h->n_vp, static_cast<const S *>(h->d_V), t, r, h->vp_cap, h->vp_wcap);
            HM_CK_LAUNCH("leaf_up");
            chain = true;
        }
        if (mid && mid_after == 2) { HM_CK(cudaEventRecord(mid, st)); chain = false; }  // leaf bases done
        const size_t usm = (2 * (size_t)HM_RMAX * HM_RMAX + (size_t)h->band_locals[0] * QC * r) * sizeof(A);
        bool up_done = false;
        if constexpr (std::is_same<S, double>::value && std::is_same<A, double>::value) {
            if (h->storage == HM_DF64) {
                // transfers in double-float arithmetic, one right-hand side per CTA
                const size_t xsm = (2 * (size_t)HM_RMAX * HM_RMAX + (size_t)h->band_locals[0] * r) * sizeof(float2);
                HM_TRY(ensure_smem(xfer_df<true>, xsm));
                const int last = last_band(h->up_band_ptr);
                for (size_t bd = 0; bd + 1 < h->up_band_ptr.size(); ++bd) {
                    const int b = h->up_band_ptr[bd], n = h->up_band_ptr[bd + 1] - b;
                    if (!n) continue;
                    HM_TRY(launch_k("xfer_up_df", xfer_df<true>, dim3(n, (unsigned)k), dim3(kWarpCta), xsm, st,
                                    pdl_on && chain, h->d_up_tasks + b, h->d_up_steps, h->d_up_ents,
                                    static_cast<const float2 *>(h->d_T), t, r, k, (int)bd != last ? 1 : 0));
                    chain = true;
                }
                up_done = true;
            }
        }
        if (up_done) {
        } else if (usm <= kTaskSmemMax) {
            const size_t xsm = usm;
            HM_TRY(ensure_smem(xfer_up_task<A, QC>, xsm));
            const int last = last_band(h->up_band_ptr);
            for (size_t bd = 0; bd + 1 < h->up_band_ptr.size(); ++bd) {
                const int b = h->up_band_ptr[bd], n = h->up_band_ptr[bd + 1] - b;
                if (!n) continue;
                // the last band is followed by the M2L grid: no early trigger
                HM_TRY(launch_k("xfer_up_task", xfer_up_task<A, QC>, dim3(n, (unsigned)nq), dim3(kWarpCta), xsm, st,
                                pdl_on && chain, h->d_up_tasks + b, h->d_up_steps, h->d_up_ents, T, t, r, k,
                                (int)bd != last ? 1 : 0));
                chain = true;
            }
        } else {
            const size_t xsm =
                (2 * (size_t)HM_RMAX * HM_RMAX + (size_t)(kWarpCta / 32) * 2 * QC * HM_RMAX) * sizeof(A);
            HM_TRY(ensure_smem(xfer_up_band<A, QC>, xsm));
            for (size_t bd = 0; bd + 1 < h->up_band_ptr.size(); ++bd) {
                const int b = h->up_band_ptr[bd], n = h->up_band_ptr[bd + 1] - b;
                if (!n) continue;
                xfer_up_band<A, QC><<<n, kWarpCta, xsm, st>>>(h->d_up_tasks + b, h->d_up_steps, h->d_up_ents, T, t,
                                                              r, k);
                HM_CK_LAUNCH("xfer_up_band");
                chain = true;
            }
        }
    }
    if (mid && mid_after == 0) { HM_CK(cudaEventRecord(mid, st)); chain = false; }    // upward pass done
    {
        StageTimer tm(h, timing ? 1 : -1, st);
        bool done = false;
        if constexpr (std::is_same<S, double>::value && std::is_same<A, double>::value) {
            if (h->n_m2l_rows && h->storage == HM_DF64) {
                // far-field blocks as double-float pairs: every right-hand side in one launch
                if (r == 20) {
                    const size_t rsm = (size_t)kM2lDfWarps * kM2lDfStages * 400 * sizeof(float2);
                    HM_TRY(launch_k("m2l_df_ring", m2l_df_ring<kM2lDfStages>,
                                    dim3((unsigned)((h->n_m2l_rows + kM2lDfWarps - 1) / kM2lDfWarps)),
                                    dim3(kM2lDfWarps * 32), rsm, st, pdl_on && chain, h->d_m2l_rows, h->n_m2l_rows,
                                    h->d_m2l_ents, static_cast<const float2 *>(h->d_F), t, s, k));
                } else {
                    HM_TRY(launch_k("m2l_df", m2l_df, dim3((unsigned)((h->n_m2l_rows + 7) / 8)), dim3(256), 0, st,
                                    pdl_on && chain, h->d_m2l_rows, h->n_m2l_rows, h->d_m2l_ents,
                                    static_cast<const float2 *>(h->d_F), h->fstride, t, s, r, k));
                }
                chain = true;
                done = true;
            }
        }
        if constexpr (QC > 1) {
            if (!done && h->n_m2l_rows && nq > 1) {
                // many right-hand sides: one CTA per row box, its blocks staged once
                const size_t smem = 8 * (size_t)h->fstride * sizeof(S) +
                                    (size_t)kWarpsPerCta * 2 * QC * HM_RMAX * sizeof(A);
                HM_TRY(ensure_smem(m2l_k<S, A, QC>, smem));
                HM_TRY(launch_k("m2l_k", m2l_k<S, A, QC>, dim3(h->n_m2l_rows), dim3(32 * kWarpsPerCta), smem, st,
                                pdl_on && chain, h->d_m2l_rows, h->n_m2l_rows, h->d_m2l_ents,
                                static_cast<const S *>(h->d_F), h->fstride, t, s, r, k));
                chain = true;
                done = true;
            }
        }
        if (!done && h->n_m2l_rows) {
            const size_t smem =
                (size_t)kWarpsPerCta * (2 * (size_t)h->fstride * sizeof(S) + 2 * (size_t)QC * HM_RMAX * sizeof(A));
            HM_TRY(ensure_smem(m2l<S, A, QC>, smem));
            HM_TRY(launch_k("m2l", m2l<S, A, QC>, dim3(warp_ctas((int64_t)h->n_m2l_rows * nq)),
                            dim3(32 * kWarpsPerCta), smem, st, pdl_on && chain, h->d_m2l_rows, h->n_m2l_rows,
                            h->d_m2l_ents, static_cast<const S *>(h->d_F), h->fstride, t, s, r, k));
            chain = true;
        }
        if (mid && mid_after == 1) { HM_CK(cudaEventRecord(mid, st)); chain = false; }  // far-field stage done
        const size_t dsm = (2 * (size_t)HM_RMAX * HM_RMAX + (size_t)h->band_locals[1] * QC * r) * sizeof(A);
        bool down_done = false;
        if constexpr (std::is_same<S, double>::value && std::is_same<A, double>::value) {
            if (h->storage == HM_DF64) {
                const size_t xsm = (2 * (size_t)HM_RMAX * HM_RMAX + (size_t)h->band_locals[1] * r) * sizeof(float2);
                HM_TRY(ensure_smem(xfer_df<false>, xsm));
                const int last = last_band(h->down_band_ptr);
                for (size_t bd = 0; bd + 1 < h->down_band_ptr.size(); ++bd) {
                    const int b = h->down_band_ptr[bd], n = h->down_band_ptr[bd + 1] - b;
                    if (!n) continue;
                    HM_TRY(launch_k("xfer_down_df", xfer_df<false>, dim3(n, (unsigned)k), dim3(kWarpCta), xsm, st,
                                    pdl_on && chain, h->d_down_tasks + b, h->d_down_steps, h->d_down_ents,
                                    static_cast<const float2 *>(h->d_T), s, r, k, (int)bd != last ? 1 : 0));
                    chain = true;
                }
                down_done = true;
            }
        }
        if (down_done) {
        } else if (dsm <= kTaskSmemMax) {
            const size_t xsm = dsm;
            HM_TRY(ensure_smem(xfer_down_task<A, QC>, xsm));
            const int last = last_band(h->down_band_ptr);
            for (size_t bd = 0; bd + 1 < h->down_band_ptr.size(); ++bd) {
                const int b = h->down_band_ptr[bd], n = h->down_band_ptr[bd + 1] - b;
                if (!n) continue;
                // the last band is followed by the far-field rows' grid: no early trigger
                HM_TRY(launch_k("xfer_down_task", xfer_down_task<A, QC>, dim3(n, (unsigned)nq), dim3(kWarpCta), xsm,
                                st, pdl_on && chain, h->d_down_tasks + b, h->d_down_steps, h->d_down_ents, T, s,
                                r, k, (int)bd != last ? 1 : 0));
                chain = true;
            }
        } else {
            const size_t xsm = (2 * (size_t)HM_RMAX * HM_RMAX + (size_t)(kWarpCta / 32) * QC * HM_RMAX) * sizeof(A);
            HM_TRY(ensure_smem(xfer_down_band<A, QC>, xsm));
            for (size_t bd = 0; bd + 1 < h->down_band_ptr.size(); ++bd) {
                const int b = h->down_band_ptr[bd], n = h->down_band_ptr[bd + 1] - b;
                if (!n) continue;
                xfer_down_band<A, QC><<<n, kWarpCta, xsm, st>>>(h->d_down_tasks + b, h->d_down_steps,
                                                                h->d_down_ents, T, s, r, k);
                HM_CK_LAUNCH("xfer_down_band");
                chain = true;
            }
        }
    }
    *ends_with_kernel = chain && pdl_on;
    return HM_OK;
}

// Whether the tree passes of a product with k right-hand sides can run the
// kernels for 32 and more (lane = right-hand side): rank 20, panels of the
// stored layout, band tasks within shared memory.
// Lane groups per warp of the lane-per-right-hand-side kernels for k right-hand
// sides: four groups of 8 up to 8, two of 16 up to 16, one warp of 32 beyond.
inline int wide_groups(int k) { return k <= 8 ? 4 : k <= 16 ? 2 : 1; }

// Whether the tree passes of a product with k right-hand sides run on those
// kernels under the schedule's `wide` (0 never, 1 from kWideMinK, 2 from 2 on):
// rank 20, panels of the stored layout, band tasks within shared memory.
template <typename S, typename A>
bool wide_tree_ok(const hm_handle *h, const MulArgs<S> &ma, int wide)
{
    const int kmin = wide >= 2 ? 2 : wide == 1 ? kWideMinK : INT32_MAX;
    if (!(std::is_same<S, A>::value && ma.k >= kmin && h->r == 20 && h->vp_wide && !ma.xin && h->fstride % 4 == 0 &&
          h->storage != HM_DF64))
        return false;
    const int G = wide_groups(ma.k);
    const size_t lv = (size_t)(32 / G) * 20 * sizeof(A);
    return (2 * 400 * sizeof(A) + (size_t)h->band_locals[0] * lv) <= kTaskSmemMax &&
           (2 * 400 * sizeof(A) + (size_t)h->band_locals[1] * lv) <= kTaskSmemMax &&
           (size_t)kWideWarps * ((size_t)h->vp_cap * 20 + 32 * ((size_t)h->vp_cap + 4)) * sizeof(A) <= 200 * 1024;
}

// The tree passes for 32 and more right-hand sides: leaf_up_w, xfer_task_w
// bands, m2l_w, the same stage and event structure as launch_tree_qc.
template <typename S, typename A, int G>
int launch_tree_wide(hm_handle *h, const MulArgs<S> &ma, cudaStream_t st, A *t, A *s, bool timing, cudaEvent_t mid,
                     int mid_after, bool *ends_with_kernel)
{
    constexpr int R = 20, QL = 32 / G;
    const int k = ma.k;
    const bool pdl_on = cur_sched(h).pdl && !(h->profile_mask & 0x3u);
    bool chain = false;
    const int64_t nq = (k + QL - 1) / QL;
    const A *T = static_cast<const A *>(h->d_T);
    const MulArgs<A> &mw = reinterpret_cast<const MulArgs<A> &>(ma);
    auto ctas = [](int64_t groups) { return (unsigned)((groups + kWideWarps * G - 1) / (kWideWarps * G)); };
    {
        StageTimer tm(h, timing ? 0 : -1, st);
        if (h->n_vp && G > 1) {
            // up to 16 right-hand sides the leaf stage keeps the chunk-of-8 kernel
            // (measured on the 512-instance batch at 8: faster than four groups of 8
            // reading their panels from global memory)
            const size_t smem = (size_t)kWarpsPerCta * leaf_up_warp_bytes<S, A, 8>(h->vp_cap, h->vp_wcap);
            HM_TRY(ensure_smem(leaf_up<S, A, 8>, smem));
            leaf_up<S, A, 8><<<warp_ctas(h->n_vp), 32 * kWarpsPerCta, smem, st>>>(
                ma, h->d_vp, h->n_vp, static_cast<const S *>(h->d_V), t, h->r, h->vp_cap, h->vp_wcap);
            HM_CK_LAUNCH("leaf_up");
            chain = true;
        } else if (h->n_vp) {
            // one right-hand side per lane (measured at 256: 0.69 ms against 0.94 ms
            // with two, whose larger staging halves the warps per SM)
            auto kern = leaf_up_w<A, R, 1, G>;
            const size_t smem = (size_t)kWideWarps * G *
                                ((G == 1 ? (size_t)h->vp_cap * R : 0) + QL * ((size_t)h->vp_cap + 4)) * sizeof(A);
            HM_TRY(ensure_smem(kern, smem));
            HM_TRY(launch_k("leaf_up_w", kern, dim3(ctas((int64_t)h->n_vp * nq)), dim3(32 * kWideWarps), smem, st,
                            false, mw, h->d_vp, h->n_vp, static_cast<const A *>(h->d_V), t, h->vp_cap));
            chain = true;
        }
        if (mid && mid_after == 2) { HM_CK(cudaEventRecord(mid, st)); chain = false; }  // leaf bases done
        const size_t xsm = (2 * (size_t)R * R + (size_t)h->band_locals[0] * QL * R) * sizeof(A);
        HM_TRY(ensure_smem(xfer_task_w<A, R, true, G>, xsm));
        const int last = last_band(h->up_band_ptr);
        for (size_t bd = 0; bd + 1 < h->up_band_ptr.size(); ++bd) {
            const int b = h->up_band_ptr[bd], n = h->up_band_ptr[bd + 1] - b;
            if (!n) continue;
            HM_TRY(launch_k("xfer_up_w", xfer_task_w<A, R, true, G>, dim3(n, (unsigned)nq), dim3(kWideTaskThreads),
                            xsm, st, pdl_on && chain, h->d_up_tasks + b, h->d_up_steps, h->d_up_ents, T, t, k,
                            (int)bd != last ? 1 : 0));
            chain = true;
        }
    }
    if (mid && mid_after == 0) { HM_CK(cudaEventRecord(mid, st)); chain = false; }    // upward pass done
    {
        StageTimer tm(h, timing ? 1 : -1, st);
        if (h->n_m2l_rows) {
            // two right-hand sides per lane from 64 on (half the shared-memory reads per FMA)
            const int qpl = (G == 1 && k >= 64) ? 2 : 1;
            auto kern = qpl == 2 ? m2l_w<A, R, 2, G> : m2l_w<A, R, 1, G>;
            const size_t smem =
                (size_t)kWideWarps * G * m2l_w_group_vals(h->fstride, QL * qpl, R, (int)sizeof(A)) * sizeof(A);
            HM_TRY(ensure_smem(kern, smem));
            const int64_t groups = (int64_t)h->n_m2l_rows * ((k + QL * qpl - 1) / (QL * qpl));
            HM_TRY(launch_k("m2l_w", kern, dim3(ctas(groups)), dim3(32 * kWideWarps), smem, st, pdl_on && chain,
                            h->d_m2l_rows, h->n_m2l_rows, h->d_m2l_ents, static_cast<const A *>(h->d_F), h->fstride,
                            t, s, k));
            chain = true;
        }
        if (mid && mid_after == 1) { HM_CK(cudaEventRecord(mid, st)); chain = false; }  // far-field stage done
        const size_t xsm = (2 * (size_t)R * R + (size_t)h->band_locals[1] * QL * R) * sizeof(A);
        HM_TRY(ensure_smem(xfer_task_w<A, R, false, G>, xsm));
        const int last = last_band(h->down_band_ptr);
        for (size_t bd = 0; bd + 1 < h->down_band_ptr.size(); ++bd) {
            const int b = h->down_band_ptr[bd], n = h->down_band_ptr[bd + 1] - b;
            if (!n) continue;
            HM_TRY(launch_k("xfer_down_w", xfer_task_w<A, R, false, G>, dim3(n, (unsigned)nq),
                            dim3(kWideTaskThreads), xsm, st, pdl_on && chain, h->d_down_tasks + b, h->d_down_steps,
                            h->d_down_ents, T, s, k, (int)bd != last ? 1 : 0));
            chain = true;
        }
    }
    *ends_with_kernel = chain && pdl_on;
    return HM_OK;
}

template <typename S, typename A>
int launch_tree(hm_handle *h, const MulArgs<S> &ma, cudaStream_t st, A *t, A *s, bool timing,
                cudaEvent_t mid = nullptr, int mid_after = 0, bool *ends_with_kernel = nullptr)
{
    bool ends = false;
    int rc;
    if constexpr (std::is_same<S, A>::value) {
        if (wide_tree_ok<S, A>(h, ma, cur_sched(h).wide)) {
            const int G = wide_groups(ma.k);
            rc = G == 4 ? launch_tree_wide<S, A, 4>(h, ma, st, t, s, timing, mid, mid_after, &ends)
                 : G == 2 ? launch_tree_wide<S, A, 2>(h, ma, st, t, s, timing, mid, mid_after, &ends)
                          : launch_tree_wide<S, A, 1>(h, ma, st, t, s, timing, mid, mid_after, &ends);
            if (ends_with_kernel) *ends_with_kernel = ends;
            return rc;
        }
    }
    rc = ma.k == 1 ? launch_tree_qc<S, A, 1>(h, ma, st, t, s, timing, mid, mid_after, &ends)
                   : launch_tree_qc<S, A, 8>(h, ma, st, t, s, timing, mid, mid_after, &ends);
    if (ends_with_kernel) *ends_with_kernel = ends;
    return rc;
}

// shared memory per streaming CTA: three per SM up to two right-hand sides
// (whose registers allow three), two for FP32 with four or more, one for FP64
constexpr size_t kStreamSmemMax3 = 74 * 1024, kStreamSmemMax2 = 112 * 1024, kStreamSmemMax1 = 200 * 1024;

// Double-float panels (HM_DF64): PART 0 near-field columns, 1 far-field
// columns, 2 every column; right-hand sides q0 .. q0 + KB - 1.
template <int PART, int KB>
int launch_df(hm_handle *h, const MulArgs<double> &ma, const double *s, const double *t, const void *panels,
              double *yfar, cudaStream_t st, bool pdl, int64_t ldf, int q0)
{
    const int maxw = std::max(h->max_width, 1);
    const size_t smem = (size_t)kWarpsPerCta * maxw * KB * sizeof(float2);
    HM_TRY(ensure_smem(expand_df<PART, KB>, smem));
    return launch_k(PART == 1 ? "expand_df_far" : "expand_df", expand_df<PART, KB>, dim3(warp_ctas(h->n_segs)),
                    dim3(32 * kWarpsPerCta), smem, st, PART == 1 && pdl, ma, h->d_segs, h->n_segs, h->d_pieces,
                    static_cast<const float2 *>(panels), s, t, h->r, maxw, yfar, ldf, q0);
}

template <typename S, typename A, bool FAR, int KB>
int launch_part_kb(hm_handle *h, const MulArgs<S> &ma, const A *s, const A *t, const void *panels, S *yfar,
                   cudaStream_t st, bool pdl = false, int64_t ldf = 0)
{
    if constexpr (std::is_same<S, double>::value && std::is_same<A, double>::value) {
        if (h->storage == HM_DF64) {
            if (FAR && h->stream_ctas > 0 && h->part_width[1] <= 64) {
                // far-field rows one thread per row, right-hand side by right-hand side
                for (int q0 = 0; q0 < ma.k; ++q0)
                    HM_TRY(launch_k("far_rows_df", far_rows_df, dim3((unsigned)((h->n_segs + 3) / 4)), dim3(256), 0,
                                    st, pdl && q0 == 0, ma, h->d_segs, h->n_segs, h->d_pieces,
                                    static_cast<const float2 *>(panels), s, t, h->r, yfar, ldf, q0));
                return HM_OK;
            }
            return launch_df<FAR ? 1 : 0, KB>(h, ma, s, t, panels, yfar, st, pdl, ldf, 0);
        }
    }
    if constexpr (FAR && KB >= 4 && std::is_same<S, A>::value) {
        // far-field rows one thread per row for 3-8 right-hand sides (the default
        // and ring schedules; the warp and streamed kernels keep their own
        // far-field form).  Measured: 512-instance batch at 8, 0.55 against
        // 0.76 ms; with 1 right-hand side at n = 2^20 the warp kernel's
        // four-rows-per-lane form stays faster (25 against 41 us)
        const Sched fs = cur_sched(h);
        if (h->stream_ctas > 0 && h->part_width[1] <= 64 && (fs.near_kernel == 0 || fs.near_kernel == 3)) {
            HM_TRY(launch_k("far_rows", far_rows<S, A, KB>, dim3((unsigned)((h->n_segs + 3) / 4)), dim3(256), 0, st,
                            pdl, ma, h->d_segs, h->n_segs, h->d_pieces, static_cast<const S *>(panels), s, t, h->r,
                            yfar, ldf));
            return HM_OK;
        }
    }
    // one warp per segment unless the streamed CTAs are asked for: measured on
    // GB300, the warp kernel reads 64-row grid panels at 6.1 TB/s (90% of the
    // copy peak) and keeps its lead on short segments and more right-hand
    // sides; the streamed form reaches 5.7 TB/s alone and overlaps the tree
    // passes no better
    const Sched sc = cur_sched(h);
    if (!FAR && h->stream_ctas > 0 && sc.near_kernel == 2) {
        const int part = FAR ? 1 : 0;
        const int gcap = std::max(h->part_width[part], 1);
        // the configured stages, right-hand sides gathered three segments
        // ahead; fewer of either until two CTAs fit on an SM
        const size_t smax = KB < 4 ? kStreamSmemMax3 : sizeof(S) == 4 ? kStreamSmemMax2 : kStreamSmemMax1;
        int nst = sc.near_stages, ngb = 4;
        size_t smem = 0;
        for (;;) {
            smem = stream_smem_bytes(nst, gcap, ngb, KB, (int)sizeof(A), h->part_segs[part], h->part_pieces[part]);
            if (smem <= smax) break;
            if (ngb > 2) ngb = 2;
            else if (nst > 2) --nst;
            else break;
        }
        if (smem <= smax) {
            HM_TRY(ensure_smem(stream_part<S, A, FAR, KB>, smem));
            stream_part<S, A, FAR, KB><<<h->stream_ctas, kStreamThreads, smem, st>>>(
                ma, h->d_segs, h->d_cta_seg + (FAR ? h->stream_ctas + 1 : 0), h->d_pieces,
                static_cast<const S *>(panels), s, t, h->r, nst, gcap, ngb, h->part_segs[part], yfar,
                h->d_status, h->wait_ns, h->test_stall);
            HM_CK_LAUNCH(FAR ? "stream_far" : "stream_near");
            return HM_OK;
        }
    }
    if constexpr (sizeof(S) == 4 && sizeof(A) == 4 && KB >= 4) {
        // per-warp rings (the default for 3-8 FP32 right-hand sides): each warp
        // keeps several chunks of its run of segments in flight
        if (h->stream_ctas > 0 && (sc.near_kernel == 0 || sc.near_kernel == 3)) {
            auto kern = sc.tile == 1   ? ring_part<KB, FAR, kRingTile[1].pf, kRingTile[1].ns>
                        : sc.tile == 2 ? ring_part<KB, FAR, kRingTile[2].pf, kRingTile[2].ns>
                                       : ring_part<KB, FAR, kRingTile[0].pf, kRingTile[0].ns>;
            const RingTile tl = kRingTile[sc.tile >= 0 && sc.tile < kRingTiles ? sc.tile : 0];
            const size_t smem = ring_smem_bytes(KB, tl.pf, tl.ns);
            HM_TRY(ensure_smem(kern, smem));
            HM_TRY(prefer_shared(kern));
            // about kRingSegsPerWarp segments per warp: CTAs retire through the
            // product and hand their slots to the tree passes on the side stream;
            // fewer per warp where that would leave SMs short of 16 warps each
            const int64_t spw = std::max<int64_t>(
                1, std::min<int64_t>(kRingSegsPerWarp, h->n_segs / ((int64_t)16 * std::max(h->sms, 1))));
            const int64_t warps = (h->n_segs + spw - 1) / spw;
            const unsigned grid = (unsigned)((warps + kRingWarps - 1) / kRingWarps);
            HM_TRY(launch_k(FAR ? "ring_far" : "ring_near", kern, dim3(grid), dim3(32 * kRingWarps), smem, st,
                            FAR && pdl, ma, h->d_segs, h->n_segs, h->d_pieces, static_cast<const float *>(panels),
                            s, t, h->r, yfar, ldf));
            return HM_OK;
        }
    }
    const int maxw = std::max(h->max_width, 1);
    const size_t smem = (size_t)kWarpsPerCta * maxw * KB * sizeof(A);
    HM_TRY(ensure_smem(expand_part<S, A, FAR, KB>, smem));
    // four or more right-hand sides: blocks limited by registers, not by the
    // default carveout (with one or two, L1 serves the x gathers: keep it)
    if (KB >= 4) HM_TRY(prefer_shared(expand_part<S, A, FAR, KB>));
    // only the far-field form waits for its predecessor (pdl_wait)
    HM_TRY(launch_k(FAR ? "expand_far" : "expand_near", expand_part<S, A, FAR, KB>, dim3(warp_ctas(h->n_segs)),
                    dim3(32 * kWarpsPerCta), smem, st, FAR && pdl, ma, h->d_segs, h->n_segs, h->d_pieces,
                    static_cast<const S *>(panels), s, t, h->r, maxw, yfar, ldf));
    return HM_OK;
}

// Near-field (FAR = false) or far-field (FAR = true) panel columns for k <= 8;
// with yfar the far-field rows go to yfar (leading dimension ldf).
template <typename S, typename A, bool FAR>
int launch_part(hm_handle *h, const MulArgs<S> &ma, const A *s, const A *t, const void *panels, cudaStream_t st,
                S *yfar = nullptr, bool pdl = false, int64_t ldf = 0)
{
    // one right-hand side: FP32 runs the warp kernel's two-column form (FMA
    // with a TwoSum fold every 64 columns issues less than per-element
    // TwoProd/TwoSum); FP64 (plain FMA either way, on the scarce FP64 pipe) and
    // the streamed kernel keep the one-column form
    if (ma.k == 1 && (sizeof(A) == 8 || (!FAR && h->stream_ctas > 0 && cur_sched(h).near_kernel == 2)))
        return launch_part_kb<S, A, FAR, 1>(h, ma, s, t, panels, yfar, st, pdl, ldf);
    if (ma.k <= 2) return launch_part_kb<S, A, FAR, 2>(h, ma, s, t, panels, yfar, st, pdl, ldf);
    if (ma.k <= 4) return launch_part_kb<S, A, FAR, 4>(h, ma, s, t, panels, yfar, st, pdl, ldf);
    return launch_part_kb<S, A, FAR, 8>(h, ma, s, t, panels, yfar, st, pdl, ldf);
}

constexpr int kTensorCoreMinK = 16;   // right-hand sides from which the tensor-core panels run

template <typename S, typename A>
int launch_expand_k(hm_handle *h, const MulArgs<S> &ma, const A *s, const A *t, const void *panels, cudaStream_t st)
{
    if constexpr (std::is_same<S, double>::value && std::is_same<A, double>::value) {
        if (h->storage == HM_DF64) {
            for (int q0 = 0; q0 < ma.k; q0 += 8)
                HM_TRY((launch_df<2, 8>(h, ma, s, t, panels, nullptr, st, false, 0, q0)));
            return HM_OK;
        }
    }
    if constexpr (sizeof(S) == 4 && sizeof(A) == 4) {
        if (cur_sched(h).tensor_cores && h->tc_ok && ma.k >= kTensorCoreMinK) {
            const int maxw = std::max(h->max_width, 1);
            const size_t smem = expand_tc_smem_bytes(maxw);
            HM_TRY(ensure_smem(expand_tc, smem));
            // right-hand-side chunks of a segment run next to each other (its panel is re-read from L2)
            const dim3 grid((unsigned)((ma.k + 127) / 128), (unsigned)h->n_segs);
            expand_tc<<<grid, 256, smem, st>>>(ma, h->d_segs, h->d_pieces, static_cast<const float *>(panels), s, t,
                                               h->r, maxw, h->d_status, h->wait_ns, h->test_stall);
            HM_CK_LAUNCH("expand_tc");
            return HM_OK;
        }
    }
    const int maxw = std::max(h->max_width, 1);
    const int qc = sizeof(A) == 8 ? 16 : 32;
    const size_t smem = ((size_t)64 * maxw * sizeof(S) + 31) / 32 * 32 + (size_t)maxw * qc * sizeof(A);
    HM_TRY(ensure_smem(expand_k<S, A>, smem));
    expand_k<S, A><<<h->n_segs, 128, smem, st>>>(ma, h->d_segs, h->d_pieces, static_cast<const S *>(panels), s,
                                                  t, h->r, maxw);
    HM_CK_LAUNCH("expand_k");
    return HM_OK;
}

// One product.  With a side stream the tree passes and the far-field rows
// (U s, into the scratch vector yfar) run there, concurrently with the
// near-field panels on the caller's stream; yfar is added to y after the join.
// side == st runs everything in order on st.
template <typename S, typename A>
int launch_pipeline(hm_handle *h, const MulArgs<S> &ma, cudaStream_t st, cudaStream_t side, cudaEvent_t fork,
                    cudaEvent_t join, void *scratch, bool timing, const void *panels = nullptr,
                    cudaEvent_t mid = nullptr)
{
    if (!panels) panels = h->d_P;
    const int k = ma.k;
    const ScratchLayout L = scratch_layout<A>(h, k);
    A *t = reinterpret_cast<A *>(static_cast<char *>(scratch) + L.t_off);
    A *s = reinterpret_cast<A *>(static_cast<char *>(scratch) + L.s_off);
    const bool split = side != st;
    const bool tree = h->n_vp || h->n_m2l_rows;
    bool tree_chain = false;         // the tree passes ended with a kernel: the next launch may be dependent
    if (tree) {
        if (split) {
            HM_CK(cudaEventRecord(fork, st));
            HM_CK(cudaStreamWaitEvent(side, fork, 0));
        }
        HM_TRY((launch_tree<S, A>(h, ma, split ? side : st, t, s, timing, split ? mid : nullptr,
                                  cur_sched(h).overlap == 3 ? 1 : cur_sched(h).overlap == 4 ? 2 : 0, &tree_chain)));
        if (split && (k > kPartMaxK || !h->n_segs)) HM_CK(cudaEventRecord(join, side));
    }
    if (!h->n_segs) {
        if (tree && split) HM_CK(cudaStreamWaitEvent(st, join, 0));
        return HM_OK;
    }
    if (k <= kPartMaxK) {
        if (tree && split) {
            // far-field rows on the side stream, into yfar (nx x k, leading dimension nx)
            S *yfar = reinterpret_cast<S *>(static_cast<char *>(scratch) + L.yfar_off);
            {
                StageTimer tm(h, timing ? 3 : -1, side);
                HM_TRY((launch_part<S, A, true>(h, ma, s, t, panels, side, yfar,
                                                tree_chain && !(h->profile_mask & 0x8u), h->nx)));
            }
            HM_CK(cudaEventRecord(join, side));
            if (mid) HM_CK(cudaStreamWaitEvent(st, mid, 0));
            {
                StageTimer tm(h, timing ? 2 : -1, st);
                HM_TRY((launch_part<S, A, false>(h, ma, s, t, panels, st)));
            }
            HM_CK(cudaStreamWaitEvent(st, join, 0));
            const int64_t nk = h->nx * (int64_t)k;
            add_far<S><<<(unsigned)((nk + 255) / 256), 256, 0, st>>>(ma, h->nx, yfar, h->nx);
            HM_CK_LAUNCH("add_far");
            return HM_OK;
        }
        {
            StageTimer tm(h, timing ? 2 : -1, st);
            HM_TRY((launch_part<S, A, false>(h, ma, s, t, panels, st)));
        }
        if (tree) {
            // after the near field on the same stream
            StageTimer tm(h, timing ? 3 : -1, st);
            HM_TRY((launch_part<S, A, true>(h, ma, s, t, panels, st, nullptr,
                                            cur_sched(h).pdl && !(h->profile_mask & 0xcu))));
        }
        return HM_OK;
    }
    if (tree && split) HM_CK(cudaStreamWaitEvent(st, join, 0));
    StageTimer tm(h, timing ? 2 : -1, st);
    return launch_expand_k<S, A>(h, ma, s, t, panels, st);
}

template <typename S, typename A>
int run_mul(hm_handle *h, MulArgs<S> ma, cudaStream_t st, const void *panels = nullptr)
{
    if (ma.k <= 0) return HM_OK;
    const Sched sched = sched_for(h, ma.k);
    SchedScope scope(&sched);
    hm_handle::StreamCtx *sc = nullptr;
    HM_TRY(stream_ctx(h, st, stream_scratch_bytes<A>(h, ma.k), &sc));
    StageTimer whole(h, 4, st);
    return launch_pipeline<S, A>(h, ma, st, sched.overlap ? sc->side : st, sc->fork, sc->join, sc->p, true, panels,
                                 sched.overlap >= 2 ? sc->mid : nullptr);
}

// Row-derivative panels (same layout as the panels), filled once.
template <typename S>
int ensure_drow(hm_handle *h, cudaStream_t st)
{
    std::lock_guard<std::mutex> lk(h->drow_mu);
    if (h->d_dP) return HM_OK;
    S *dP = nullptr;
    HM_TRY(h->alloc(&dP, (size_t)h->pstore_elems));
    if (!dP) return HM_OK;
    HM_CK(cudaMemsetAsync(dP, 0, sizeof(S) * h->pstore_elems, st));
    FillArgs fa;
    fa.x = h->d_x; fa.y = h->d_y; fa.cheb = h->d_cheb; fa.lam = h->d_lam; fa.r = h->r; fa.kernel = h->kernel;
    fa.swap = h->swap;
    if (h->n_segs) {
        fill_segments<S, true><<<h->n_segs, 128, 0, st>>>(fa, h->d_segs, h->d_pieces, h->d_seg_fill, h->n_segs, dP);
        HM_CK_LAUNCH("fill_segments<drow>");
    }
    if constexpr (sizeof(S) == 8) {
        if (h->storage == HM_DF64) HM_TRY(to_double_float(h, reinterpret_cast<double *>(dP), h->pstore_elems, st));
    }
    // complete before the panels are published: a later product may run on another stream
    HM_CK(cudaStreamSynchronize(st));
    h->d_dP = dP;
    return HM_OK;
}

int dispatch_mul(hm_handle *h, const void *x, int64_t incx, int64_t ldx, void *y, int64_t incy, int64_t ldy,
                 int k, int accumulate, cudaStream_t st, void *yout = nullptr, const void *xin = nullptr)
{
    if (f64_vectors(h->storage)) {
        MulArgs<double> ma{static_cast<const double *>(x), static_cast<double *>(y), incx, ldx, incy, ldy, k, accumulate};
        ma.yout = static_cast<double *>(yout);
        ma.xin = static_cast<const double *>(xin);
        return run_mul<double, double>(h, ma, st);
    }
    MulArgs<float> ma{static_cast<const float *>(x), static_cast<float *>(y), incx, ldx, incy, ldy, k, accumulate};
    ma.yout = static_cast<float *>(yout);
    ma.xin = static_cast<const float *>(xin);
    return run_mul<float, float>(h, ma, st);
}

// True when leaf_up can bring the right-hand sides in: its panels cover every
// row of x once, and every later reader of x (the near field) starts after it.
bool leaf_reads_input(const hm_handle *h, int k)
{
    return h->vp_covers_x && h->n_vp > 0 && sched_for(h, k).overlap != 1;
}

// Device-accessible address of a page-locked host buffer, or nullptr.
void *pinned_device_ptr(const void *p)
{
    cudaPointerAttributes pa{};
    void *d = nullptr;
    if (cudaPointerGetAttributes(&pa, p) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
        d = pa.devicePointer;
    cudaGetLastError();           // an unregistered pointer is not an error here
    return d;
}

// True when a product with k right-hand sides ends with add_far (tree passes
// on the side stream, k <= kPartMaxK, row segments present), which can then
// write the result to MulArgs::yout.
bool ends_with_add_far(const hm_handle *h, int k)
{
    return (h->n_vp || h->n_m2l_rows) && h->n_segs > 0 && k <= kPartMaxK && sched_for(h, k).overlap != 0;
}

// ---- autotuned schedules ----------------------------------------------------
//
// The fastest options for a product differ with the number of right-hand
// sides and with the tree: when the near field should start beside the tree
// passes (it shares HBM with the leaf stage and the far field), whether the
// warp-per-segment or the streamed near-field kernel wins (segment lengths),
// its ring depth, and whether FP32 panels with many right-hand sides run
// faster on the tensor cores or on the FP32 pipes.  hm_autotune times every
// candidate on the caller's stream and keeps the fastest for the call's
// right-hand-side bucket.

void drop_host_graph(hm_handle *h)
{
    if (h->host_graph.exec) {
        cudaStreamSynchronize(h->host_stream);
        cudaGraphExecDestroy(h->host_graph.exec);
    }
    h->host_graph = hm_handle::HostGraph();
}

std::vector<Sched> sched_candidates(const hm_handle *h, int k, bool fp32)
{
    const Sched base = configured_sched(h);
    const bool tree = h->n_vp || h->n_m2l_rows;
    std::vector<int> overlaps = !tree ? std::vector<int>{base.overlap}
                                      : k <= kPartMaxK ? std::vector<int>{0, 1, 2, 3, 4} : std::vector<int>{0, 1};
    // near-field kernels: the default (per-warp rings for 3-8 FP32 right-hand
    // sides, else one warp per segment), the warp kernel where that differs,
    // and the streamed CTAs
    std::vector<int> kernels{base.near_kernel};
    if (k <= kPartMaxK && h->stream_ctas > 0 && h->n_segs && h->storage != HM_DF64) {
        kernels = {0, 2};
        if (fp32 && k >= 3) kernels = {0, 1, 2};
    }
    std::vector<int> tcs = (fp32 && h->tc_ok && k >= kTensorCoreMinK) ? std::vector<int>{1, 0}
                                                                       : std::vector<int>{base.tensor_cores};
    // ring tiles where the per-warp rings run (3-8 FP32 right-hand sides), and
    // the lane-per-right-hand-side tree kernels on and off (32+, unless the
    // option turned them off)
    const bool ring = fp32 && k >= 3 && k <= kPartMaxK && h->stream_ctas > 0 && h->n_segs;
    // (from 32 right-hand sides: on or off; from 2 to 31: the chunk-of-8 kernels or the grouped ones)
    std::vector<int> wides{base.wide};
    if (tree && h->wide_tree && k >= kWideMinK) wides = {1, 0};
    else if (tree && h->wide_tree && k >= 2) wides = {1, 2};
    std::vector<Sched> c{base};       // the configured schedule first, timed for comparison
    auto add = [&c](Sched s) {
        for (const Sched &o : c)
            if (o.overlap == s.overlap && o.near_kernel == s.near_kernel && o.near_stages == s.near_stages &&
                o.tensor_cores == s.tensor_cores && o.pdl == s.pdl && o.tile == s.tile && o.wide == s.wide)
                return;
        c.push_back(s);
    };
    const std::vector<int> pdls = tree ? std::vector<int>{1, 0} : std::vector<int>{base.pdl};
    for (int ov : overlaps)
        for (int nk : kernels)
            for (int tc : tcs)
                for (int pd : pdls)
                    for (int wd : wides) {
                        if (nk == 2) {
                            for (int ns : {3, 4, 6}) add(Sched{ov, nk, ns, tc, pd, 0, wd});
                        } else if (ring && (nk == 0 || nk == 3)) {
                            for (int tl = 0; tl < kRingTiles; ++tl) add(Sched{ov, nk, base.near_stages, tc, pd, tl, wd});
                        } else {
                            add(Sched{ov, nk, base.near_stages, tc, pd, 0, wd});
                        }
                    }
    return c;
}

template <typename S>
int autotune(hm_handle *h, int k, int reps, cudaStream_t st, int32_t *choice, double *ms_out)
{
    const std::vector<Sched> cand = sched_candidates(h, k, sizeof(S) == 4);
    const size_t nv = (size_t)h->ny * k, nu = (size_t)h->nx * k;
    S *v = nullptr, *u = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = cuda_status(device_malloc_async((void **)&v, std::max<size_t>(nv, 1) * sizeof(S), st), "cudaMallocAsync");
    if (!rc) rc = cuda_status(device_malloc_async((void **)&u, std::max<size_t>(nu, 1) * sizeof(S), st), "cudaMallocAsync");
    // finite, normal inputs (0x3f bytes); the kernels' time does not depend on the values
    if (!rc) rc = cuda_status(cudaMemsetAsync(v, 0x3f, nv * sizeof(S), st), "cudaMemsetAsync");
    if (!rc) rc = cuda_status(cudaEventCreate(&e0), "cudaEventCreate");
    if (!rc) rc = cuda_status(cudaEventCreate(&e1), "cudaEventCreate");
    std::vector<double> best(cand.size(), 1e300);
    const MulArgs<S> ma{v, u, 1, h->ny, 1, h->nx, k, 0};
    // two rounds over the candidates, the better time of each kept, so that a
    // clock ramp at the start favours none of them
    for (int round = 0; round < 2 && !rc; ++round) {
        for (size_t c = 0; c < cand.size() && !rc; ++c) {
            SchedScope scope(&cand[c]);
            for (int w = 0; w < 2 && !rc; ++w) rc = run_mul<S, S>(h, ma, st);
            if (!rc) rc = cuda_status(cudaEventRecord(e0, st), "cudaEventRecord");
            for (int i = 0; i < reps && !rc; ++i) rc = run_mul<S, S>(h, ma, st);
            if (!rc) rc = cuda_status(cudaEventRecord(e1, st), "cudaEventRecord");
            if (!rc) rc = cuda_status(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float t = 0.f;
            if (!rc) rc = cuda_status(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime");
            if (!rc) best[c] = std::min(best[c], (double)t / reps);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (v) cudaFreeAsync(v, st);
    if (u) cudaFreeAsync(u, st);
    const int rs = cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (rc) return rc;
    if (rs) return rs;
    size_t bi = 0;
    for (size_t c = 1; c < cand.size(); ++c)
        if (best[c] < best[bi]) bi = c;
    const int b = sched_bucket(k);
    {
        std::lock_guard<std::mutex> lk(h->mu);
        h->tuned[b] = cand[bi];
        h->tuned_ok[b] = true;
    }
    drop_host_graph(h);             // it was captured with the previous schedule
    if (choice) {
        choice[0] = cand[bi].overlap;
        choice[1] = cand[bi].near_kernel;
        choice[2] = cand[bi].near_stages;
        choice[3] = cand[bi].tensor_cores;
        choice[4] = cand[bi].pdl;
    }
    if (ms_out) {
        ms_out[0] = best[bi];
        ms_out[1] = best[0];
    }
    return HM_OK;
}

// ---- allocation-free single right-hand-side product ------------------------
//
// Some callers cannot let the library allocate device memory during a
// product: processes whose device memory is entirely reserved up front by
// another allocator (a framework memory pool that takes most of HBM at
// start-up), and loops that must not call cudaMalloc/cudaFree after
// initialisation because those calls can synchronise the device and take an
// unbounded time.  hm_mul_noalloc serves them: its coefficient scratch is this
// file-scope device array, sized at compile time and held by every GPU that
// loads the library until the process exits.  All calls share it.
#define HM_NOALLOC_SCRATCH_BYTES (16u << 20)
static __device__ __align__(256) unsigned char hm_noalloc_scratch[HM_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[256];   // device address of hm_noalloc_scratch, per device ordinal

// In host code `hm_noalloc_scratch` names a host-side stand-in, not device
// memory: the device address is looked up once per device, with that device
// current, and cached.
int noalloc_scratch(void **out)
{
    int dev = -1;
    HM_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) { set_error("device ordinal %d out of range", dev); return HM_ERR_UNSUPPORTED; }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, hm_noalloc_scratch);
        if (e != cudaSuccess) {
            set_error("cudaGetSymbolAddress(hm_noalloc_scratch): %s", cudaGetErrorString(e));
            return HM_ERR_CUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return HM_OK;
}

}  // namespace

struct hm_plan {
    Plan P;
    std::vector<double> cheb, lam, T;
};

extern "C" {

int hm_chebyshev(int n, double *x, double *lambda)
{
    g_last_error.clear();
    if (n < 1 || !x || !lambda) { set_error("hm_chebyshev: bad arguments"); return HM_ERR_INVALID_ARG; }
    std::vector<double> xs, ws;
    chebyshev_first_kind(n, xs, ws);
    for (int k = 0; k < n; ++k) { x[k] = xs[k]; lambda[k] = ws[k]; }
    return HM_OK;
}

int hm_plan_create(const double *x, int64_t nx, const double *y, int64_t ny, double a, double b, double c,
                   double d, int rank, int64_t blocksize, hm_plan **out)
{
    if (!out) { set_error("out is NULL"); return HM_ERR_INVALID_ARG; }
    *out = nullptr;
    if (nx < 0 || ny < 0 || (nx > 0 && !x) || (ny > 0 && !y)) {
        set_error("negative length or NULL point list");
        return HM_ERR_INVALID_ARG;
    }
    if (nx == 0 || ny == 0) {
        // the reference's first indsplit reads x[1] (y[1]) of the empty list
        set_error("index out of bounds: indsplit reads the first point of an empty point list");
        return HM_ERR_BOUNDS;
    }
    if (nx >= (int64_t)1 << 31 || ny >= (int64_t)1 << 31) { set_error("more than 2^31 points"); return HM_ERR_UNSUPPORTED; }
    if (rank == 0) rank = 20;
    if (rank < 1 || rank > HM_RMAX) { set_error("rank %d outside 1..%d", rank, HM_RMAX); return HM_ERR_UNSUPPORTED; }
    if (blocksize == 0) blocksize = 4 * (int64_t)rank;
    if (blocksize < 1) { set_error("blocksize %lld < 1", (long long)blocksize); return HM_ERR_INVALID_ARG; }
    if (std::isnan(a) || std::isnan(b) || std::isnan(c) || std::isnan(d)) { set_error("NaN box end"); return HM_ERR_NAN; }
    if (!(a > b) || !(c > d)) { set_error("box ends must satisfy a > b and c > d"); return HM_ERR_BOX; }
    int st = check_points(x, nx, "x");
    if (!st) st = check_points(y, ny, "y");
    if (st) return st;
    hm_plan *pl = new hm_plan();
    chebyshev_first_kind(rank, pl->cheb, pl->lam);
    transfer_matrices(rank, pl->cheb, pl->lam, pl->T);
    st = build_plan(x, nx, y, ny, a, b, c, d, rank, blocksize, kSegRows, pl->P);
    if (st == PLAN_ERR_BOUNDS) {
        set_error("indsplit would read past the end of the point list");
        delete pl;
        return HM_ERR_BOUNDS;
    }
    if (st) { set_error("degenerate partition (status %d)", st); delete pl; return HM_ERR_DEGENERATE; }
    *out = pl;
    return HM_OK;
}

int hm_batch_plan_create(int ninst, const int64_t *nx, const int64_t *ny, const double *x, const double *y,
                         const double *boxes, int rank, int64_t blocksize, hm_plan **out)
{
    if (!out) { set_error("out is NULL"); return HM_ERR_INVALID_ARG; }
    *out = nullptr;
    if (ninst < 1 || !nx || !ny || !x || !y || !boxes) { set_error("hm_batch: bad arguments"); return HM_ERR_INVALID_ARG; }
    std::vector<int64_t> xo(ninst + 1, 0), yo(ninst + 1, 0);
    for (int i = 0; i < ninst; ++i) {
        if (nx[i] < 1 || ny[i] < 1) { set_error("instance %d is empty", i); return HM_ERR_INVALID_ARG; }
        xo[i + 1] = xo[i] + nx[i];
        yo[i + 1] = yo[i] + ny[i];
    }
    if (xo[ninst] >= (int64_t)1 << 31 || yo[ninst] >= (int64_t)1 << 31) { set_error("more than 2^31 points"); return HM_ERR_UNSUPPORTED; }
    std::vector<hm_plan *> parts(ninst, nullptr);
    std::vector<int> status(ninst, HM_OK);
    std::vector<std::string> errs(ninst);
    const int nth = std::max(1, std::min<int>(ninst, (int)std::thread::hardware_concurrency()));
    std::atomic<int> next(0);
    auto work = [&]() {
        for (int i = next++; i < ninst; i = next++) {
            const double *bx = boxes + 4 * (size_t)i;
            status[i] = hm_plan_create(x + xo[i], nx[i], y + yo[i], ny[i], bx[0], bx[1], bx[2], bx[3], rank, blocksize,
                                       &parts[i]);
            if (status[i]) errs[i] = g_last_error;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nth; ++t) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    int st = HM_OK;
    for (int i = 0; i < ninst && !st; ++i)
        if (status[i]) { st = status[i]; set_error("instance %d: %s", i, errs[i].c_str()); }
    hm_plan *pl = nullptr;
    if (!st) {
        pl = new hm_plan();
        std::vector<Plan> ps;
        ps.reserve(ninst);
        for (int i = 0; i < ninst; ++i) ps.push_back(std::move(parts[i]->P));
        merge_plans(ps, pl->P);
        pl->cheb = parts[0]->cheb; pl->lam = parts[0]->lam; pl->T = parts[0]->T;
    }
    for (hm_plan *p : parts) delete p;
    if (st) return st;
    *out = pl;
    return HM_OK;
}

int hm_plan_table(const hm_plan *pl, int which, const void **data, int64_t *count, int64_t *elem_bytes)
{
    if (!pl || !data || !count || !elem_bytes) return HM_ERR_INVALID_ARG;
    const Plan &P = pl->P;
#define HM_TAB(vec) { *data = (vec).data(); *count = (int64_t)(vec).size(); *elem_bytes = (int64_t)sizeof((vec)[0]); return HM_OK; }
    switch (which) {
    case 0: HM_TAB(P.vpanels)
    case 1: HM_TAB(P.vpanel_fill)
    case 2: HM_TAB(P.up)
    case 3: HM_TAB(P.up_level_ptr)
    case 4: HM_TAB(P.m2l_rows)
    case 5: HM_TAB(P.m2l_ents)
    case 6: HM_TAB(P.f_fill)
    case 7: HM_TAB(P.down)
    case 8: HM_TAB(P.down_level_ptr)
    case 9: HM_TAB(P.segs)
    case 10: HM_TAB(P.pieces)
    case 11: HM_TAB(P.seg_fill)
    case 12: HM_TAB(pl->T)
    case 13: HM_TAB(pl->cheb)
    case 14: HM_TAB(pl->lam)
    case 15: HM_TAB(P.up_ents)
    case 16: HM_TAB(P.up_steps)
    case 17: HM_TAB(P.up_tasks)
    case 18: HM_TAB(P.up_band_ptr)
    case 19: HM_TAB(P.down_ents)
    case 20: HM_TAB(P.down_steps)
    case 21: HM_TAB(P.down_tasks)
    case 22: HM_TAB(P.down_band_ptr)
    default: return HM_ERR_INVALID_ARG;
    }
#undef HM_TAB
}

int hm_plan_sizes(const hm_plan *pl, int64_t *out, int nout)
{
    if (!pl || !out) return 0;
    const Plan &P = pl->P;
    const int64_t v[] = {P.r, P.nx, P.ny, P.n_xslots, P.n_yslots, P.vstore_elems, P.fstore_elems,
                         P.pstore_elems, P.max_width, P.stats.n_bary, P.stats.n_dense, P.stats.depth,
                         P.stats.canonical_values, P.stats.reference_values, P.stats.stored_values,
                         P.stats.dense_values, P.stats.n_segments};
    const int nv = (int)(sizeof(v) / sizeof(v[0]));
    const int w = std::min(nv, nout);
    for (int i = 0; i < w; ++i) out[i] = v[i];
    return w;
}

void hm_plan_free(hm_plan *pl) { delete pl; }

const char *hm_status_string(int status)
{
    switch (status) {
    case HM_OK: return "ok";
    case HM_ERR_INVALID_ARG: return "invalid argument";
    case HM_ERR_UNSORTED: return "points are not in non-increasing order";
    case HM_ERR_BOUNDS: return "index out of bounds";
    case HM_ERR_NAN: return "NaN input";
    case HM_ERR_CUDA: return "CUDA error";
    case HM_ERR_ALLOC: return "device allocation failed";
    case HM_ERR_UNSUPPORTED: return "unsupported parameter";
    case HM_ERR_BOX: return "box ends must satisfy a > b and c > d";
    case HM_ERR_DEGENERATE: return "degenerate partition";
    case HM_ERR_NOT_POSDEF: return "matrix is not positive definite";
    default: return "unknown status";
    }
}

const char *hm_last_error(void) { return g_last_error.c_str(); }

int hm_version(void) { return 100; }

int hm_blockrank(double eps)
{
    if (!(eps > 0.0) || !(eps < 1.0)) return 0;
    const double v = 0.5 * (std::log(1.0 / eps) / std::log(3.0 + std::sqrt(8.0)));
    return 2 * (int)std::llround(v);
}

int hm_indsplit(const double *x, int64_t n, int64_t start, int64_t len, double a, double b, int64_t *out4)
{
    if (!x || !out4 || n < 0 || start < 0 || len < 0) { set_error("hm_indsplit: bad arguments"); return HM_ERR_INVALID_ARG; }
    const double mid = 0.5 * (a + b);
    int64_t i = start;
    // The reference's scan (src/BarycentricMatrix.jl:299-307), first element
    // read even for an empty range.
    for (;;) {
        if (i >= n) { set_error("indsplit: index %lld past the end (%lld)", (long long)i, (long long)n); return HM_ERR_BOUNDS; }
        if (!(x[i] >= mid)) break;
        i += 1;
        if (i > start + len - 1) break;
    }
    out4[0] = start; out4[1] = i - start;
    out4[2] = i; out4[3] = std::max<int64_t>(0, start + len - i);
    return HM_OK;
}

}  // extern "C"

namespace {

int build_from_plan(int kernel, int swap, hm_plan *pl, const double *x, const double *y, int storage, void *stream,
                    hm_handle **out);

// Builds the KernelMatrix of (x, y) -- or, with swap = 1, the matrix with
// entries f(y_j, x_i), i.e. the transpose of the KernelMatrix of (y, x).
int build_kernelmatrix(int kernel, int swap, const double *x, int64_t nx, const double *y, int64_t ny, double a,
                       double b, double c, double d, int rank, int64_t blocksize, int storage, void *stream,
                       hm_handle **out)
{
    if (!out) { set_error("out is NULL"); return HM_ERR_INVALID_ARG; }
    *out = nullptr;
    if (kernel < HM_KERNEL_CAUCHY || kernel > HM_KERNEL_LOG) { set_error("unknown kernel %d", kernel); return HM_ERR_UNSUPPORTED; }
    if (storage != HM_F64 && storage != HM_F32 && storage != HM_DF64) { set_error("unknown storage %d", storage); return HM_ERR_UNSUPPORTED; }
    hm_plan *pl = nullptr;
    int st = hm_plan_create(x, nx, y, ny, a, b, c, d, rank, blocksize, &pl);
    if (st) return st;
    st = build_from_plan(kernel, swap, pl, x, y, storage, stream, out);
    if (*out) {
        hm_handle *h = *out;
        h->hx.assign(x, x + nx);
        h->hy.assign(y, y + ny);
        h->box[0] = a; h->box[1] = b; h->box[2] = c; h->box[3] = d;
        h->blocksize = blocksize ? blocksize : 4 * (int64_t)h->r;
    }
    return st;
}

// Uploads a plan and compresses on the GPU; frees the plan.
int build_from_plan(int kernel, int swap, hm_plan *pl, const double *x, const double *y, int storage, void *stream,
                    hm_handle **out)
{
    *out = nullptr;
    int st = HM_OK;
    const Plan &P = pl->P;
    const int64_t nx = P.nx, ny = P.ny;
    const int rank = P.r;
    const std::vector<double> &cheb = pl->cheb, &lam = pl->lam, &T = pl->T;

    hm_handle *h = new hm_handle();
    cudaGetDevice(&h->device);
    h->kernel = kernel; h->storage = storage; h->r = rank; h->nx = nx; h->ny = ny; h->swap = swap;
    h->stats = P.stats;
    h->n_xslots = P.n_xslots; h->n_yslots = P.n_yslots; h->max_width = P.max_width;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    st = f64_vectors(storage) ? build_device<double>(h, P, cheb, lam, T, x, y, cs)
                             : build_device<float>(h, P, cheb, lam, T, x, y, cs);
    hm_plan_free(pl);
    auto nonempty = [](const std::vector<int> &ptr) {
        int c = 0;
        for (size_t i = 0; i + 1 < ptr.size(); ++i) c += ptr[i + 1] > ptr[i];
        return c;
    };
    h->launches_per_mul = (h->n_vp > 0) + nonempty(h->up_band_ptr) + (h->n_m2l_rows > 0) + nonempty(h->down_band_ptr) +
                          (h->n_segs > 0) * (1 + 2 * ((h->n_vp > 0) || (h->n_m2l_rows > 0)));
    if (st) { hm_free(h); return st; }
    *out = h;
    return HM_OK;
}

}  // namespace

extern "C" {

int hm_kernelmatrix_build(int kernel, const double *x, int64_t nx, const double *y, int64_t ny,
                          double a, double b, double c, double d, int rank, int64_t blocksize,
                          int storage, void *stream, hm_handle **out)
{
    g_last_error.clear();
    return build_kernelmatrix(kernel, 0, x, nx, y, ny, a, b, c, d, rank, blocksize, storage, stream, out);
}

int hm_kernelmatrix_batch_build(int kernel, int ninst, const int64_t *nx, const int64_t *ny, const double *x,
                                const double *y, const double *boxes, int rank, int64_t blocksize, int storage,
                                void *stream, hm_handle **out)
{
    g_last_error.clear();
    if (!out) { set_error("out is NULL"); return HM_ERR_INVALID_ARG; }
    *out = nullptr;
    if (kernel < HM_KERNEL_CAUCHY || kernel > HM_KERNEL_LOG) { set_error("unknown kernel %d", kernel); return HM_ERR_UNSUPPORTED; }
    if (storage != HM_F64 && storage != HM_F32 && storage != HM_DF64) { set_error("unknown storage %d", storage); return HM_ERR_UNSUPPORTED; }
    hm_plan *pl = nullptr;
    HM_TRY(hm_batch_plan_create(ninst, nx, ny, x, y, boxes, rank, blocksize, &pl));
    const int st = build_from_plan(kernel, 0, pl, x, y, storage, stream, out);
    if (*out) (*out)->ninst = ninst;
    return st;
}

int hm_hier_build(int storage, int64_t m, int64_t n, int nblocks, const int32_t *kinds, const int64_t *row0,
                  const int64_t *rows, const int64_t *col0, const int64_t *cols, const int64_t *ranks,
                  const double *values, const int64_t *offsets, void *stream, hm_handle **out)
{
    g_last_error.clear();
    if (!out) { set_error("out is NULL"); return HM_ERR_INVALID_ARG; }
    *out = nullptr;
    if (storage != HM_F64 && storage != HM_F32 && storage != HM_DF64) { set_error("unknown storage %d", storage); return HM_ERR_UNSUPPORTED; }
    if (m < 0 || n < 0 || nblocks < 0 || (nblocks && (!kinds || !row0 || !rows || !col0 || !cols || !ranks || !values || !offsets))) {
        set_error("hm_hier_build: bad arguments");
        return HM_ERR_INVALID_ARG;
    }
    if (m >= (int64_t)1 << 31 || n >= (int64_t)1 << 31) { set_error("more than 2^31 rows or columns"); return HM_ERR_UNSUPPORTED; }
    std::vector<HierBlock> blocks(nblocks);
    for (int i = 0; i < nblocks; ++i) {
        HierBlock &b = blocks[i];
        b.kind = kinds[i]; b.row0 = row0[i]; b.rows = rows[i]; b.col0 = col0[i]; b.cols = cols[i];
        b.rank = b.kind == 0 ? 0 : ranks[i];
        b.data = values + offsets[i];
        if (b.kind < 0 || b.kind > 2 || b.rows < 0 || b.cols < 0 || b.rank < 0) {
            set_error("block %d: bad kind or size", i);
            return HM_ERR_INVALID_ARG;
        }
        if (b.row0 < 0 || b.col0 < 0 || b.row0 + b.rows > m || b.col0 + b.cols > n) {
            set_error("block %d: rows [%lld, %lld) or columns [%lld, %lld) outside the %lld x %lld matrix", i,
                      (long long)b.row0, (long long)(b.row0 + b.rows), (long long)b.col0, (long long)(b.col0 + b.cols),
                      (long long)m, (long long)n);
            return HM_ERR_BOUNDS;
        }
    }
    Plan P;
    std::vector<double> vs, fs, ps;
    if (build_hier_plan(m, n, blocks, P, vs, fs, ps)) {
        set_error("core (BarycentricMatrix2D) blocks need rank <= 32 in a matrix whose ranks are all <= 32");
        return HM_ERR_UNSUPPORTED;
    }
    hm_handle *h = new hm_handle();
    cudaGetDevice(&h->device);
    h->kernel = -1; h->storage = storage; h->r = P.r; h->nx = m; h->ny = n;
    h->stats = P.stats;
    h->n_xslots = P.n_xslots; h->n_yslots = P.n_yslots; h->max_width = P.max_width;
    h->ninst = 0;       // no transposed or derivative plans for user-assembled matrices
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    const int st = storage == HM_F64 ? build_hier_device<double>(h, P, vs, fs, ps, cs)
                                     : build_hier_device<float>(h, P, vs, fs, ps, cs);
    h->launches_per_mul = (h->n_vp > 0) + (h->n_m2l_rows > 0) +
                          (h->n_segs > 0) * (1 + 2 * ((h->n_vp > 0) || (h->n_m2l_rows > 0)));
    if (st) { hm_free(h); return st; }
    *out = h;
    return HM_OK;
}

// ---- block-level products on device arrays -----------------------------------

static int check_strided(int64_t len, int64_t start, int64_t inc, int64_t count, const char *name)
{
    if (start < 1 || inc < 1) { set_error("%s: start and increment must be >= 1", name); return HM_ERR_INVALID_ARG; }
    if (count > 0 && (start - 1) + (count - 1) * inc >= len) {
        set_error("%s: strided access past the end (length %lld)", name, (long long)len);
        return HM_ERR_BOUNDS;
    }
    return HM_OK;
}

int hm_dense_mul(int trans, int dtype, const void *A, int64_t m, int64_t n, int64_t lda, const void *x, int64_t lenx,
                 int64_t jstart, int64_t incx, void *y, int64_t leny, int64_t istart, int64_t incy, void *stream)
{
    g_last_error.clear();
    if (!A || !x || !y || m < 0 || n < 0 || lda < std::max<int64_t>(m, 1)) { set_error("hm_dense_mul: bad arguments"); return HM_ERR_INVALID_ARG; }
    if (dtype != HM_F64 && dtype != HM_F32) { set_error("unknown dtype %d", dtype); return HM_ERR_UNSUPPORTED; }
    const int64_t nin = trans ? m : n, nout = trans ? n : m;
    HM_TRY(check_strided(lenx, jstart, incx, nin, "x"));
    HM_TRY(check_strided(leny, istart, incy, nout, "y"));
    if (nout == 0) return HM_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t es = dtype == HM_F64 ? 8 : 4;
    const void *xb = static_cast<const char *>(x) + (size_t)(jstart - 1) * es;
    void *yb = static_cast<char *>(y) + (size_t)(istart - 1) * es;
    if (!trans) {
        const unsigned grid = (unsigned)((m + 255) / 256);
        if (dtype == HM_F64) gemv_n<double><<<grid, 256, 0, st>>>((const double *)A, m, n, lda, (const double *)xb, incx, (double *)yb, incy);
        else gemv_n<float><<<grid, 256, 0, st>>>((const float *)A, m, n, lda, (const float *)xb, incx, (float *)yb, incy);
    } else {
        const unsigned grid = (unsigned)((n * 32 + 255) / 256);
        if (dtype == HM_F64) gemv_t<double><<<grid, 256, 0, st>>>((const double *)A, m, n, lda, (const double *)xb, incx, (double *)yb, incy);
        else gemv_t<float><<<grid, 256, 0, st>>>((const float *)A, m, n, lda, (const float *)xb, incx, (float *)yb, incy);
    }
    HM_CK_LAUNCH("hm_dense_mul");
    return HM_OK;
}

}  // extern "C"

template <typename T>
static int lowrank_mul_t(int adjoint, const T *U, const T *core, int core_diag, const T *V, int64_t m, int64_t n,
                         int64_t r, const T *x, int64_t incx, T *y, int64_t incy, cudaStream_t st)
{
    // product:  t = V^T x, y += U (C t);  adjoint:  t = U^T x, y += V (C^T t)
    const T *Win = adjoint ? U : V, *Wout = adjoint ? V : U;
    const int64_t rin = adjoint ? m : n, rout = adjoint ? n : m;
    if (r == 0 || rout == 0) return HM_OK;
    T *t = nullptr;
    HM_CK(device_malloc_async((void **)&t, sizeof(T) * r, st));
    lr_project<T><<<(unsigned)((r * 32 + 255) / 256), 256, 0, st>>>(Win, rin, rin, r, x, incx, t);
    int e = cuda_status(cudaGetLastError(), "lr_project");
    if (!e) {
        const size_t smem = sizeof(T) * r;
        if (smem > 48 * 1024) e = cuda_status(cudaFuncSetAttribute(lr_expand<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(smem, 227 * 1024)), "lr_expand attribute");
        if (!e && smem > 227 * 1024) { set_error("rank %lld too large", (long long)r); e = HM_ERR_UNSUPPORTED; }
        if (!e) {
            lr_expand<T><<<(unsigned)((rout + 255) / 256), 256, smem, st>>>(Wout, rout, rout, r, core, core_diag, adjoint, t, y, incy);
            e = cuda_status(cudaGetLastError(), "lr_expand");
        }
    }
    cudaError_t fe = cudaFreeAsync(t, st);
    if (!e) e = cuda_status(fe, "cudaFreeAsync");
    return e;
}

extern "C" {

int hm_lowrank_mul(int adjoint, int dtype, const void *U, const void *core, int core_diag, const void *V, int64_t m,
                   int64_t n, int64_t r, const void *x, int64_t lenx, int64_t jstart, int64_t incx, void *y,
                   int64_t leny, int64_t istart, int64_t incy, void *stream)
{
    g_last_error.clear();
    if (!U || !core || !V || !x || !y || m < 0 || n < 0 || r < 0) { set_error("hm_lowrank_mul: bad arguments"); return HM_ERR_INVALID_ARG; }
    if (dtype != HM_F64 && dtype != HM_F32) { set_error("unknown dtype %d", dtype); return HM_ERR_UNSUPPORTED; }
    const int64_t nin = adjoint ? m : n, nout = adjoint ? n : m;
    HM_TRY(check_strided(lenx, jstart, incx, nin, "x"));
    HM_TRY(check_strided(leny, istart, incy, nout, "y"));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64)
        return lowrank_mul_t<double>(adjoint, (const double *)U, (const double *)core, core_diag, (const double *)V, m, n, r,
                                     (const double *)x + (jstart - 1), incx, (double *)y + (istart - 1), incy, st);
    return lowrank_mul_t<float>(adjoint, (const float *)U, (const float *)core, core_diag, (const float *)V, m, n, r,
                                (const float *)x + (jstart - 1), incx, (float *)y + (istart - 1), incy, st);
}

int hm_bary_factors(int kernel, int rank, double a, double b, double c, double d, const double *x, int64_t nx,
                    const double *y, int64_t ny, int dtype, void *U, void *F, void *V, void *stream)
{
    g_last_error.clear();
    if (kernel < HM_KERNEL_CAUCHY || kernel > HM_KERNEL_LOG) { set_error("unknown kernel %d", kernel); return HM_ERR_UNSUPPORTED; }
    if (dtype != HM_F64 && dtype != HM_F32) { set_error("unknown dtype %d", dtype); return HM_ERR_UNSUPPORTED; }
    if (rank < 1 || rank > HM_RMAX) { set_error("rank %d outside 1..%d", rank, HM_RMAX); return HM_ERR_UNSUPPORTED; }
    if (!x || !y || !U || !F || !V || nx < 0 || ny < 0) { set_error("hm_bary_factors: bad arguments"); return HM_ERR_INVALID_ARG; }
    std::vector<double> cheb, lam;
    chebyshev_first_kind(rank, cheb, lam);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *dbuf = nullptr;
    const size_t nbuf = 2 * (size_t)rank + nx + ny;
    HM_CK(device_malloc_async((void **)&dbuf, sizeof(double) * std::max<size_t>(nbuf, 1), st));
    int e = cuda_status(cudaMemcpyAsync(dbuf, cheb.data(), sizeof(double) * rank, cudaMemcpyHostToDevice, st), "copy");
    if (!e) e = cuda_status(cudaMemcpyAsync(dbuf + rank, lam.data(), sizeof(double) * rank, cudaMemcpyHostToDevice, st), "copy");
    if (!e && nx) e = cuda_status(cudaMemcpyAsync(dbuf + 2 * rank, x, sizeof(double) * nx, cudaMemcpyHostToDevice, st), "copy");
    if (!e && ny) e = cuda_status(cudaMemcpyAsync(dbuf + 2 * rank + nx, y, sizeof(double) * ny, cudaMemcpyHostToDevice, st), "copy");
    if (!e) {
        const int64_t work = std::max<int64_t>({(int64_t)rank * rank, nx, ny});
        const unsigned grid = (unsigned)((work + 127) / 128);
        if (dtype == HM_F64)
            bary_factors<double><<<grid, 128, 0, st>>>(kernel, rank, a, b, c, d, dbuf, dbuf + rank, dbuf + 2 * rank, nx,
                                                       dbuf + 2 * rank + nx, ny, (double *)U, (double *)F, (double *)V);
        else
            bary_factors<float><<<grid, 128, 0, st>>>(kernel, rank, a, b, c, d, dbuf, dbuf + rank, dbuf + 2 * rank, nx,
                                                      dbuf + 2 * rank + nx, ny, (float *)U, (float *)F, (float *)V);
        e = cuda_status(cudaGetLastError(), "bary_factors");
    }
    cudaError_t fe = cudaFreeAsync(dbuf, st);
    if (!e) e = cuda_status(fe, "cudaFreeAsync");
    if (!e) e = cuda_status(cudaStreamSynchronize(st), "bary_factors sync");
    return e;
}

int hm_mul_t(hm_handle *h, const void *v, int64_t ldv, void *u, int64_t ldu, int nrhs, int accumulate,
             void *stream)
{
    g_last_error.clear();
    if (!h) { set_error("NULL handle"); return HM_ERR_INVALID_ARG; }
    if (h->ninst != 1 || h->hx.empty()) { set_error("hm_mul_t: not available for batched or user-assembled handles"); return HM_ERR_UNSUPPORTED; }
    if (nrhs == 0) return HM_OK;          // nothing read or written (the vectors may be NULL)
    {
        std::lock_guard<std::mutex> lk(h->trans_mu);
        if (!h->trans) {
            // H^T = the matrix of f(row, col) swapped, on the tree of (y, x)
            HM_TRY(build_kernelmatrix(h->kernel, 1 - h->swap, h->hy.data(), h->ny, h->hx.data(), h->nx, h->box[2],
                                      h->box[3], h->box[0], h->box[1], h->r, h->blocksize, h->storage, stream,
                                      &h->trans));
        }
    }
    return hm_mul(h->trans, v, ldv, u, ldu, nrhs, accumulate, stream);
}

int hm_size(const hm_handle *h, int64_t *m, int64_t *n)
{
    if (!h || !m || !n) return HM_ERR_INVALID_ARG;
    *m = h->nx; *n = h->ny;
    return HM_OK;
}

int hm_storage(const hm_handle *h) { return h ? h->storage : -1; }

int hm_stats(const hm_handle *h, int64_t *out, int nout)
{
    if (!h || !out) return 0;
    const int64_t v[] = {h->stats.n_bary, h->stats.n_dense, h->stats.depth, h->stats.n_xslots,
                         h->stats.n_yslots, h->stats.canonical_values, h->stats.reference_values,
                         h->stats.stored_values, h->stats.dense_values, h->stats.n_segments,
                         h->stats.max_width, h->device_bytes, h->launches_per_mul};
    const int nv = (int)(sizeof(v) / sizeof(v[0]));
    const int w = std::min(nv, nout);
    for (int i = 0; i < w; ++i) out[i] = v[i];
    return w;
}

int hm_device_status(hm_handle *h, int *code, int reset)
{
    if (!h || !code) return HM_ERR_INVALID_ARG;
    *code = 0;
    if (!h->d_status) return HM_OK;
    HM_CK(cudaDeviceSynchronize());
    HM_CK(cudaMemcpy(code, h->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (reset) HM_CK(cudaMemset(h->d_status, 0, sizeof(int)));
    if (h->trans && *code == 0) return hm_device_status(h->trans, code, reset);
    return HM_OK;
}

int hm_mul(hm_handle *h, const void *v, int64_t ldv, void *u, int64_t ldu, int nrhs, int accumulate,
           void *stream)
{
    g_last_error.clear();
    if (!h) { set_error("NULL handle"); return HM_ERR_INVALID_ARG; }
    if (nrhs < 0) { set_error("nrhs < 0"); return HM_ERR_INVALID_ARG; }
    if (nrhs == 0) return HM_OK;          // nothing read or written (the vectors may be NULL)
    if (!v || !u) { set_error("NULL argument"); return HM_ERR_INVALID_ARG; }
    if (nrhs > 1 && (ldv < h->ny || ldu < h->nx)) { set_error("leading dimension too small"); return HM_ERR_BOUNDS; }
    return dispatch_mul(h, v, 1, ldv, u, 1, ldu, nrhs, accumulate ? 1 : 0, static_cast<cudaStream_t>(stream));
}

int hm_mul_drow(hm_handle *h, int transposed, const void *v, int64_t ldv, void *u, int64_t ldu, int nrhs,
                int accumulate, void *stream)
{
    g_last_error.clear();
    if (!h) { set_error("NULL handle"); return HM_ERR_INVALID_ARG; }
    if (nrhs < 0) { set_error("nrhs < 0"); return HM_ERR_INVALID_ARG; }
    if (nrhs == 0) return HM_OK;          // nothing read or written (the vectors may be NULL)
    if (!v || !u) { set_error("NULL argument"); return HM_ERR_INVALID_ARG; }
    if (transposed) {
        if (h->ninst != 1 || h->hx.empty()) { set_error("transposed products are not available for batched or user-assembled handles"); return HM_ERR_UNSUPPORTED; }
        {
            std::lock_guard<std::mutex> lk(h->trans_mu);
            if (!h->trans)
                HM_TRY(build_kernelmatrix(h->kernel, 1 - h->swap, h->hy.data(), h->ny, h->hx.data(), h->nx, h->box[2],
                                          h->box[3], h->box[0], h->box[1], h->r, h->blocksize, h->storage, stream,
                                          &h->trans));
        }
        return hm_mul_drow(h->trans, 0, v, ldv, u, ldu, nrhs, accumulate, stream);
    }
    if (h->kernel < 0) { set_error("derivative products need a KernelMatrix handle"); return HM_ERR_UNSUPPORTED; }
    if (nrhs < 0) { set_error("nrhs < 0"); return HM_ERR_INVALID_ARG; }
    if (nrhs > 1 && (ldv < h->ny || ldu < h->nx)) { set_error("leading dimension too small"); return HM_ERR_BOUNDS; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (f64_vectors(h->storage)) {
        HM_TRY(ensure_drow<double>(h, st));
        MulArgs<double> ma{static_cast<const double *>(v), static_cast<double *>(u), 1, ldv, 1, ldu, nrhs, accumulate ? 1 : 0};
        return run_mul<double, double>(h, ma, st, h->d_dP);
    }
    HM_TRY(ensure_drow<float>(h, st));
    MulArgs<float> ma{static_cast<const float *>(v), static_cast<float *>(u), 1, ldv, 1, ldu, nrhs, accumulate ? 1 : 0};
    return run_mul<float, float>(h, ma, st, h->d_dP);
}

int hm_mul_strided(hm_handle *h, const void *x, int64_t lenx, int64_t jstart, int64_t incx, void *y,
                   int64_t leny, int64_t istart, int64_t incy, void *stream)
{
    g_last_error.clear();
    if (!h || !x || !y) { set_error("NULL argument"); return HM_ERR_INVALID_ARG; }
    if (istart < 1 || jstart < 1 || incx < 1 || incy < 1) { set_error("istart/jstart/INCX/INCY must be >= 1"); return HM_ERR_INVALID_ARG; }
    if ((jstart - 1) + (h->ny - 1) * incx >= lenx || (istart - 1) + (h->nx - 1) * incy >= leny) {
        set_error("strided access past the end of x or y");
        return HM_ERR_BOUNDS;
    }
    const size_t es = f64_vectors(h->storage) ? 8 : 4;
    const char *xb = static_cast<const char *>(x) + (size_t)(jstart - 1) * es;
    char *yb = static_cast<char *>(y) + (size_t)(istart - 1) * es;
    return dispatch_mul(h, xb, incx, 0, yb, incy, 0, 1, 1, static_cast<cudaStream_t>(stream));
}

int hm_mul_host(hm_handle *h, const void *v, void *u, int nrhs, int accumulate)
{
    g_last_error.clear();
    if (!h || nrhs < 0) { set_error("bad argument"); return HM_ERR_INVALID_ARG; }
    if (nrhs == 0) return HM_OK;          // nothing read or written (the vectors may be NULL)
    if (!v || !u) { set_error("NULL argument"); return HM_ERR_INVALID_ARG; }
    const size_t es = f64_vectors(h->storage) ? 8 : 4;
    const size_t bv = (size_t)h->ny * nrhs * es, bu = (size_t)h->nx * nrhs * es;
    if (!h->host_stream) HM_CK(cudaStreamCreateWithFlags(&h->host_stream, cudaStreamNonBlocking));
    cudaStream_t st = h->host_stream;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        if (h->stage_bytes < bv + bu) {
            if (h->d_stage) HM_CK(cudaFree(h->d_stage));
            h->d_stage = nullptr; h->stage_bytes = 0;
            HM_CK(device_malloc(&h->d_stage, bv + bu));
            h->stage_bytes = bv + bu;
        }
    }
    char *dv = static_cast<char *>(h->d_stage), *du = dv + bv;
    // a page-locked destination is written by the product's last kernel
    // directly (no separate device-to-host copy after it)
    void *uout = ends_with_add_far(h, nrhs) ? pinned_device_ptr(u) : nullptr;
    // a page-locked source is read by the leaf stage, which stores it for the
    // near field (no separate host-to-device copy before the product)
    const void *vin = leaf_reads_input(h, nrhs) ? pinned_device_ptr(v) : nullptr;
    if (!vin) HM_CK(cudaMemcpyAsync(dv, v, bv, cudaMemcpyHostToDevice, st));
    if (accumulate) HM_CK(cudaMemcpyAsync(du, u, bu, cudaMemcpyHostToDevice, st));
    auto &hg = h->host_graph;
    const int acc = accumulate ? 1 : 0;
    if (hg.nrhs != nrhs || hg.acc != acc || hg.stage != h->d_stage || hg.out != uout || hg.in != vin) {
        if (hg.exec) cudaGraphExecDestroy(hg.exec);
        hg = hm_handle::HostGraph();
        hg.nrhs = nrhs; hg.acc = acc; hg.stage = h->d_stage; hg.out = uout; hg.in = vin;
    }
    if (!hg.exec && hg.warm && h->profile_mask == 0) {
        HM_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int e = dispatch_mul(h, dv, 1, h->ny, du, 1, h->nx, nrhs, acc, st, uout, vin);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (e) { if (g) cudaGraphDestroy(g); return e; }
        if (ce != cudaSuccess) { set_error("hm_mul_host capture: %s", cudaGetErrorString(ce)); return HM_ERR_CUDA; }
        const cudaError_t ie = cudaGraphInstantiate(&hg.exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) { hg.exec = nullptr; set_error("hm_mul_host graph: %s", cudaGetErrorString(ie)); return HM_ERR_CUDA; }
    }
    if (hg.exec && h->profile_mask == 0) {
        HM_CK(cudaGraphLaunch(hg.exec, st));
    } else {
        const int e = dispatch_mul(h, dv, 1, h->ny, du, 1, h->nx, nrhs, acc, st, uout, vin);
        if (e) return e;
        hg.warm = true;
    }
    if (!uout) HM_CK(cudaMemcpyAsync(u, du, bu, cudaMemcpyDeviceToHost, st));
    HM_CK(cudaStreamSynchronize(st));
    return HM_OK;
}

int hm_direct_rows(hm_handle *h, const double *b, const int64_t *rows, int64_t nrows, double *out, void *stream)
{
    g_last_error.clear();
    if (!h || !b || !rows || !out || nrows < 0) { set_error("bad argument"); return HM_ERR_INVALID_ARG; }
    if (nrows == 0) return HM_OK;
    direct_rows<<<(unsigned)nrows, 256, 0, static_cast<cudaStream_t>(stream)>>>(h->kernel, h->d_x, h->nx, h->d_y, h->ny,
                                                                              b, rows, nrows, out);
    HM_CK_LAUNCH("direct_rows");
    return HM_OK;
}

int hm_mul_noalloc(hm_handle *h, const void *v, void *u, int accumulate, void *stream)
{
    g_last_error.clear();
    if (!h || !v || !u) { set_error("NULL argument"); return HM_ERR_INVALID_ARG; }
    const size_t need = f64_vectors(h->storage) ? scratch_layout<double>(h, 1).bytes : scratch_layout<float>(h, 1).bytes;
    if (need > HM_NOALLOC_SCRATCH_BYTES) {
        set_error("hm_mul_noalloc: this matrix needs %zu bytes of coefficient scratch; the library's fixed "
                  "scratch holds %u bytes (use hm_mul)", need, (unsigned)HM_NOALLOC_SCRATCH_BYTES);
        return HM_ERR_UNSUPPORTED;
    }
    int dev = -1;
    HM_CK(cudaGetDevice(&dev));
    if (dev != h->device) {
        set_error("hm_mul_noalloc: the handle was built on device %d, device %d is current", h->device, dev);
        return HM_ERR_INVALID_ARG;
    }
    void *scratch = nullptr;
    HM_TRY(noalloc_scratch(&scratch));
    // the schedule hm_mul would use for one right-hand side (the autotuned one
    // when there is one), with every stage in order on the caller's stream:
    // no side stream, no event
    Sched sched = sched_for(h, 1);
    sched.overlap = 0;
    SchedScope scope(&sched);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (f64_vectors(h->storage)) {
        MulArgs<double> ma{static_cast<const double *>(v), static_cast<double *>(u), 1, h->ny, 1, h->nx, 1,
                           accumulate ? 1 : 0};
        return launch_pipeline<double, double>(h, ma, st, st, nullptr, nullptr, scratch, false);
    }
    MulArgs<float> ma{static_cast<const float *>(v), static_cast<float *>(u), 1, h->ny, 1, h->nx, 1,
                      accumulate ? 1 : 0};
    return launch_pipeline<float, float>(h, ma, st, st, nullptr, nullptr, scratch, false);
}

int hm_autotune_choice(const hm_handle *h, int nrhs, int32_t *out, int nout)
{
    if (!h || nrhs <= 0 || !out || nout < 0) { set_error("hm_autotune_choice: bad argument"); return -HM_ERR_INVALID_ARG; }
    const int b = sched_bucket(nrhs);
    Sched sc;
    {
        std::lock_guard<std::mutex> lk(const_cast<hm_handle *>(h)->mu);
        sc = h->tuned_ok[b] ? h->tuned[b] : configured_sched(h);
    }
    const int32_t v[7] = {sc.overlap, sc.near_kernel, sc.near_stages, sc.tensor_cores, sc.pdl, sc.tile, sc.wide};
    const int n = std::min(nout, 7);
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return n;
}

int hm_debug_fail_alloc(int64_t after)
{
    if (after < -1) { set_error("hm_debug_fail_alloc: after must be >= -1"); return HM_ERR_INVALID_ARG; }
    hm::g_fail_alloc.store(after);
    return HM_OK;
}

int hm_autotune(hm_handle *h, int nrhs, int reps, void *stream, int32_t *choice, double *ms)
{
    g_last_error.clear();
    if (!h || nrhs <= 0 || reps <= 0) { set_error("hm_autotune: bad argument"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    HM_CK(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
        set_error("hm_autotune: not allowed while the stream is being captured");
        return HM_ERR_INVALID_ARG;
    }
    return f64_vectors(h->storage) ? autotune<double>(h, nrhs, reps, st, choice, ms)
                                : autotune<float>(h, nrhs, reps, st, choice, ms);
}

int hm_configure(hm_handle *h, int option, int64_t value)
{
    if (!h) return HM_ERR_INVALID_ARG;
    // options of the bounded waits: no schedule changes, tuned schedules kept
    // (the host-buffer graph holds the old kernel arguments: dropped)
    if (option == HM_OPT_WIDE_TREE) {
        if (value < 0 || value > 2) { set_error("HM_OPT_WIDE_TREE must be 0, 1 or 2"); return HM_ERR_INVALID_ARG; }
        drop_host_graph(h);
        {
            std::lock_guard<std::mutex> lk(h->mu);
            h->wide_tree = (int)value;
            for (Sched &t : h->tuned) t.wide = (int)value;
        }
        if (h->trans) return hm_configure(h->trans, option, value);
        return HM_OK;
    }
    if (option == HM_OPT_WAIT_LIMIT_NS || option == HM_OPT_TEST_STALL) {
        if (option == HM_OPT_WAIT_LIMIT_NS && (value < 1 || value > 2000000000)) {
            set_error("HM_OPT_WAIT_LIMIT_NS must be in [1, 2e9]");
            return HM_ERR_INVALID_ARG;
        }
        drop_host_graph(h);
        if (option == HM_OPT_WAIT_LIMIT_NS) h->wait_ns = (unsigned long long)value;
        else h->test_stall = value != 0 ? 1 : 0;
        if (h->trans) return hm_configure(h->trans, option, value);
        return HM_OK;
    }
    switch (option) {
    case HM_OPT_OVERLAP:
        if (value < 0 || value > 4) { set_error("HM_OPT_OVERLAP must be in [0, 4]"); return HM_ERR_INVALID_ARG; }
        break;
    case HM_OPT_TENSOR_CORES: break;
    case HM_OPT_NEAR_KERNEL:
        if (value < 0 || value > 3) { set_error("HM_OPT_NEAR_KERNEL must be 0, 1, 2 or 3"); return HM_ERR_INVALID_ARG; }
        break;
    case HM_OPT_NEAR_STAGES:
        if (value < 2 || value > 16) { set_error("HM_OPT_NEAR_STAGES must be in [2, 16]"); return HM_ERR_INVALID_ARG; }
        break;
    case HM_OPT_AUTOTUNED:
        if (value != 0) { set_error("HM_OPT_AUTOTUNED takes 0 (forget the tuned schedules)"); return HM_ERR_INVALID_ARG; }
        break;
    case HM_OPT_PDL: break;
    case HM_OPT_RING_TILE:
        if (value < 0 || value >= kRingTiles) { set_error("HM_OPT_RING_TILE must be 0, 1 or 2"); return HM_ERR_INVALID_ARG; }
        break;
    default: set_error("unknown option %d", option); return HM_ERR_INVALID_ARG;
    }
    // the host-buffer product's captured graph follows the options: drop it;
    // an explicit option also replaces the autotuned schedules
    drop_host_graph(h);
    {
        std::lock_guard<std::mutex> lk(h->mu);
        for (bool &ok : h->tuned_ok) ok = false;
    }
    switch (option) {
    case HM_OPT_OVERLAP: h->overlap = (int)value; break;
    case HM_OPT_TENSOR_CORES: h->tensor_cores = value != 0; break;
    case HM_OPT_NEAR_KERNEL: h->near_kernel = (int)value; break;
    case HM_OPT_NEAR_STAGES: h->near_stages = (int)value; break;
    case HM_OPT_PDL: h->pdl = value != 0 ? 1 : 0; break;
    case HM_OPT_RING_TILE: h->ring_tile = (int)value; break;
    default: break;
    }
    return HM_OK;
}

int hm_profile(hm_handle *h, int stage_mask)
{
    if (!h) return HM_ERR_INVALID_ARG;
    h->profile_mask = (unsigned)stage_mask & ((1u << HM_NSTAGES) - 1);
    return HM_OK;
}

int hm_profile_read(hm_handle *h, double *ms, int64_t *launches, int n, int reset)
{
    if (!h) return HM_ERR_INVALID_ARG;
    for (auto &e : h->events) {
        HM_CK(cudaEventSynchronize(e.b));
        float t = 0.f;
        HM_CK(cudaEventElapsedTime(&t, e.a, e.b));
        h->stage_ms[e.stage] += t;
        h->stage_launches[e.stage] += 1;
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    h->events.clear();
    for (int i = 0; i < n && i < HM_NSTAGES; ++i) {
        if (ms) ms[i] = h->stage_ms[i];
        if (launches) launches[i] = h->stage_launches[i];
    }
    if (reset)
        for (int i = 0; i < HM_NSTAGES; ++i) { h->stage_ms[i] = 0; h->stage_launches[i] = 0; }
    return HM_OK;
}

int hm_profile_timeline(hm_handle *h, double *out, int nmax)
{
    if (!h || (nmax > 0 && !out)) return HM_ERR_INVALID_ARG;
    // the earliest start among the pending events is the origin
    int first = -1;
    float best = 0.f;
    for (size_t i = 0; i < h->events.size(); ++i) {
        HM_CK(cudaEventSynchronize(h->events[i].b));
        if (first < 0) { first = (int)i; continue; }
        float t = 0.f;
        HM_CK(cudaEventElapsedTime(&t, h->events[first].a, h->events[i].a));
        if (t < best) best = t;
    }
    int n = 0;
    for (auto &e : h->events) {
        float t0 = 0.f, t1 = 0.f, d = 0.f;
        HM_CK(cudaEventElapsedTime(&t0, h->events[first].a, e.a));
        HM_CK(cudaEventElapsedTime(&t1, h->events[first].a, e.b));
        HM_CK(cudaEventElapsedTime(&d, e.a, e.b));
        if (n < nmax) {
            out[3 * n] = e.stage;
            out[3 * n + 1] = t0 - best;
            out[3 * n + 2] = t1 - best;
        }
        ++n;
        h->stage_ms[e.stage] += d;
        h->stage_launches[e.stage] += 1;
    }
    for (auto &e : h->events) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    h->events.clear();
    return n;
}

void hm_free(hm_handle *h)
{
    if (!h) return;
    cudaDeviceSynchronize();
    if (h->trans) hm_free(h->trans);
    for (auto &kv : h->streams) {
        if (kv.second.p) cudaFree(kv.second.p);
        if (kv.second.side) cudaStreamDestroy(kv.second.side);
        if (kv.second.fork) cudaEventDestroy(kv.second.fork);
        if (kv.second.join) cudaEventDestroy(kv.second.join);
        if (kv.second.mid) cudaEventDestroy(kv.second.mid);
    }
    if (h->host_graph.exec) cudaGraphExecDestroy(h->host_graph.exec);
    for (auto &e : h->events) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    if (h->d_stage) cudaFree(h->d_stage);
    if (h->host_stream) cudaStreamDestroy(h->host_stream);
    for (void *p : h->allocs) cudaFree(p);
    delete h;
}

}  // extern "C"
