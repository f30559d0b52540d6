// Low-rank arithmetic, dense block updates, Cholesky factors of dense blocks
// and the transposed block triangular solve (src/LowRankMatrix.jl:70-171,
// src/algebra.jl:394-524, src/hierarchical.jl:174-231, src/cholesky.jl) as
// batched GPU calls.  The recursion over blocks (which block meets which, in
// the reference's order) runs on the host in hierarchicalmatrices/algebra.py;
// the arithmetic of every block runs here, one CTA per block problem.
//
// Truncated SVD of P M Q^T (hm_lr_svd): Householder QR of the tall factors in
// a global workspace (L2-resident; one warp computes each reflector, every
// warp then updates the columns it owns), the small core R_P M R_Q^T formed
// in shared memory, a one-sided (Hestenes) Jacobi SVD of the core in shared
// memory with round-robin column pairs (one warp per pair), singular values
// sorted descending, getrank truncation, and the outputs Q_P W and Q_Q Z
// formed by applying the reflectors to the kept singular vectors.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <cmath>
#include <vector>

#include "hm_kernels.cuh"
#include "hmgpu.h"

namespace hm {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kJacobiSweeps = 40;
constexpr int kTkChunk = 128;       // coefficients per warp of a low-rank solve update
constexpr int kInvMax = 256;        // largest block of an HM_SOLVE_INV or HM_SOLVE_LTRSM op
constexpr int kLtrsmSmem = 64;      // HM_SOLVE_LTRSM blocks up to this size are staged in shared memory

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Julia's eps(x) for x >= 0: the distance from x to the next larger value of T.
__device__ __forceinline__ double ulp_of(double x)
{
    if (!(x >= 2.2250738585072014e-308)) return 4.9406564584124654e-324;
    int e;
    frexp(x, &e);                   // x = f 2^e, f in [0.5, 1)
    return ldexp(1.0, e - 53);
}
__device__ __forceinline__ float ulp_of(float x)
{
    if (!(x >= 1.17549435e-38f)) return 1.40129846e-45f;
    int e;
    frexpf(x, &e);
    return ldexpf(1.0f, e - 24);
}

template <typename T> struct Lim;
template <> struct Lim<double> { static constexpr double eps = 2.220446049250313e-16; static constexpr double big = 1e150; };
template <> struct Lim<float> { static constexpr float eps = 1.1920929e-7f; static constexpr float big = 1e18f; };

template <typename T>
__device__ __forceinline__ const T *stack_col(const void *X1, int64_t ld1, int k1, const void *X2, int64_t ld2, int l)
{
    return l < k1 ? static_cast<const T *>(X1) + ld1 * l : static_cast<const T *>(X2) + ld2 * (l - k1);
}

// Householder QR of the m x k panel A (ld m) in place, LAPACK xGEQR2
// conventions: H_j = I - tau_j v v^T with v_j = 1 and v below the diagonal of
// column j, beta = -sign(alpha) ||(alpha, x)||, R in the upper triangle.
template <typename T>
__device__ void house_qr(T *A, int64_t m, int k, T *tau)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int kk = (int)(m < k ? m : k);
    for (int j = 0; j < kk; ++j) {
        T *x = A + m * j;
        if (warp == j % kWarps) {
            T ss = 0;
            for (int64_t i = j + 1 + lane; i < m; i += 32) ss = fma(x[i], x[i], ss);
            ss = warp_sum(ss);
            const T alpha = x[j];
            T t = 0;
            if (ss != T(0)) {
                const T beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
                t = (beta - alpha) / beta;
                const T sc = T(1) / (alpha - beta);
                for (int64_t i = j + 1 + lane; i < m; i += 32) x[i] *= sc;
                __syncwarp();
                if (lane == 0) x[j] = beta;
            }
            if (lane == 0) tau[j] = t;
        }
        __syncthreads();
        const T tj = tau[j];
        if (tj != T(0)) {
            for (int c = warp; c < k; c += kWarps) {
                if (c <= j) continue;
                T *y = A + m * c;
                const T yj = y[j];
                T w = 0;
                for (int64_t i = j + 1 + lane; i < m; i += 32) w = fma(x[i], y[i], w);
                w = tj * (warp_sum(w) + yj);
                __syncwarp();
                if (lane == 0) y[j] = yj - w;
                for (int64_t i = j + 1 + lane; i < m; i += 32) y[i] = fma(-w, x[i], y[i]);
            }
        }
        __syncthreads();
    }
}

// y <- Q y = H_0 H_1 ... H_{kk-1} y for one column y (length m) by one warp.
template <typename T>
__device__ void apply_q(const T *A, int64_t m, int kk, const T *tau, T *y)
{
    const int lane = threadIdx.x & 31;
    for (int j = kk - 1; j >= 0; --j) {
        const T tj = tau[j];
        if (tj == T(0)) continue;
        const T *x = A + m * j;
        const T yj = y[j];
        T w = 0;
        for (int64_t i = j + 1 + lane; i < m; i += 32) w = fma(x[i], y[i], w);
        w = tj * (warp_sum(w) + yj);
        __syncwarp();
        if (lane == 0) y[j] = yj - w;
        for (int64_t i = j + 1 + lane; i < m; i += 32) y[i] = fma(-w, x[i], y[i]);
        __syncwarp();
    }
}

// The Jacobi rotation of lr_svd: t = tan(theta) is the smaller root of
// t^2 + 2 zeta t - 1 = 0, zeta = (be - al) / (2 ga), i.e.
// |t| = |g| / (|a| + sqrt(a^2 + g^2)) with a = be - al, g = 2 ga and the sign
// of a g.  t is formed in FP32 (FP64 issue time is scarce on GB300): from a
// and g scaled by a common power of two when |g| >= 2^-30 |a|, else as
// t = g / (2a) from the two mantissas with the exponents applied apart
// (strongly graded columns give angles far below FP32's range).  Its
// relative error, about 1e-7, only leaves an inner product of that relative
// size for the next sweep.  c = (1 + t^2)^(-1/2) is then refined in T from
// the FP32 estimate, so c^2 + s^2 = 1 to T's rounding and
// every rotation is orthogonal in T (c by one Halley step from the FP32
// estimate).  Returns false when t underflows.
__device__ __forceinline__ int exponent_of(double x) { return ((__double2hiint(x) >> 20) & 0x7ff) - 1023; }
__device__ __forceinline__ int exponent_of(float x) { return ((__float_as_int(x) >> 23) & 0xff) - 127; }
template <typename T> __device__ __forceinline__ T pow2(int e);
template <> __device__ __forceinline__ double pow2<double>(int e)
{
    e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
    return __hiloint2double((1023 + e) << 20, 0);
}
template <> __device__ __forceinline__ float pow2<float>(int e)
{
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((127 + e) << 23);
}

template <typename T>
__device__ __forceinline__ bool jacobi_tangent(T al, T be, T ga, T &t)
{
    const T a = be - al, g = ga + ga;
    const int ea = a == T(0) ? -100000 : exponent_of(a), eg = exponent_of(g);
    if (eg < ea - 30) {
        const float am = (float)(a * pow2<T>(-ea)), gm = (float)(g * pow2<T>(-eg));
        if (eg - ea < (sizeof(T) == 8 ? -1000 : -120)) return false;     // t below T's normal range
        t = (T)(gm / (am + am)) * pow2<T>(eg - ea);
    } else {
        const int e = ea > eg ? ea : eg;
        const T sc = pow2<T>(-e);
        const float af = (float)(a * sc), gf = (float)(g * sc);
        float t32 = fabsf(gf) / (fabsf(af) + sqrtf(fmaf(af, af, gf * gf)));
        if ((af < 0.f) != (gf < 0.f)) t32 = -t32;
        t = (T)t32;
    }
    return t != T(0);
}

// d^(-1/2) for d > 0 from the FP32 estimate refined by Halley's iteration;
// d outside FP32's range is first scaled to m in [1, 4) by an even power of
// two.  (Subnormal d: the library square root.)
__device__ __forceinline__ double rsqrt_halley(double d, double y0)
{
    // one step of Halley's iteration for d^(-1/2): with e = 1 - d y0^2,
    // y = y0 (1 + e/2 + 3e^2/8) leaves 5e^3/16, below double rounding for
    // the 2^-23 of an FP32 estimate; four dependent FP64 operations
    const double e = fma(-d, y0 * y0, 1.0);
    return fma(y0 * e, fma(0.375, e, 0.5), y0);
}
__device__ __forceinline__ double rsqrt_pos(double d)
{
    if (d > 1e-30 && d < 1e30) return rsqrt_halley(d, (double)rsqrtf((float)d));
    if (d < 1e-300) return 1.0 / sqrt(d);
    int e = exponent_of(d);
    e -= e & 1;
    const double m = d * pow2<double>(-e);
    return rsqrt_halley(m, (double)rsqrtf((float)m)) * pow2<double>(-e / 2);
}
__device__ __forceinline__ float rsqrt_pos(float d)
{
    if (d < 1e-36f) return 1.f / sqrtf(d);
    const float y = rsqrtf(d);
    return y * fmaf(-0.5f * d, y * y, 1.5f);
}

template <typename T>
__device__ __forceinline__ bool jacobi_rotation(T al, T be, T ga, T &c, T &s)
{
    T t;
    if (!jacobi_tangent(al, be, ga, t)) return false;
    const float tf = (float)t;
    const T u = fma(t, t, T(1));
    const T c0 = (T)rsqrtf(fmaf(tf, tf, 1.f));
    T cc;
    if constexpr (sizeof(T) == 8) {
        cc = rsqrt_halley(u, c0);
    } else {
        cc = c0 * fmaf(-0.5f * u, c0 * c0, 1.5f);
    }
    c = cc;
    s = cc * t;
    return true;
}

// One problem of lr_svd as the kernel reads it: the public descriptor and,
// for the hierarchical Cholesky's A22 - R12'R12 updates, an optional full
// middle block for part 2: M = diag(s1 ; sign2 * M2) with M2 a2 x a2 (ld
// ldm2) in place of diag(s2) (then a1 == b1, a2 == b2 and both factors are
// orthonormalised).  M2 = R12'R12 lets that update skip the separate
// truncated SVD of R12'R12: its truncation would drop only singular values
// below q eps(sigma_1), and the update's own SVD truncates the sum.
struct LrJob {
    hm_lr_problem p;
    const void *M2;
    int64_t ldm2;
};

// Core storage of lr_svd: D (p x q core, ld p), then J (q x q right
// rotations, before that the staging area of the Xm^T Ym product), sigma (q)
// and the sort order (q ints).  In shared memory (D takes d_elems values)
// when core_off < 0, else at ws + core_off for cores too large for it.
template <typename T>
__global__ void __launch_bounds__(kThreads) lr_svd_kernel(const LrJob *jobs, const int64_t *ws_off,
                                                          const int64_t *core_off, T *ws, int *ranks, int64_t d_elems,
                                                          int64_t xoff)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const hm_lr_problem pr = jobs[blockIdx.x].p;
    const T *M2 = static_cast<const T *>(jobs[blockIdx.x].M2);
    const int64_t ldm2 = jobs[blockIdx.x].ldm2;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int a = pr.a1 + pr.a2, b = pr.b1 + pr.b2;
    const int64_t m = pr.m, n = pr.n;
    const int ka = pr.qr_left ? (int)(m < a ? m : a) : a;
    const int kb = pr.qr_right ? (int)(n < b ? n : b) : b;
    const bool tr = kb > ka;
    const int p = tr ? kb : ka, q = tr ? ka : kb;
    __shared__ int s_flag, s_rank;
    __shared__ T s_scale, s_unscale;
    if (q == 0) {
        if (tid == 0) ranks[blockIdx.x] = 0;
        return;
    }
    T *WP = ws + ws_off[blockIdx.x];
    T *WQ = WP + (pr.qr_left ? m * a : 0);
    T *tauP = WQ + (pr.qr_right ? n * b : 0);
    T *tauQ = tauP + a;
    const int64_t co = core_off[blockIdx.x];
    T *D = co < 0 ? reinterpret_cast<T *>(smem_raw) : ws + co;
    T *J = D + (co < 0 ? d_elems : (int64_t)p * q);

    // 1. orthonormalise the factors that the operation orthonormalises
    if (pr.qr_left) {
        for (int64_t e = tid; e < m * a; e += kThreads) {
            const int l = (int)(e / m);
            WP[e] = stack_col<T>(pr.P1, pr.ldp1, pr.a1, pr.P2, pr.ldp2, l)[e - m * l];
        }
        __syncthreads();
        house_qr(WP, m, a, tauP);
    }
    if (pr.qr_right) {
        for (int64_t e = tid; e < n * b; e += kThreads) {
            const int l = (int)(e / n);
            WQ[e] = stack_col<T>(pr.Q1, pr.ldq1, pr.b1, pr.Q2, pr.ldq2, l)[e - n * l];
        }
        __syncthreads();
        house_qr(WQ, n, b, tauQ);
    }

    // 2. the core C (ka x kb), stored as D = C (p = ka) or D = C^T (p = kb)
    auto didx = [&](int i, int j) -> int64_t { return tr ? (int64_t)j + (int64_t)p * i : (int64_t)i + (int64_t)p * j; };
    if (pr.Xm) {
        // M = diag(s1) Xm^T Ym diag(s2), a x b, staged 32 rows of Xm and Ym at a time in J
        const T *Xm = static_cast<const T *>(pr.Xm), *Ym = static_cast<const T *>(pr.Ym);
        for (int e = tid; e < a * b; e += kThreads) D[didx(e % a, e / a)] = 0;
        T *Xs = J, *Ys = J + 32 * a;
        for (int64_t t0 = 0; t0 < pr.t; t0 += 32) {
            __syncthreads();
            for (int e = tid; e < 32 * a; e += kThreads) {
                const int r = e & 31, c = e >> 5;
                Xs[e] = t0 + r < pr.t ? Xm[(t0 + r) + pr.ldx * c] : T(0);
            }
            for (int e = tid; e < 32 * b; e += kThreads) {
                const int r = e & 31, c = e >> 5;
                Ys[e] = t0 + r < pr.t ? Ym[(t0 + r) + pr.ldy * c] : T(0);
            }
            __syncthreads();
            for (int e = tid; e < a * b; e += kThreads) {
                const int i = e % a, j = e / a;
                T acc = 0;
#pragma unroll 8
                for (int r = 0; r < 32; ++r) acc = fma(Xs[r + 32 * i], Ys[r + 32 * j], acc);
                D[didx(i, j)] += acc;
            }
        }
        __syncthreads();
        const T *s1 = static_cast<const T *>(pr.s1), *s2 = static_cast<const T *>(pr.s2);
        for (int e = tid; e < a * b; e += kThreads) {
            const int i = e % a, j = e / a;
            D[didx(i, j)] *= s1[i] * s2[j];
        }
    } else if (M2) {
        // C = R_P diag(s1 ; sign2 M2) R_Q^T: first Tm = R_P M (ka x b) in J's area
        const T *s1 = static_cast<const T *>(pr.s1);
        const T sign2 = (T)pr.sign2;
        T *Tm = J;
        for (int e = tid; e < ka * b; e += kThreads) {
            const int i = e % ka, l2 = e / ka;
            T acc = 0;
            if (l2 < pr.a1) {
                if (l2 >= i) acc = WP[i + m * l2] * s1[l2];
            } else {
                for (int l = i > pr.a1 ? i : pr.a1; l < a; ++l)
                    acc = fma(WP[i + m * l], M2[(l - pr.a1) + ldm2 * (l2 - pr.a1)], acc);
                acc *= sign2;
            }
            Tm[e] = acc;
        }
        __syncthreads();
        for (int e = tid; e < ka * kb; e += kThreads) {
            const int i = e % ka, j = e / ka;
            T acc = 0;
            for (int l2 = j; l2 < b; ++l2) acc = fma(Tm[i + ka * l2], WQ[j + n * l2], acc);
            D[didx(i, j)] = acc;
        }
        __syncthreads();                                   // Tm is read before J is written
    } else {
        // C = L diag(sd) R^T with L = R_P (ka x a) or I, R = R_Q (kb x b) or I
        const T *s1 = static_cast<const T *>(pr.s1), *s2 = static_cast<const T *>(pr.s2);
        const T sign2 = (T)pr.sign2;
        for (int e = tid; e < ka * kb; e += kThreads) {
            const int i = e % ka, j = e / ka;
            T acc = 0;
            if (!pr.qr_left && !pr.qr_right) {
                if (i == j) acc = i < pr.a1 ? s1[i] : sign2 * s2[i - pr.a1];
            } else if (!pr.qr_left) {                  // C(i, j) = sd_i R_Q(j, i)
                if (i >= j) acc = (i < pr.a1 ? s1[i] : sign2 * s2[i - pr.a1]) * WQ[j + n * i];
            } else if (!pr.qr_right) {                 // C(i, j) = R_P(i, j) sd_j
                if (j >= i) acc = WP[i + m * j] * (j < pr.a1 ? s1[j] : sign2 * s2[j - pr.a1]);
            } else {
                for (int l = i > j ? i : j; l < a; ++l) {
                    const T sd = l < pr.a1 ? s1[l] : sign2 * s2[l - pr.a1];
                    acc = fma(WP[i + m * l] * sd, WQ[j + n * l], acc);
                }
            }
            D[didx(i, j)] = acc;
        }
    }
    for (int e = tid; e < q * q; e += kThreads) J[e] = (e % q == e / q) ? T(1) : T(0);
    __syncthreads();

    // 3. one-sided Jacobi on the columns of D (p x q, q <= p).  D is first
    //    scaled by a power of two to max |D| in [0.5, 1) (exact; the singular
    //    values are scaled back in step 4), so that the squared column norms
    //    of the convergence test neither overflow nor underflow early.  A
    //    group of G lanes takes one column pair (rows strided by G), so that
    //    small cores keep every lane of a warp busy: on GB300 an FP64 warp
    //    instruction costs the same issue time with 1 or 32 lanes active.
    {
        T mx = 0;
        for (int64_t e = tid; e < (int64_t)p * q; e += kThreads) mx = fmax(mx, fabs(D[e]));
#pragma unroll
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        __shared__ T s_red[kWarps];
        if (lane == 0) s_red[warp] = mx;
        __syncthreads();
        if (tid == 0) {
            T m = 0;
            for (int w = 0; w < kWarps; ++w) m = fmax(m, s_red[w]);
            int ex = 0;
            if (m > T(0) && isfinite(m)) frexp(m, &ex);
            s_scale = ldexp(T(1), -ex);
            s_unscale = ldexp(T(1), ex);
        }
        __syncthreads();
        const T sc = s_scale;
        if (sc != T(1))
            for (int64_t e = tid; e < (int64_t)p * q; e += kThreads) D[e] *= sc;
        __syncthreads();
    }
    // QR preconditioning (cores in shared memory, q >= 4, formed from QR'd
    // factors): D = Q R, and the Jacobi sweeps run on X = R^T, whose columns
    // are far closer to orthogonal for the graded spectra of low-rank sums
    // (about half the sweeps); then D = (Q J) Sigma U_x^T with X J = U_x Sigma.
    // The Xm^T Ym cores of L1' * L2 gain fewer sweeps than the QR costs.
    const bool pre = co < 0 && xoff >= 0 && q >= 4 && !pr.Xm;
    T *Xs = nullptr, *Lf = nullptr, *tq = nullptr;
    if (pre) {
        Xs = reinterpret_cast<T *>(smem_raw) + xoff;   // q x q
        Lf = Xs + (int64_t)q * q;                      // p x q
        tq = Lf + (int64_t)p * q;                      // q
        house_qr(D, (int64_t)p, q, tq);
        for (int e = tid; e < q * q; e += kThreads) {
            const int i = e % q, j = e / q;
            Xs[e] = i >= j ? D[j + (int64_t)p * i] : T(0);
        }
        __syncthreads();
    }
    T *const Dj = pre ? Xs : D;
    const int pj = pre ? q : p;
    const int qq = (q + 1) & ~1, npairs = qq / 2;
    const int G = pj <= 32 ? 8 : (pj <= 64 ? 16 : 32);
    const int gpw = 32 / G, lg = lane & (G - 1), grp = lane / G;
    const T eps2 = Lim<T>::eps * Lim<T>::eps;
    for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
        if (tid == 0) s_flag = 0;
        __syncthreads();
        for (int round = 0; round < qq - 1; ++round) {
            for (int pb = warp * gpw; pb < npairs; pb += kWarps * gpw) {     // warp-uniform
                const int pi = pb + grp;
                int i = 0, j = q;
                if (pi < npairs) {
                    if (pi == 0) { i = round; j = qq - 1; }
                    else { i = (round + pi) % (qq - 1); j = (round - pi + qq - 1) % (qq - 1); }
                    if (i > j) { const int tmp = i; i = j; j = tmp; }
                }
                const bool live = j < q;
                T *di = Dj + (int64_t)pj * i, *dj = Dj + (int64_t)pj * (live ? j : i);
                T al = 0, be = 0, ga = 0;
                if (live)
                    for (int r = lg; r < pj; r += G) {
                        const T u = di[r], v = dj[r];
                        al = fma(u, u, al); be = fma(v, v, be); ga = fma(u, v, ga);
                    }
                for (int o = G >> 1; o; o >>= 1) {              // within the aligned group of G lanes
                    al += __shfl_xor_sync(0xffffffffu, al, o);
                    be += __shfl_xor_sync(0xffffffffu, be, o);
                    ga += __shfl_xor_sync(0xffffffffu, ga, o);
                }
                if (!live || al == T(0) || be == T(0) || !(ga * ga > eps2 * al * be)) continue;
                T c, sn;
                if (!jacobi_rotation(al, be, ga, c, sn)) continue;
                for (int r = lg; r < pj; r += G) {
                    const T u = di[r], v = dj[r];
                    di[r] = c * u - sn * v;
                    dj[r] = sn * u + c * v;
                }
                T *ji = J + (int64_t)q * i, *jj = J + (int64_t)q * j;
                for (int r = lg; r < q; r += G) {
                    const T u = ji[r], v = jj[r];
                    ji[r] = c * u - sn * v;
                    jj[r] = sn * u + c * v;
                }
                if (lg == 0) s_flag = 1;
            }
            __syncthreads();
        }
        const int any = s_flag;
        __syncthreads();
        if (!any) break;
    }
    if (pre) {
        // D's columns become Q [J_j; 0] sigma_j (sigma_j = |X_j|) and J's X_j / sigma_j,
        // the form the unpreconditioned sweeps leave
        for (int j = warp; j < q; j += kWarps) {
            const T *xj = Xs + (int64_t)q * j;
            T ss = 0;
            for (int r = lane; r < q; r += 32) ss = fma(xj[r], xj[r], ss);
            const T sgm = sqrt(warp_sum(ss));
            T *y = Lf + (int64_t)p * j;
            T *jc = J + (int64_t)q * j;
            for (int i = lane; i < p; i += 32) y[i] = i < q ? jc[i] : T(0);
            __syncwarp();
            apply_q(D, (int64_t)p, q, tq, y);
            for (int i = lane; i < p; i += 32) y[i] *= sgm;
            const T inv = sgm > T(0) ? T(1) / sgm : T(0);
            for (int r = lane; r < q; r += 32) jc[r] = sgm > T(0) ? xj[r] * inv : (r == j ? T(1) : T(0));
        }
        __syncthreads();
        for (int e = tid; e < p * q; e += kThreads) D[e] = Lf[e];
        __syncthreads();
    }

    // 4. singular values, descending order, getrank
    T *sig = J + (int64_t)q * q;
    int *perm = reinterpret_cast<int *>(sig + q);
    for (int j = warp; j < q; j += kWarps) {
        T *dj = D + (int64_t)p * j, *jj = J + (int64_t)q * j;
        T ss = 0, sj = 0;
        for (int r = lane; r < p; r += 32) ss = fma(dj[r], dj[r], ss);
        for (int r = lane; r < q; r += 32) sj = fma(jj[r], jj[r], sj);
        const T sv = sqrt(warp_sum(ss)), nj = sqrt(warp_sum(sj));
        if (sv > T(0)) {
            const T inv = T(1) / sv;
            for (int r = lane; r < p; r += 32) dj[r] *= inv;
        }
        const T invj = T(1) / nj;
        for (int r = lane; r < q; r += 32) jj[r] *= invj;
        if (lane == 0) sig[j] = sv * invj * s_unscale;
    }
    __syncthreads();
    // descending order, ties by index; a NaN ranks below everything (its key
    // is -1), so that perm is a permutation whatever the values
    for (int j = tid; j < q; j += kThreads) {
        int pos = 0;
        const T sj = sig[j] == sig[j] ? sig[j] : T(-1);
        for (int l = 0; l < q; ++l) {
            const T sl = sig[l] == sig[l] ? sig[l] : T(-1);
            pos += (sl > sj) || (sl == sj && l < j);
        }
        perm[pos] = j;
    }
    __syncthreads();
    if (tid == 0) {
        const T tol = (T)q * ulp_of(sig[perm[0]]);
        int r = q;
        while (r >= 1 && !(sig[perm[r - 1]] > tol)) --r;
        s_rank = r;
        ranks[blockIdx.x] = r;
    }
    __syncthreads();
    const int rk = s_rank;

    // 5. outputs: U = (Q_P or P) W, V = (Q_Q or Q) Z for the kept columns
    T *U = static_cast<T *>(pr.U), *V = static_cast<T *>(pr.V), *so = static_cast<T *>(pr.s);
    for (int k = warp; k < rk; k += kWarps) {
        const int j = perm[k];
        const T *wv = tr ? J + (int64_t)q * j : D + (int64_t)p * j;     // length ka
        const T *zv = tr ? D + (int64_t)p * j : J + (int64_t)q * j;     // length kb
        T *u = U + m * k;
        if (pr.qr_left) {
            for (int64_t i = lane; i < m; i += 32) u[i] = i < ka ? wv[i] : T(0);
            __syncwarp();
            apply_q(WP, m, ka, tauP, u);
        } else {
            for (int64_t i = lane; i < m; i += 32) {
                T acc = 0;
                for (int l = 0; l < a; ++l)
                    acc = fma(stack_col<T>(pr.P1, pr.ldp1, pr.a1, pr.P2, pr.ldp2, l)[i], wv[l], acc);
                u[i] = acc;
            }
        }
        T *v = V + n * k;
        if (pr.qr_right) {
            for (int64_t i = lane; i < n; i += 32) v[i] = i < kb ? zv[i] : T(0);
            __syncwarp();
            apply_q(WQ, n, kb, tauQ, v);
        } else if (!pr.Q1) {
            for (int64_t i = lane; i < n; i += 32) v[i] = zv[i];
        } else {
            for (int64_t i = lane; i < n; i += 32) {
                T acc = 0;
                for (int l = 0; l < b; ++l)
                    acc = fma(stack_col<T>(pr.Q1, pr.ldq1, pr.b1, pr.Q2, pr.ldq2, l)[i], zv[l], acc);
                v[i] = acc;
            }
        }
        if (lane == 0) so[k] = sig[j];
    }
}

// D = beta D + alpha P diag(s) Q^T, 64 x 64 output tiles; the tile list of
// all problems is one grid (tile0: first tile of each problem).  Thread
// (tx, ty) of a 16 x 16 block owns rows tx + 16u and columns ty + 16v.
template <typename T>
__global__ void __launch_bounds__(256) gemm_batched(const hm_gemm_problem *probs, const int64_t *tile0, int nprob)
{
    __shared__ T Ps[16][64], Qs[16][64];
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tile0[mid] <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const hm_gemm_problem g = probs[lo];
    const int64_t tm = (g.m + 63) / 64;
    const int64_t tl = (int64_t)blockIdx.x - tile0[lo];
    const int64_t i0 = (tl % tm) * 64, j0 = (tl / tm) * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const T *P = static_cast<const T *>(g.P), *Q = static_cast<const T *>(g.Q), *s = static_cast<const T *>(g.s);
    T acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0;
    for (int64_t k0 = 0; k0 < g.k; k0 += 16) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int idx = threadIdx.x + 256 * e;
            int kc, ii;
            if (!g.transp) { ii = idx & 63; kc = idx >> 6; } else { kc = idx & 15; ii = idx >> 4; }
            const int64_t gi = i0 + ii, gk = k0 + kc;
            T v = 0;
            if (gi < g.m && gk < g.k) v = g.transp ? P[gk + g.ldp * gi] : P[gi + g.ldp * gk];
            if (s && gk < g.k) v *= s[gk];
            Ps[kc][ii] = v;
            if (!g.transq) { ii = idx & 63; kc = idx >> 6; } else { kc = idx & 15; ii = idx >> 4; }
            const int64_t gj = j0 + ii, gk2 = k0 + kc;
            T w = 0;
            if (gj < g.n && gk2 < g.k) w = g.transq ? Q[gk2 + g.ldq * gj] : Q[gj + g.ldq * gk2];
            Qs[kc][ii] = w;
        }
        __syncthreads();
#pragma unroll
        for (int kc = 0; kc < 16; ++kc) {
            T pv[4], qv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) pv[u] = Ps[kc][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) qv[v] = Qs[kc][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(pv[u], qv[v], acc[u][v]);
        }
        __syncthreads();
    }
    T *Dm = static_cast<T *>(g.D);
    const T *Cm = g.C ? static_cast<const T *>(g.C) : Dm;
    const int64_t ldc = g.C ? g.ldc : g.ldd;
    const T alpha = (T)g.alpha, beta = (T)g.beta;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const int64_t j = j0 + ty + 16 * v;
        if (j >= g.n) continue;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + tx + 16 * u;
            if (i >= g.m) continue;
            const T add = alpha * acc[u][v];
            Dm[i + g.ldd * j] = beta == T(0) ? add : fma(beta, Cm[i + ldc * j], add);
        }
    }
}

template <typename T>
__global__ void axpby_batched(const hm_axpby_problem *probs)
{
    const hm_axpby_problem g = probs[blockIdx.y];
    const T *A = static_cast<const T *>(g.A), *B = static_cast<const T *>(g.B);
    const T *dr = static_cast<const T *>(g.dr), *dc = static_cast<const T *>(g.dc);
    T *Dm = static_cast<T *>(g.D);
    const T al = (T)g.alpha, be = (T)g.beta;
    const int64_t total = g.m * g.n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / g.m, i = e - j * g.m;
        T v = al * A[i + g.lda * j];
        if (dr) v *= dr[i];
        if (dc) v *= dc[j];
        Dm[i + g.ldd * j] = be == T(0) ? v : fma(be, B[i + g.ldb * j], v);
    }
}

// Right-looking upper Cholesky of one block per CTA: in shared memory when
// n <= nsmem, else in place in R.  Reads only A's upper triangle (the
// reference factors Symmetric(A), whose default view is the upper one).
template <typename T>
__global__ void __launch_bounds__(kThreads) potrf_batched(const hm_potrf_problem *probs, int *info, int64_t nsmem)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const hm_potrf_problem g = probs[blockIdx.x];
    const int64_t n = g.n;
    const bool in_smem = n <= nsmem;
    T *R = static_cast<T *>(g.R);
    T *S = in_smem ? reinterpret_cast<T *>(smem_raw) : R;
    const int64_t ld = in_smem ? n : g.ldr;
    const T *A = static_cast<const T *>(g.A);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ int s_fail;
    for (int64_t j = warp; j < n; j += kWarps)
        for (int64_t i = lane; i < n; i += 32) S[i + ld * j] = i <= j ? A[i + g.lda * j] : T(0);
    if (threadIdx.x == 0) s_fail = 0;
    __syncthreads();
    for (int64_t j = 0; j < n; ++j) {
        if (warp == 0) {                    // the pivot row, by one warp (FP64 issue time is scarce)
            const T d = S[j + ld * j];
            if (!(d > T(0))) {
                if (lane == 0) s_fail = (int)(j + 1);
            } else {
                const T y = rsqrt_pos(d);
                for (int64_t i = j + 1 + lane; i < n; i += 32) S[j + ld * i] *= y;
                if (lane == 0) S[j + ld * j] = d * y;
            }
        }
        __syncthreads();
        if (s_fail) break;
        for (int64_t l = j + 1 + warp; l < n; l += kWarps) {
            const T rl = S[j + ld * l];
            for (int64_t i = j + 1 + lane; i <= l; i += 32) S[i + ld * l] = fma(-S[j + ld * i], rl, S[i + ld * l]);
        }
        __syncthreads();
    }
    if (in_smem)
        for (int64_t j = warp; j < n; j += kWarps)
            for (int64_t i = lane; i < n; i += 32) R[i + g.ldr * j] = S[i + n * j];
    if (threadIdx.x == 0) info[blockIdx.x] = s_fail;
}

// x <- R^{-T} x for an upper triangular n x n block R by one warp (forward
// substitution).  Up to 256 unknowns stay in registers (lane l holds
// x[l + 32 t]) and the right-looking order is used: once x_i is final (its
// owner multiplies by the pivot's reciprocal, computed for all rows up front)
// it is broadcast by a shuffle and every lane subtracts R[i, l] x_i from the
// rows l > i it holds; each step is one shuffle and independent loads, with
// no reduction on the dependent path.  Larger blocks use column dot products.
template <typename T>
__device__ void trsm_t_warp(const T *R, int64_t ld, int64_t n, T *x)
{
    const int lane = threadIdx.x & 31;
    if (n <= 256) {
        T xr[8], rinv[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int64_t i = lane + 32 * t;
            xr[t] = i < n ? x[i] : T(0);
            rinv[t] = i < n ? T(1) / R[i + ld * i] : T(0);
        }
        for (int64_t i = 0; i < n; ++i) {
            const int owner = (int)(i & 31), ti = (int)(i >> 5);
            T xi = 0;
#pragma unroll
            for (int t = 0; t < 8; ++t)
                if (t == ti) xi = xr[t] * rinv[t];
            xi = __shfl_sync(0xffffffffu, xi, owner);
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int64_t l = lane + 32 * t;
                if (t == ti && lane == owner) xr[t] = xi;
                else if (l > i && l < n) xr[t] = fma(-R[i + ld * l], xi, xr[t]);
            }
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) { const int64_t i = lane + 32 * t; if (i < n) x[i] = xr[t]; }
    } else {
        for (int64_t i = 0; i < n; ++i) {
            const T *col = R + ld * i;
            T part = 0;
            for (int64_t l = lane; l < i; l += 32) part = fma(col[l], x[l], part);
            part = warp_sum(part);
            if (lane == 0) x[i] = (x[i] - part) / col[i];
            __syncwarp();
        }
    }
    __syncwarp();
}

// (i, j), i <= j, of the p-th entry of an upper triangle in column order
__device__ __forceinline__ void upper_pair(int p, int &i, int &j)
{
    int l = (int)((sqrtf(8.f * (float)p + 1.f) - 1.f) * 0.5f);
    while (l * (l + 1) / 2 > p) --l;
    while ((l + 1) * (l + 2) / 2 <= p) ++l;
    j = l;
    i = p - l * (l + 1) / 2;
}

// A dense diagonal leaf of the hierarchical Cholesky: R = chol(A) (the upper
// triangle of A read) and L = R^T, one CTA, in shared memory (ld n + 1).
// Right-looking with lookahead: warp 0 applies step j to row j + 1 and forms
// pivot j + 1 (a Halley reciprocal square root; the dependent FP64 chain is
// the kernel's critical path on GB300, 64 cycles per operation) while the
// other warps apply step j to the rows below, its entries spread evenly over
// them (an FP64 warp instruction costs the same with idle lanes); one barrier
// per step.  L is what the forward substitutions of the solves read (its
// columns contiguous).
struct LeafChol {
    int64_t n;
    const void *A; int64_t lda;
    void *R; int64_t ldr;
    void *L; int64_t ldl;
};
// largest leaf that leaf_chol keeps in shared memory
template <typename T>
int64_t leaf_chol_max()
{
    int64_t n = 0;
    while (((n + 1) * (n + 2) + (n + 1)) * (int64_t)sizeof(T) <= 200 * 1024) ++n;
    return n;
}
template <typename T>
__global__ void __launch_bounds__(kThreads) leaf_chol(const LeafChol *probs, int *info)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const LeafChol g = probs[blockIdx.x];
    const int n = (int)g.n, ls = n + 1, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T *S = reinterpret_cast<T *>(smem_raw);            // n x n, ld n + 1
    __shared__ int s_fail;
    const T *A = static_cast<const T *>(g.A);
    for (int e = tid; e < n * n; e += kThreads) {
        const int i = e % n, j = e / n;
        S[i + ls * j] = i <= j ? A[i + g.lda * j] : T(0);
    }
    if (tid == 0) s_fail = 0;
    __syncthreads();
    auto pivot = [&](int j) {
        const T d = S[j + ls * j];
        if (!(d > T(0))) {
            if (lane == 0) s_fail = j + 1;
            return;
        }
        const T y = rsqrt_pos(d);
        for (int l = j + 1 + lane; l < n; l += 32) S[j + ls * l] *= y;
        if (lane == 0) S[j + ls * j] = d * y;
    };
    if (warp == 0) pivot(0);
    __syncthreads();
    for (int j = 0; j < n && !s_fail; ++j) {
        if (warp == 0) {
            if (j + 1 < n) {
                const T a = S[j + ls * (j + 1)];
                for (int l = j + 1 + lane; l < n; l += 32) S[j + 1 + ls * l] = fma(-a, S[j + ls * l], S[j + 1 + ls * l]);
                __syncwarp();
                pivot(j + 1);
            }
        } else {
            const int m = n - j - 2, tj = m > 0 ? m * (m + 1) / 2 : 0;
            for (int p = tid - 32; p < tj; p += kThreads - 32) {
                int i, l;
                upper_pair(p, i, l);
                i += j + 2;
                l += j + 2;
                S[i + ls * l] = fma(-S[j + ls * i], S[j + ls * l], S[i + ls * l]);
            }
        }
        __syncthreads();
    }
    if (tid == 0) info[blockIdx.x] = s_fail;
    // R and L are written also after a failed pivot (the partial factor, as
    // potrf_batched leaves it): what follows reads finite values
    T *R = static_cast<T *>(g.R), *Lo = static_cast<T *>(g.L);
    for (int e = tid; e < n * n; e += kThreads) {
        const int i = e % n, j = e / n;
        R[i + g.ldr * j] = S[i + ls * j];
        Lo[i + g.ldl * j] = i >= j ? S[j + ls * i] : T(0);
    }
}

// H = diag(s) X^T X diag(s) for a tall X (rows x r, r <= kGramMax) by
// several CTAs: CTA c sums rows [c chunk, (c + 1) chunk) into its partial
// Gram matrix (ws + c r^2; thread e owns entries e, e + 256, ...; 32 rows of X
// staged in shared memory at a time); the last CTA to finish (a counter,
// reset by it for the next launch) adds the partials in CTA order, so the
// result does not depend on which CTA finishes last.
constexpr int kGramMax = 64;
template <typename T>
__global__ void __launch_bounds__(kThreads) hchol_gram(const T *X, int64_t ldx, int64_t rows, int r, const T *s,
                                                        T *ws, unsigned *counter, T *H, int64_t chunk)
{
    __shared__ T xs[kGramMax * 33];
    __shared__ bool last;
    const int tid = threadIdx.x, no = r * r;
    constexpr int kPer = kGramMax * kGramMax / kThreads;
    T acc[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) acc[u] = T(0);
    const int64_t r0 = (int64_t)blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
    for (int64_t b = r0; b < r1; b += 32) {
        const int nb = (int)(r1 - b < 32 ? r1 - b : 32);
        __syncthreads();
        for (int e = tid; e < 32 * r; e += kThreads) {
            const int c = e >> 5, i = e & 31;
            xs[c * 33 + i] = i < nb ? X[(b + i) + ldx * c] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int e = tid + kThreads * u;
            if (e < no) {
                const T *xi = xs + (e % r) * 33, *xj = xs + (e / r) * 33;
                T a = acc[u];
#pragma unroll 8
                for (int k = 0; k < 32; ++k) a = fma(xi[k], xj[k], a);
                acc[u] = a;
            }
        }
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
        const int e = tid + kThreads * u;
        if (e < no) ws[(int64_t)blockIdx.x * no + e] = acc[u];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int e = tid; e < no; e += kThreads) {
        T v = 0;
        for (unsigned c = 0; c < gridDim.x; ++c) v += __ldcg(ws + (int64_t)c * no + e);
        H[e] = s[e % r] * v * s[e / r];
    }
    if (tid == 0) *counter = 0u;
}

// Dense leaves of A22 - R12'R12: D_out = D_in - Vp H Vp^T on the upper
// triangle (the part the leaf's Cholesky reads), one CTA per leaf, Vp (n x r)
// and T = Vp H in shared memory.
struct LeafUpd {
    int64_t n;
    const void *Vp; int64_t ldv;
    const void *Din; int64_t ldi;
    void *Dout; int64_t ldo;
};
constexpr int kLeafUpdMax = 256;
template <typename T>
__global__ void __launch_bounds__(kThreads) hchol_leaf_update(const LeafUpd *ups, const T *H, int r)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const LeafUpd u = ups[blockIdx.x];
    const int n = (int)u.n, tid = threadIdx.x;
    T *Vs = reinterpret_cast<T *>(smem_raw);       // n x r
    T *Ts = Vs + (int64_t)n * r;                    // n x r
    T *Hs = Ts + (int64_t)n * r;                    // r x r
    const T *Vp = static_cast<const T *>(u.Vp);
    for (int e = tid; e < n * r; e += kThreads) Vs[e] = Vp[(e % n) + u.ldv * (e / n)];
    for (int e = tid; e < r * r; e += kThreads) Hs[e] = H[e];
    __syncthreads();
    for (int e = tid; e < n * r; e += kThreads) {
        const int i = e % n, k = e / n;
        T a = 0;
        for (int m = 0; m < r; ++m) a = fma(Vs[i + n * m], Hs[m + r * k], a);
        Ts[e] = a;
    }
    __syncthreads();
    const T *Din = static_cast<const T *>(u.Din);
    T *Dout = static_cast<T *>(u.Dout);
    const int npair = n * (n + 1) / 2;
    for (int e = tid; e < npair; e += kThreads) {
        // (i, l), i <= l, of the e-th upper entry in column order
        int l = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
        while (l * (l + 1) / 2 > e) --l;
        while ((l + 1) * (l + 2) / 2 <= e) ++l;
        const int i = e - l * (l + 1) / 2;
        T a = Din[i + u.ldi * l];
        for (int k = 0; k < r; ++k) a = fma(-Ts[i + n * k], Vs[l + n * k], a);
        Dout[i + u.ldo * l] = a;
    }
}

// x <- L^{-1} x for a lower triangular n x n block L (n <= 256) by one warp,
// right-looking: lane l holds x[l + 32 t]; once x_i is final (its owner
// multiplies by 1/L_ii, formed for all rows up front) a shuffle broadcasts it
// and every lane subtracts L[l, i] x_i from its rows l > i.  Column i of L is
// read contiguously (from shared memory when the caller staged L there) and
// the next column is loaded while the current one is applied.  Per step: one
// FP64 multiply, one shuffle and one FMA per 32 rows on the dependent path.
template <typename T>
__device__ void ltrsm_warp(const T *L, int64_t ld, int n, T *x)
{
    const int lane = threadIdx.x & 31, nt = (n + 31) >> 5;
    T xr[8], rinv[8], col[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int i = lane + 32 * t;
        xr[t] = t < nt && i < n ? x[i] : T(0);
        rinv[t] = t < nt && i < n ? T(1) / L[i + ld * i] : T(0);
        col[t] = t < nt && i > 0 && i < n ? L[i] : T(0);
    }
    for (int i = 0; i < n; ++i) {
        T nxt[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int row = lane + 32 * t;
            nxt[t] = t < nt && i + 1 < n && row > i + 1 && row < n ? L[row + ld * (i + 1)] : T(0);
        }
        const int owner = i & 31, ti = i >> 5;
        T xs = xr[0], rs = rinv[0];
#pragma unroll
        for (int t = 1; t < 8; ++t)
            if (t == ti) { xs = xr[t]; rs = rinv[t]; }
        const T xi = __shfl_sync(0xffffffffu, xs * rs, owner);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            if (t >= nt) break;
            const int row = lane + 32 * t;
            if (row == i) xr[t] = xi;
            else if (row > i) xr[t] = fma(-col[t], xi, xr[t]);
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) col[t] = nxt[t];
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int i = lane + 32 * t;
        if (t < nt && i < n) x[i] = xr[t];
    }
    __syncwarp();
}

// W = R^{-1} for upper triangular n x n blocks, one CTA per block, R staged in
// shared memory.  Column j of W is the back substitution R w = e_j, run by a
// group of four lanes (partial sums over k = i+1+q, i+5+q, ... reduced by two
// shuffles); warp w takes the columns w, w+8, w+16, ... so that the long
// columns are spread over all warps.  GB300's FP64 rate is low (about two
// FMAs per clock per SM), so the work is spread over every SM sub-partition.
template <typename T>
__global__ void __launch_bounds__(kThreads) trtri_batched(const hm_trtri_problem *probs, int64_t nmax)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const hm_trtri_problem g = probs[blockIdx.x];
    const int64_t n = g.n, ls = nmax + 1;
    T *Rs = reinterpret_cast<T *>(smem_raw);            // ls x n, padded
    T *Ws = Rs + ls * nmax;                              // ls x n, padded
    T *rinv = Ws + ls * nmax;                            // n
    const T *R = static_cast<const T *>(g.R);
    T *W = static_cast<T *>(g.W);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, q = lane & 3;
    for (int64_t k = warp; k < n; k += kWarps)
        for (int64_t i = lane; i < n; i += 32) Rs[i + ls * k] = i <= k ? R[i + g.ldr * k] : T(0);
    __syncthreads();
    for (int64_t i = tid; i < n; i += kThreads) rinv[i] = T(1) / Rs[i + ls * i];
    __syncthreads();
    // columns j = warp + 8 (g8 + 8 c), g8 = lane / 4 the lane group; the loop
    // bounds are the same for every lane of a warp, so the shuffles are uniform
    for (int64_t c = 0; c * 64 < n; ++c) {
        const int64_t j = warp + 8 * ((lane >> 2) + 8 * c);
        for (int64_t i = n - 1; i >= 0; --i) {
            T part = 0;
            if (j < n && i < j)
                for (int64_t k = i + 1 + q; k <= j; k += 4) part = fma(Rs[i + ls * k], Ws[k + ls * j], part);
            part += __shfl_xor_sync(0xffffffffu, part, 1);
            part += __shfl_xor_sync(0xffffffffu, part, 2);
            if (j < n && q == 0) Ws[i + ls * j] = i == j ? rinv[i] : i < j ? -part * rinv[i] : T(0);
            __syncwarp();
        }
    }
    __syncthreads();
    for (int64_t j = warp; j < n; j += kWarps)
        for (int64_t i = lane; i < n; i += 32) W[i + g.ldw * j] = Ws[i + ls * j];
}

// One CTA per column of B walks the whole schedule in order: a triangular
// block on warp 0, low-rank and dense updates on all warps (coefficients of a
// low-rank block one warp each, then the rows of x2 over all threads).
// Global writes of x are made visible to the CTA by the barrier after each op.
template <typename T>
__global__ void __launch_bounds__(kThreads) solve_schedule(const hm_solve_op *ops, int nops, T *B, int64_t ldb,
                                                           int64_t base)
{
    __shared__ T tk[kTkChunk];
    __shared__ T xs[kInvMax];
    __shared__ T ls[kLtrsmSmem * kLtrsmSmem];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T *const xb = B + ldb * (int64_t)blockIdx.x;
    auto xat = [&](int64_t o) { return xb + (o - base); };    // row o of the schedule is row o - base of B
    for (int o = 0; o < nops; ++o) {
        const hm_solve_op op = ops[o];
        const T *A = static_cast<const T *>(op.A);
        if (op.kind == HM_SOLVE_TRSM) {
            if (warp == 0) trsm_t_warp(A, op.ld, op.n1, xat(op.o1));
        } else if (op.kind == HM_SOLVE_LTRSM) {
            if (op.n1 <= kLtrsmSmem) {                  // L staged by all warps, then one warp substitutes
                for (int e = tid; e < op.n1 * op.n1; e += kThreads) {
                    const int i = e % (int)op.n1, j = e / (int)op.n1;
                    ls[i + kLtrsmSmem * j] = i >= j ? A[i + op.ld * j] : T(0);
                }
                __syncthreads();
                if (warp == 0) ltrsm_warp<T>(ls, kLtrsmSmem, (int)op.n1, xat(op.o1));
            } else if (warp == 0) {
                ltrsm_warp<T>(A, op.ld, (int)op.n1, xat(op.o1));
            }
        } else if (op.kind == HM_SOLVE_INV) {
            // x1 <- W^T x1, W = R^{-1} upper: four lanes per output, all warps
            T *x1 = xat(op.o1);
            for (int64_t i = tid; i < op.n1; i += kThreads) xs[i] = x1[i];
            __syncthreads();
            const int q = lane & 3;
            for (int64_t jb = 0; jb < op.n1; jb += kThreads / 4) {
                const int64_t j = jb + (tid >> 2);
                T part = 0;
                if (j < op.n1) {
                    const T *col = A + op.ld * j;
                    for (int64_t i = q; i <= j; i += 4) part = fma(col[i], xs[i], part);
                }
                part += __shfl_xor_sync(0xffffffffu, part, 1);
                part += __shfl_xor_sync(0xffffffffu, part, 2);
                if (j < op.n1 && q == 0) x1[j] = part;
            }
        } else if (op.kind == HM_SOLVE_LR) {
            const T *s = static_cast<const T *>(op.s), *V = static_cast<const T *>(op.B);
            const T *x1 = xat(op.o1);
            T *x2 = xat(op.o2);
            for (int k0 = 0; k0 < op.r; k0 += kTkChunk) {
                const int kn = op.r - k0 < kTkChunk ? op.r - k0 : kTkChunk;
                for (int k = warp; k < kn; k += kWarps) {
                    const T *u = A + op.ld * (k0 + k);
                    T part = 0;
                    for (int64_t i = lane; i < op.n1; i += 32) part = fma(u[i], x1[i], part);
                    part = warp_sum(part);
                    if (lane == 0) tk[k] = part * s[k0 + k];
                }
                __syncthreads();
                for (int64_t j = tid; j < op.n2; j += kThreads) {
                    T acc = 0;
                    for (int k = 0; k < kn; ++k) acc = fma(V[j + op.ld2 * (k0 + k)], tk[k], acc);
                    x2[j] -= acc;
                }
                __syncthreads();
            }
        } else {
            const T *x1 = xat(op.o1);
            for (int64_t j = warp; j < op.n2; j += kWarps) {
                const T *col = A + op.ld * j;
                T part = 0;
                for (int64_t i = lane; i < op.n1; i += 32) part = fma(col[i], x1[i], part);
                part = warp_sum(part);
                if (lane == 0) xat(op.o2)[j] -= part;
            }
        }
        __syncthreads();
    }
}

// ---- host side ---------------------------------------------------------------

int cuda_fail(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return HM_OK;
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? HM_ERR_ALLOC : HM_ERR_CUDA;
}

#define ALG_CK(call)                                          \
    do {                                                      \
        int st_ = cuda_fail((call), #call);                   \
        if (st_) return st_;                                  \
    } while (0)

#define ALG_TRY(call)                                         \
    do {                                                      \
        int st_ = (call);                                     \
        if (st_) return st_;                                  \
    } while (0)

// Device copies of host arrays for one call, freed stream-ordered.
struct Staged {
    std::vector<void *> ptrs;
    cudaStream_t st;
    explicit Staged(cudaStream_t s) : st(s) {}
    ~Staged() { for (void *p : ptrs) cudaFreeAsync(p, st); }
    template <typename T>
    int put(const T *host, size_t count, T **dev)
    {
        void *p = nullptr;
        ALG_CK(device_malloc_pooled(&p, std::max<size_t>(count, 1) * sizeof(T), st));
        ptrs.push_back(p);
        if (count) ALG_CK(cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, st));
        *dev = static_cast<T *>(p);
        return HM_OK;
    }
    template <typename T>
    int zeros(size_t count, T **dev)
    {
        void *p = nullptr;
        ALG_CK(device_malloc_pooled(&p, std::max<size_t>(count, 1) * sizeof(T), st));
        ptrs.push_back(p);
        *dev = static_cast<T *>(p);
        return HM_OK;
    }
};

template <typename K>
int set_smem(K kernel, size_t bytes)
{
    if (bytes <= 48 * 1024) return HM_OK;
    if (bytes > 227 * 1024) { set_last_error("kernel needs %zu bytes of shared memory", bytes); return HM_ERR_UNSUPPORTED; }
    ALG_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return HM_OK;
}

// Cores whose storage exceeds this many bytes run from the global workspace.
constexpr size_t kCoreSmemBytes = 200 * 1024;
// Cores whose storage with the QR preconditioner's fits in this many bytes
// are preconditioned.
constexpr size_t kPreconSmemBytes = 224 * 1024;

// Workspace layout and shared memory of one lr_svd launch.
struct LrPlan {
    std::vector<int64_t> off, coff;
    int64_t ws = 0, dmax = 1, xoff = -1;
    size_t smem = 0;
};

template <typename T>
int lr_svd_plan(int nprob, const LrJob *jobs, LrPlan &pl)
{
    pl.off.assign(nprob, 0);
    pl.coff.assign(nprob, -1);
    int64_t ws = 0, dmax = 1, jmax = 1, xmax = 0;
    int qmax = 1;
    for (int i = 0; i < nprob; ++i) {
        const hm_lr_problem &p = jobs[i].p;
        const bool full2 = jobs[i].M2 != nullptr;
        const int a = p.a1 + p.a2, b = p.b1 + p.b2;
        if (p.m < 0 || p.n < 0 || p.a1 < 0 || p.a2 < 0 || p.b1 < 0 || p.b2 < 0) {
            set_last_error("problem %d: negative size", i);
            return HM_ERR_INVALID_ARG;
        }
        if (p.Xm) {
            if (full2 || p.a2 || p.b2 || p.qr_left || p.qr_right || p.t < 0 || (p.t > 0 && !p.Ym) || (p.a1 && !p.s1) ||
                (p.b1 && !p.s2)) {
                set_last_error("problem %d: the Xm^T Ym core takes one part per side, no QR", i);
                return HM_ERR_INVALID_ARG;
            }
        } else if (a != b || (p.a1 && !p.s1) || (p.a2 && !p.s2 && !full2)) {
            set_last_error("problem %d: a diagonal middle needs a1 + a2 == b1 + b2 and its values", i);
            return HM_ERR_INVALID_ARG;
        }
        if (full2 && (p.a1 != p.b1 || !p.qr_left || !p.qr_right || jobs[i].ldm2 < p.a2)) {
            set_last_error("problem %d: a full middle block needs a1 == b1, both QRs and ldm2 >= a2", i);
            return HM_ERR_INVALID_ARG;
        }
        if (!p.Q1 && p.b1 && (p.n != p.b1 || p.b2 || p.qr_right)) {
            set_last_error("problem %d: an identity right factor needs n == b1, b2 == 0 and no QR", i);
            return HM_ERR_INVALID_ARG;
        }
        if ((p.a1 && !p.P1) || (p.a2 && !p.P2) || (p.b2 && !p.Q2)) {
            set_last_error("problem %d: NULL factor", i);
            return HM_ERR_INVALID_ARG;
        }
        const int64_t ka = p.qr_left ? std::min<int64_t>(p.m, a) : a;
        const int64_t kb = p.qr_right ? std::min<int64_t>(p.n, b) : b;
        if (ka > 4096 || kb > 4096 || (p.Xm && (a > 4096 || b > 4096))) {
            set_last_error("problem %d: core %lld x %lld exceeds 4096", i, (long long)ka, (long long)kb);
            return HM_ERR_UNSUPPORTED;
        }
        const int64_t q = std::min(ka, kb), pp = std::max(ka, kb);
        if (q > 0 && (!p.U || !p.s || !p.V)) { set_last_error("problem %d: NULL output", i); return HM_ERR_INVALID_ARG; }
        pl.off[i] = ws;
        ws += (p.qr_left ? p.m * a : 0) + (p.qr_right ? p.n * b : 0) + a + b;
        ws = (ws + 31) / 32 * 32;
        const int64_t jn = std::max({q * q, p.Xm ? (int64_t)32 * (a + b) : 0, full2 ? ka * b : 0});
        const size_t need = (size_t)(pp * q + jn + q) * sizeof(T) + (size_t)q * sizeof(int) + 64;
        if (need <= kCoreSmemBytes) {
            dmax = std::max(dmax, pp * q);
            jmax = std::max(jmax, jn);
            qmax = std::max<int>(qmax, (int)q);
            xmax = std::max(xmax, q * q + pp * q + q);
        } else {
            pl.coff[i] = ws;
            ws += pp * q + jn + 2 * q;          // sigma (q values) and the order (q ints) after J
            ws = (ws + 31) / 32 * 32;
        }
    }
    pl.ws = std::max<int64_t>(ws, 1);
    pl.dmax = dmax;
    // J also holds sigma (q values) and the sort order (q ints) after it; then,
    // when it fits, the QR preconditioner's area (R^T, Q J and the reflectors' tau)
    pl.smem = (size_t)(dmax + jmax + qmax) * sizeof(T) + (size_t)qmax * sizeof(int) + 64;
    const int64_t xoff = (int64_t)((pl.smem + sizeof(T) - 1) / sizeof(T));
    if (xmax > 0 && (size_t)(xoff + xmax) * sizeof(T) <= kPreconSmemBytes) {
        pl.xoff = xoff;
        pl.smem = (size_t)(xoff + xmax) * sizeof(T);
    }
    return set_smem(lr_svd_kernel<T>, pl.smem);
}

template <typename T>
int lr_svd_run(int nprob, const hm_lr_problem *probs, int32_t *ranks, cudaStream_t st)
{
    std::vector<LrJob> jobs(nprob);
    for (int i = 0; i < nprob; ++i) jobs[i] = LrJob{probs[i], nullptr, 0};
    LrPlan pl;
    ALG_TRY(lr_svd_plan<T>(nprob, jobs.data(), pl));
    if (nprob == 0) return HM_OK;
    Staged S(st);
    LrJob *d_jobs = nullptr;
    int64_t *d_off = nullptr, *d_coff = nullptr;
    T *d_ws = nullptr;
    int *d_ranks = nullptr;
    ALG_TRY(S.put(jobs.data(), (size_t)nprob, &d_jobs));
    ALG_TRY(S.put(pl.off.data(), pl.off.size(), &d_off));
    ALG_TRY(S.put(pl.coff.data(), pl.coff.size(), &d_coff));
    ALG_TRY(S.zeros((size_t)pl.ws, &d_ws));
    ALG_TRY(S.zeros((size_t)nprob, &d_ranks));
    lr_svd_kernel<T><<<nprob, kThreads, pl.smem, st>>>(d_jobs, d_off, d_coff, d_ws, d_ranks, pl.dmax, pl.xoff);
    ALG_CK(cudaGetLastError());
    std::vector<int> hr(nprob);
    ALG_CK(cudaMemcpyAsync(hr.data(), d_ranks, nprob * sizeof(int), cudaMemcpyDeviceToHost, st));
    ALG_CK(cudaStreamSynchronize(st));
    for (int i = 0; i < nprob; ++i) ranks[i] = hr[i];
    return HM_OK;
}

template <typename T, typename Stage>
int gemm_launch(int nprob, const hm_gemm_problem *probs, cudaStream_t st, Stage &S)
{
    std::vector<int64_t> tile0(nprob + 1, 0);
    for (int i = 0; i < nprob; ++i) {
        const hm_gemm_problem &g = probs[i];
        if (g.m < 0 || g.n < 0 || g.k < 0) { set_last_error("problem %d: negative size", i); return HM_ERR_INVALID_ARG; }
        if (g.m && g.n && (!g.D || (g.k && (!g.P || !g.Q)))) { set_last_error("problem %d: NULL operand", i); return HM_ERR_INVALID_ARG; }
        tile0[i + 1] = tile0[i] + ((g.m + 63) / 64) * ((g.n + 63) / 64);
    }
    const int64_t tiles = tile0[nprob];
    if (tiles == 0) return HM_OK;
    if (tiles > INT32_MAX) { set_last_error("too many output tiles"); return HM_ERR_UNSUPPORTED; }
    hm_gemm_problem *d_probs = nullptr;
    int64_t *d_tile0 = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    ALG_TRY(S.put(tile0.data(), tile0.size(), &d_tile0));
    gemm_batched<T><<<(unsigned)tiles, 256, 0, st>>>(d_probs, d_tile0, nprob);
    ALG_CK(cudaGetLastError());
    return HM_OK;
}

template <typename T>
int gemm_run(int nprob, const hm_gemm_problem *probs, cudaStream_t st)
{
    Staged S(st);
    return gemm_launch<T>(nprob, probs, st, S);
}

template <typename T, typename Stage>
int axpby_launch(int nprob, const hm_axpby_problem *probs, cudaStream_t st, Stage &S)
{
    int64_t most = 0;
    for (int i = 0; i < nprob; ++i) {
        const hm_axpby_problem &g = probs[i];
        if (g.m < 0 || g.n < 0) { set_last_error("problem %d: negative size", i); return HM_ERR_INVALID_ARG; }
        if (g.m && g.n && (!g.A || !g.D || (g.beta != 0.0 && !g.B))) {
            set_last_error("problem %d: NULL operand", i);
            return HM_ERR_INVALID_ARG;
        }
        most = std::max(most, g.m * g.n);
    }
    if (nprob == 0 || most == 0) return HM_OK;
    if (nprob > 65535) { set_last_error("more than 65535 problems"); return HM_ERR_UNSUPPORTED; }
    hm_axpby_problem *d_probs = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    const unsigned bx = (unsigned)std::min<int64_t>((most + 255) / 256, 1024);
    axpby_batched<T><<<dim3(bx, nprob), 256, 0, st>>>(d_probs);
    ALG_CK(cudaGetLastError());
    return HM_OK;
}

template <typename T>
int axpby_run(int nprob, const hm_axpby_problem *probs, cudaStream_t st)
{
    Staged S(st);
    return axpby_launch<T>(nprob, probs, st, S);
}

template <typename T>
int64_t potrf_nsmem(int64_t nmax)
{
    // blocks up to nsmem rows are factored in shared memory (<= 200 KB)
    int64_t nsmem = 0;
    while ((nsmem + 1) * (nsmem + 1) * (int64_t)sizeof(T) <= 200 * 1024) ++nsmem;
    return std::min(nsmem, nmax);
}

template <typename T>
int potrf_run(int nprob, const hm_potrf_problem *probs, int32_t *info, cudaStream_t st, int32_t *d_info_out = nullptr)
{
    int64_t nmax = 0;
    for (int i = 0; i < nprob; ++i) {
        const hm_potrf_problem &g = probs[i];
        if (g.n < 0 || (g.n && (!g.A || !g.R || g.lda < g.n || g.ldr < g.n))) {
            set_last_error("problem %d: bad block", i);
            return HM_ERR_INVALID_ARG;
        }
        nmax = std::max(nmax, g.n);
    }
    if (nprob == 0) return HM_OK;
    // blocks up to nsmem rows are factored in shared memory (<= 200 KB)
    int64_t nsmem = 0;
    while ((nsmem + 1) * (nsmem + 1) * (int64_t)sizeof(T) <= 200 * 1024) ++nsmem;
    nsmem = std::min(nsmem, nmax);
    const size_t smem = (size_t)nsmem * nsmem * sizeof(T);
    ALG_TRY(set_smem(potrf_batched<T>, smem));
    Staged S(st);
    hm_potrf_problem *d_probs = nullptr;
    int *d_info = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    if (d_info_out) {
        // asynchronous form: the kernel writes every problem's info word
        potrf_batched<T><<<nprob, kThreads, smem, st>>>(d_probs, d_info_out, nsmem);
        ALG_CK(cudaGetLastError());
        return HM_OK;
    }
    ALG_TRY(S.zeros((size_t)nprob, &d_info));
    potrf_batched<T><<<nprob, kThreads, smem, st>>>(d_probs, d_info, nsmem);
    ALG_CK(cudaGetLastError());
    std::vector<int> hi(nprob);
    ALG_CK(cudaMemcpyAsync(hi.data(), d_info, nprob * sizeof(int), cudaMemcpyDeviceToHost, st));
    ALG_CK(cudaStreamSynchronize(st));
    int bad = 0;
    for (int i = 0; i < nprob; ++i) {
        if (info) info[i] = hi[i];
        if (hi[i] && !bad) {
            bad = 1;
            set_last_error("PosDefException: block %d is not positive definite (pivot %d)", i, hi[i]);
        }
    }
    return bad ? HM_ERR_NOT_POSDEF : HM_OK;
}

// largest block trtri_batched keeps in shared memory (R, W and the pivots)
template <typename T>
int64_t trtri_max()
{
    int64_t n = 0;
    while ((2 * (n + 1) * (n + 2) + (n + 1)) * (int64_t)sizeof(T) <= 200 * 1024) ++n;
    return n;
}

template <typename T, typename Stage>
int trtri_launch(int nprob, const hm_trtri_problem *probs, cudaStream_t st, Stage &S)
{
    int64_t nmax = 0;
    for (int i = 0; i < nprob; ++i) {
        const hm_trtri_problem &g = probs[i];
        if (g.n < 0 || (g.n && (!g.R || !g.W || g.ldr < g.n || g.ldw < g.n))) {
            set_last_error("problem %d: bad block", i);
            return HM_ERR_INVALID_ARG;
        }
        nmax = std::max(nmax, g.n);
    }
    if (nmax > trtri_max<T>()) {
        set_last_error("hm_trtri_batched: blocks up to %lld rows, got %lld", (long long)trtri_max<T>(), (long long)nmax);
        return HM_ERR_UNSUPPORTED;
    }
    if (nprob == 0 || nmax == 0) return HM_OK;
    const size_t smem = (size_t)(2 * (nmax + 1) * nmax + nmax) * sizeof(T);
    ALG_TRY(set_smem(trtri_batched<T>, smem));
    hm_trtri_problem *d_probs = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    trtri_batched<T><<<nprob, kThreads, smem, st>>>(d_probs, nmax);
    ALG_CK(cudaGetLastError());
    return HM_OK;
}

template <typename T>
int trtri_run(int nprob, const hm_trtri_problem *probs, cudaStream_t st)
{
    Staged S(st);
    return trtri_launch<T>(nprob, probs, st, S);
}

template <typename T>
int solve_run(int nops, const hm_solve_op *ops, void *B, int64_t ldb, int64_t ncols, cudaStream_t st)
{
    int64_t extent = 0;
    for (int i = 0; i < nops; ++i) {
        const hm_solve_op &o = ops[i];
        if (o.kind < HM_SOLVE_TRSM || o.kind > HM_SOLVE_LTRSM || ((o.kind == HM_SOLVE_INV || o.kind == HM_SOLVE_LTRSM) && o.n1 > kInvMax) || o.n1 < 0 || o.n2 < 0 || o.o1 < 0 || o.o2 < 0 ||
            !o.A || (o.kind == HM_SOLVE_LR && (o.r < 0 || (o.r && (!o.s || !o.B || o.ld < o.n1 || o.ld2 < o.n2)))) ||
            (o.kind != HM_SOLVE_LR && o.ld < o.n1)) {
            set_last_error("solve op %d: bad operation", i);
            return HM_ERR_INVALID_ARG;
        }
        const bool diag = o.kind == HM_SOLVE_TRSM || o.kind == HM_SOLVE_INV;
        extent = std::max(extent, std::max(o.o1 + o.n1, diag ? 0 : o.o2 + o.n2));
    }
    if (ncols < 0 || (ncols > 0 && (!B || ldb < extent))) {
        set_last_error("right-hand sides: %lld rows needed, leading dimension %lld", (long long)extent, (long long)ldb);
        return HM_ERR_BOUNDS;
    }
    if (nops == 0 || ncols == 0) return HM_OK;
    Staged S(st);
    hm_solve_op *d_ops = nullptr;
    ALG_TRY(S.put(ops, (size_t)nops, &d_ops));
    if (ncols > 0x7fffffff) { set_last_error("too many right-hand sides"); return HM_ERR_INVALID_ARG; }
    solve_schedule<T><<<(unsigned)ncols, kThreads, 0, st>>>(d_ops, nops, static_cast<T *>(B), ldb, 0);
    ALG_CK(cudaGetLastError());
    return HM_OK;
}


// ---- hierarchical Cholesky driver (hm_hchol_factor) --------------------------
//
// src/cholesky.jl:12-92 on a HODLR tree (2 x 2 blocks; upper off-diagonal
// blocks LowRankMatrix, diagonal blocks hierarchical or dense), the
// reference's recursion and block order run on the host in C++:
//   R11 = chol(A11);  R12 = R11^{-T} A12 (the U factor solved);
//   A22 <- A22 - R12'R12;  R22 = chol(A22).
// Every block of A22 is updated when its ancestor is reached, as the
// reference does: a dense leaf D <- D - V_p H V_p^T (two batched GEMMs) and a
// LowRankMatrix block by one truncated SVD of [U_b | V_p] diag(s_b ; -H)
// [V_b | V_q]^T (all blocks of A22 in one launch), where R12 = X diag(s) V^T
// and H = diag(s) X^T X diag(s), so R12'R12 = V H V^T.  The reference forms
// R12'R12 as a truncated SVD first; passing H whole skips that SVD (it would
// drop only singular values below q eps(sigma_1)) and the update's SVD
// truncates the sum.  R12 = R11^{-T} U runs through the left subtree's
// forward-substitution schedule (its leaves as products with their inverses).
// The A22 updates' truncated SVDs run on a pool of other streams, one launch
// per level of A22's tree (the deepest, needed first, first; blocks of one
// depth in the tree always on the same stream): a block updated at node N is
// next needed when the factorisation reaches it, after the part of A22 before
// it, so the SVDs overlap with the chain of leaf factorisations and solves,
// and a large block's SVD does not hold up the small ones.  The host reads a
// block's new rank (which sizes the problems that use it) only when it next
// uses the block, waiting on that update's event; nothing else waits until the
// end.  Problem descriptors go to the device from pinned host memory.

// Device memory handed out in 256-byte aligned pieces from chunks of at
// least 32 MB, all released together.
struct Arena {
    std::vector<void *> chunks;
    char *cur = nullptr;
    size_t left = 0;
    Arena() = default;
    Arena(const Arena &) = delete;
    Arena &operator=(const Arena &) = delete;
    ~Arena() { release(); }
    void release()
    {
        for (void *c : chunks) cudaFree(c);
        chunks.clear();
        cur = nullptr;
        left = 0;
    }
    template <typename T>
    int get(size_t count, T **p)
    {
        const size_t bytes = (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
        if (bytes > left) {
            const size_t sz = std::max<size_t>(bytes, size_t(32) << 20);
            void *c = nullptr;
            ALG_CK(device_malloc(&c, sz));
            chunks.push_back(c);
            cur = static_cast<char *>(c);
            left = sz;
        }
        *p = reinterpret_cast<T *>(cur);
        cur += bytes;
        left -= bytes;
        return HM_OK;
    }
};

// Descriptor staging through pinned host memory (asynchronous copies) and a
// device scratch area, both reused from the start once the caller has
// synchronised the stream (drained()); a full buffer is replaced by a larger
// one and kept until the end, so pointers handed out stay valid.
struct PinnedStager {
    cudaStream_t st;
    std::vector<char *> old_host, old_dev;
    char *host = nullptr, *dev = nullptr, *scratch = nullptr;
    size_t cap = 0, used = 0, scap = 0, sused = 0;
    explicit PinnedStager(cudaStream_t s) : st(s) {}
    PinnedStager(const PinnedStager &) = delete;
    PinnedStager &operator=(const PinnedStager &) = delete;
    ~PinnedStager()
    {
        for (char *h : old_host) cudaFreeHost(h);
        for (char *d : old_dev) cudaFree(d);
        if (host) cudaFreeHost(host);
        if (dev) cudaFree(dev);
        if (scratch) cudaFree(scratch);
    }
    void drained() { used = sused = 0; }
    template <typename T>
    int put(const T *src, size_t count, T **d)
    {
        const size_t bytes = count * sizeof(T), al = (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
        if (used + al > cap) {
            const size_t nc = std::max(al, std::max<size_t>(2 * cap, size_t(1) << 20));
            char *h = nullptr, *dv = nullptr;
            ALG_CK(cudaMallocHost((void **)&h, nc));
            const int st_ = cuda_fail(device_malloc((void **)&dv, nc), "device_malloc");
            if (st_) { cudaFreeHost(h); return st_; }
            if (host) { old_host.push_back(host); old_dev.push_back(dev); }
            host = h; dev = dv; cap = nc; used = 0;
        }
        if (bytes) {
            std::memcpy(host + used, src, bytes);
            ALG_CK(cudaMemcpyAsync(dev + used, host + used, bytes, cudaMemcpyHostToDevice, st));
        }
        *d = reinterpret_cast<T *>(dev + used);
        used += al;
        return HM_OK;
    }
    template <typename T>
    int zeros(size_t count, T **d)
    {
        const size_t al = (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
        if (sused + al > scap) {
            const size_t nc = std::max(al, std::max<size_t>(2 * scap, size_t(32) << 20));
            char *dv = nullptr;
            ALG_CK(device_malloc((void **)&dv, nc));
            if (scratch) old_dev.push_back(scratch);
            scratch = dv; scap = nc; sused = 0;
        }
        *d = reinterpret_cast<T *>(scratch + sused);
        sused += al;
        return HM_OK;
    }
};

// What hm_hchol_factor hands back: R's pieces, in memory owned here.
struct HCholResult {
    Arena keep;
    std::vector<hm_hchol_out> out;
};

template <typename T>
struct HChol {
    struct Node {
        int64_t off = 0;
        int inord = -1, leaf = -1, ob = 0, oe = 0;      // in-order position, leaf number, subtree's op range
        int depth = 0;
        const T *U = nullptr, *s = nullptr, *V = nullptr;   // the current A12 (internal nodes)
        int64_t ldu = 1, ldv = 1;
        int r = 0;
        const T *D = nullptr;                            // the current block (leaves)
        int64_t ldd = 1;
        cudaEvent_t ev = nullptr;                        // r is pending: *slot once ev has completed
        const int32_t *slot = nullptr;
    };
    const hm_hchol_node *in;
    int nn;
    cudaStream_t st;
    HCholResult *res;
    std::vector<Node> nd;
    std::vector<int> inorder;
    Arena temp;
    PinnedStager S;
    hm_solve_op *h_ops = nullptr;                        // the whole tree's schedule, in order
    int32_t *h_small = nullptr, *d_info = nullptr;       // h_small: pinned, ranks and pivot words read back
    unsigned *counter = nullptr;                         // hchol_gram's last-CTA counter
    std::vector<T *> lts;                                // per leaf: R^T for the forward substitutions
    static constexpr int kUpdStreams = 8;
    cudaStream_t sup[kUpdStreams] = {};                 // the A22 updates' truncated SVDs
    cudaStream_t sw = nullptr;                           // the leaves' inverses
    std::vector<cudaEvent_t> wev;                        // per node: its leaf inverse is done
    std::vector<cudaEvent_t> events;
    std::vector<int32_t *> pinned_ints;                  // rank words read back by the side stream
    size_t pinned_left = 0, pinned_cap = 0;
    int64_t h_small_n = 0;
    int nleaves = 0;

    HChol(const hm_hchol_node *nodes, int n, cudaStream_t s, HCholResult *r) : in(nodes), nn(n), st(s), res(r), S(s) {}
    ~HChol()
    {
        for (cudaStream_t &x : sup) {
            if (!x) continue;
            cudaStreamSynchronize(x);                    // nothing in flight reads memory freed below
            cudaStreamDestroy(x);
        }
        if (sw) {
            cudaStreamSynchronize(sw);
            cudaStreamDestroy(sw);
        }
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        for (int32_t *p : pinned_ints) cudaFreeHost(p);
        if (h_ops) cudaFreeHost(h_ops);
        if (h_small) cudaFreeHost(h_small);
    }

    int new_event(cudaEvent_t *e)
    {
        ALG_CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        events.push_back(*e);
        return HM_OK;
    }

    int pinned_words(int n, int32_t **p)
    {
        if ((size_t)n > pinned_left) {
            const size_t cnt = std::max<size_t>(n, 16384);
            int32_t *h = nullptr;
            ALG_CK(cudaMallocHost((void **)&h, cnt * sizeof(int32_t)));
            pinned_ints.push_back(h);
            pinned_cap = pinned_left = cnt;
        }
        *p = pinned_ints.back() + (pinned_cap - pinned_left);
        pinned_left -= n;
        return HM_OK;
    }

    // the rank of node i's current A12 on the host (waits for the update that made it)
    int resolve(int i)
    {
        Node &N = nd[i];
        if (!N.ev) return HM_OK;
        ALG_CK(cudaEventSynchronize(N.ev));
        ALG_CK(cudaStreamWaitEvent(st, N.ev, 0));
        N.r = *N.slot;
        N.ev = nullptr;
        N.slot = nullptr;
        return HM_OK;
    }

    static bool is_leaf(const hm_hchol_node &g) { return g.left < 0 && g.right < 0; }

    // offsets, in-order numbering and the checks of the tree (iterative: trees may be deep)
    int layout(int root)
    {
        if (root < 0 || root >= nn) { set_last_error("root %d out of range", root); return HM_ERR_INVALID_ARG; }
        nd.assign(nn, Node());
        std::vector<char> seen(nn, 0);
        struct Frame { int i, stage; };
        std::vector<Frame> stack{{root, 0}};
        seen[root] = 1;
        nd[root].off = 0;
        while (!stack.empty()) {
            Frame &f = stack.back();
            const hm_hchol_node &g = in[f.i];
            Node &N = nd[f.i];
            if (f.stage == 0) {
                N.ob = (int)inorder.size();
                if (g.n < 1) { set_last_error("node %d: %lld rows", f.i, (long long)g.n); return HM_ERR_INVALID_ARG; }
                if (is_leaf(g)) {
                    if (!g.D || g.ldd < g.n) { set_last_error("leaf %d: no block or ld < n", f.i); return HM_ERR_INVALID_ARG; }
                    N.D = static_cast<const T *>(g.D);
                    N.ldd = g.ldd;
                    N.inord = (int)inorder.size();
                    N.leaf = nleaves++;
                    inorder.push_back(f.i);
                    N.oe = (int)inorder.size();
                    stack.pop_back();
                    continue;
                }
                const int64_t n1 = g.n1, n2 = g.n - g.n1;
                if (g.left < 0 || g.right < 0 || g.left >= nn || g.right >= nn || g.left == g.right || seen[g.left] ||
                    seen[g.right] || n1 < 1 || n2 < 1 || in[g.left].n != n1 || in[g.right].n != n2) {
                    set_last_error("node %d: children or sizes inconsistent", f.i);
                    return HM_ERR_INVALID_ARG;
                }
                if (g.r < 0 || (g.r > 0 && (!g.U || !g.s || !g.V || g.ldu < n1 || g.ldv < n2))) {
                    set_last_error("node %d: bad LowRankMatrix block", f.i);
                    return HM_ERR_INVALID_ARG;
                }
                N.U = static_cast<const T *>(g.U);
                N.s = static_cast<const T *>(g.s);
                N.V = static_cast<const T *>(g.V);
                N.ldu = std::max<int64_t>(g.ldu, 1);
                N.ldv = std::max<int64_t>(g.ldv, 1);
                N.r = g.r;
                seen[g.left] = seen[g.right] = 1;
                nd[g.left].off = N.off;
                nd[g.right].off = N.off + n1;
                nd[g.left].depth = nd[g.right].depth = N.depth + 1;
                f.stage = 1;
                stack.push_back({g.left, 0});
            } else if (f.stage == 1) {
                N.inord = (int)inorder.size();
                inorder.push_back(f.i);
                f.stage = 2;
                stack.push_back({g.right, 0});
            } else {
                N.oe = (int)inorder.size();
                stack.pop_back();
            }
        }
        return HM_OK;
    }

    int small_host(int64_t n)
    {
        if (n <= h_small_n) return HM_OK;
        if (h_small) cudaFreeHost(h_small);
        h_small = nullptr;
        h_small_n = 0;
        ALG_CK(cudaMallocHost((void **)&h_small, sizeof(int32_t) * n));
        h_small_n = n;
        return HM_OK;
    }

    int setup(int root)
    {
        ALG_TRY(layout(root));
        for (cudaStream_t &x : sup) ALG_CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        ALG_CK(cudaStreamCreateWithFlags(&sw, cudaStreamNonBlocking));
        res->out.assign(nn, hm_hchol_out{});
        lts.assign(nn, nullptr);
        wev.assign(nn, nullptr);
        ALG_CK(cudaMallocHost((void **)&h_ops, sizeof(hm_solve_op) * inorder.size()));
        ALG_TRY(temp.get((size_t)nleaves, &d_info));
        ALG_TRY(temp.get(1, &counter));
        ALG_CK(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
        ALG_TRY(small_host(std::max(nleaves, 64)));
        const void *any = nullptr;
        for (int i : inorder) {
            const hm_hchol_node &g = in[i];
            hm_solve_op &op = h_ops[nd[i].inord];
            op = hm_solve_op{};
            op.o1 = nd[i].off;
            op.n1 = is_leaf(g) ? g.n : g.n1;
            if (is_leaf(g)) {
                T *R = nullptr, *W = nullptr;
                ALG_TRY(res->keep.get((size_t)(g.n * g.n), &R));
                hm_hchol_out &o = res->out[i];
                o.R = R;
                o.ldr = g.n;
                op.A = R;
                op.ld = g.n;
                op.kind = HM_SOLVE_TRSM;
                if (g.n <= leaf_chol_max<T>() && g.n <= kInvMax) {  // leaf_chol, its transpose for the solves
                    T *Lt = nullptr;
                    ALG_TRY(temp.get((size_t)(g.n * g.n), &Lt));
                    lts[i] = Lt;
                    op.A = Lt;
                    op.kind = HM_SOLVE_LTRSM;
                }
                if (g.n <= trtri_max<T>()) {          // the inverse, made on its own stream
                    ALG_TRY(res->keep.get((size_t)(g.n * g.n), &W));
                    o.W = W;
                    o.ldw = g.n;
                }
                any = R;
            } else {
                op.kind = HM_SOLVE_LR;                 // rank 0 until the node is reached
                op.o2 = nd[i].off + g.n1;
                op.n2 = g.n - g.n1;
                op.ld = std::max<int64_t>(g.n1, 1);
                op.ld2 = std::max<int64_t>(op.n2, 1);
            }
        }
        for (int i : inorder)
            if (!h_ops[nd[i].inord].A) h_ops[nd[i].inord].A = any;
        return HM_OK;
    }

    int leaf(int i)
    {
        const hm_hchol_node &g = in[i];
        Node &N = nd[i];
        hm_hchol_out &o = res->out[i];
        if (lts[i]) {
            const LeafChol lc{g.n, N.D, N.ldd, o.R, o.ldr, lts[i], g.n};
            const size_t smem = (size_t)(g.n * (g.n + 1)) * sizeof(T);
            ALG_TRY(set_smem(leaf_chol<T>, smem));
            LeafChol *dl = nullptr;
            ALG_TRY(S.put(&lc, 1, &dl));
            leaf_chol<T><<<1, kThreads, smem, st>>>(dl, d_info + N.leaf);
            ALG_CK(cudaGetLastError());
            return inverse(i);
        }
        const hm_potrf_problem pp{g.n, N.D, N.ldd, o.R, o.ldr};
        const int64_t nsmem = potrf_nsmem<T>(g.n);
        const size_t smem = (size_t)nsmem * nsmem * sizeof(T);
        ALG_TRY(set_smem(potrf_batched<T>, smem));
        hm_potrf_problem *dp = nullptr;
        ALG_TRY(S.put(&pp, 1, &dp));
        potrf_batched<T><<<1, kThreads, smem, st>>>(dp, d_info + N.leaf, nsmem);
        ALG_CK(cudaGetLastError());
        return inverse(i);
    }

    // W = R^{-1} of leaf i on the inverses' stream; the solves use it once done
    int inverse(int i)
    {
        hm_hchol_out &o = res->out[i];
        if (!o.W) return HM_OK;
        cudaEvent_t e = nullptr;
        ALG_TRY(new_event(&e));
        ALG_TRY(new_event(&wev[i]));
        ALG_CK(cudaEventRecord(e, st));
        ALG_CK(cudaStreamWaitEvent(sw, e, 0));
        const hm_trtri_problem tp{in[i].n, o.R, o.ldr, o.W, o.ldw};
        S.st = sw;
        const int rc = trtri_launch<T>(1, &tp, sw, S);
        S.st = st;
        ALG_TRY(rc);
        ALG_CK(cudaEventRecord(wev[i], sw));
        return HM_OK;
    }

    // the forward-substitution schedule of the subtree of node j: each leaf
    // as a product with its inverse when that is already made, else by
    // substitution (nothing waits for an inverse)
    int schedule(int j, hm_solve_op **d)
    {
        const Node &J = nd[j];
        std::vector<hm_solve_op> ops(h_ops + J.ob, h_ops + J.oe);
        for (int k = J.ob; k < J.oe; ++k) {
            const int i = inorder[k];
            if (!is_leaf(in[i]) || !wev[i]) continue;
            const cudaError_t q = cudaEventQuery(wev[i]);
            if (q == cudaErrorNotReady) continue;
            ALG_CK(q);
            hm_solve_op &op = ops[k - J.ob];
            op.kind = HM_SOLVE_INV;
            op.A = res->out[i].W;
            op.ld = res->out[i].ldw;
        }
        return S.put(ops.data(), ops.size(), d);
    }

    // every node and leaf below node j (j itself included)
    void subtree(int j, std::vector<int> &leaves, std::vector<int> &inner)
    {
        for (int k = nd[j].ob; k < nd[j].oe; ++k) {
            const int i = inorder[k];
            (is_leaf(in[i]) ? leaves : inner).push_back(i);
        }
    }

    // A22 <- A22 - V H V^T over the right subtree of node i (X n1 x r, V n2 x r)
    int update(int i, const T *X, const T *sk, const T *Vk, int r)
    {
        const hm_hchol_node &g = in[i];
        const int64_t n1 = g.n1, n2 = g.n - g.n1, b0 = nd[g.right].off;
        T *H = nullptr;
        ALG_TRY(temp.get((size_t)r * r, &H));
        if (r <= kGramMax) {
            const int64_t nch = std::max<int64_t>(1, std::min<int64_t>((n1 + 255) / 256, 128));
            const int64_t chunk = ((n1 + nch - 1) / nch + 31) / 32 * 32;
            const int64_t nblk = (n1 + chunk - 1) / chunk;
            T *ws = nullptr;
            ALG_TRY(S.zeros((size_t)(nblk * r * r), &ws));
            hchol_gram<T><<<(unsigned)nblk, kThreads, 0, st>>>(X, n1, n1, r, sk, ws, counter, H, chunk);
            ALG_CK(cudaGetLastError());
        } else {
            T *G = nullptr;
            ALG_TRY(temp.get((size_t)r * r, &G));
            hm_gemm_problem gp{};
            gp.m = r; gp.n = r; gp.k = n1;
            gp.P = X; gp.ldp = n1; gp.transp = 1;
            gp.Q = X; gp.ldq = n1; gp.transq = 1;
            gp.alpha = 1.0; gp.beta = 0.0;
            gp.D = G; gp.ldd = r;
            ALG_TRY(gemm_launch<T>(1, &gp, st, S));
            hm_axpby_problem ap{};
            ap.m = r; ap.n = r; ap.A = G; ap.lda = r; ap.dr = sk; ap.dc = sk; ap.alpha = 1.0; ap.beta = 0.0;
            ap.D = H; ap.ldd = r;
            ALG_TRY(axpby_launch<T>(1, &ap, st, S));
        }

        std::vector<int> leaves, inner;
        subtree(g.right, leaves, inner);
        int64_t nlmax = 0;
        for (int L : leaves) nlmax = std::max(nlmax, in[L].n);
        const size_t lsmem = (size_t)(2 * nlmax * r + r * r) * sizeof(T);
        if (!leaves.empty() && r <= kGramMax && nlmax <= kLeafUpdMax && lsmem <= kCoreSmemBytes) {
            std::vector<LeafUpd> ups(leaves.size());
            for (size_t k = 0; k < leaves.size(); ++k) {
                const int L = leaves[k];
                const int64_t nl = in[L].n;
                T *Dn = nullptr;
                ALG_TRY(temp.get((size_t)(nl * nl), &Dn));
                ups[k] = LeafUpd{nl, Vk + (nd[L].off - b0), n2, nd[L].D, nd[L].ldd, Dn, nl};
                nd[L].D = Dn;
                nd[L].ldd = nl;
            }
            ALG_TRY(set_smem(hchol_leaf_update<T>, lsmem));
            LeafUpd *du = nullptr;
            ALG_TRY(S.put(ups.data(), ups.size(), &du));
            hchol_leaf_update<T><<<(unsigned)ups.size(), kThreads, lsmem, st>>>(du, H, r);
            ALG_CK(cudaGetLastError());
        } else if (!leaves.empty()) {
            std::vector<hm_gemm_problem> p1(leaves.size()), p2(leaves.size());
            for (size_t k = 0; k < leaves.size(); ++k) {
                const int L = leaves[k];
                const int64_t nl = in[L].n;
                const T *Vp = Vk + (nd[L].off - b0);
                T *TL = nullptr, *Dn = nullptr;
                ALG_TRY(temp.get((size_t)(nl * r), &TL));
                ALG_TRY(temp.get((size_t)(nl * nl), &Dn));
                hm_gemm_problem &a = p1[k];
                a = hm_gemm_problem{};
                a.m = nl; a.n = r; a.k = r;
                a.P = Vp; a.ldp = n2; a.Q = H; a.ldq = r;
                a.alpha = 1.0; a.beta = 0.0; a.D = TL; a.ldd = nl;
                hm_gemm_problem &b = p2[k];
                b = hm_gemm_problem{};
                b.m = nl; b.n = nl; b.k = r;
                b.P = TL; b.ldp = nl; b.Q = Vp; b.ldq = n2;
                b.alpha = -1.0; b.beta = 1.0; b.C = nd[L].D; b.ldc = nd[L].ldd;
                b.D = Dn; b.ldd = nl;
                nd[L].D = Dn;
                nd[L].ldd = nl;
            }
            ALG_TRY(gemm_launch<T>((int)p1.size(), p1.data(), st, S));
            ALG_TRY(gemm_launch<T>((int)p2.size(), p2.data(), st, S));
        }
        if (inner.empty()) return HM_OK;
        for (int M : inner) ALG_TRY(resolve(M));         // their previous updates are done
        // one batch per level of the subtree, the deepest first (needed first)
        std::vector<int> depth(inner.size());
        int dmax = 0;
        for (size_t k = 0; k < inner.size(); ++k) {
            int dd = 0;
            for (int64_t w = in[inner[k]].n; w < in[g.right].n; w *= 2) ++dd;
            depth[k] = dd;
            dmax = std::max(dmax, dd);
        }
        cudaEvent_t eh = nullptr;
        ALG_TRY(new_event(&eh));
        ALG_CK(cudaEventRecord(eh, st));
        for (int lev = dmax; lev >= 0; --lev) {
            std::vector<int> grp;
            for (size_t k = 0; k < inner.size(); ++k)
                if (depth[k] == lev) grp.push_back(inner[k]);
            if (grp.empty()) continue;
            ALG_TRY(svd_batch(grp, H, Vk, r, n2, b0, eh));
        }
        return HM_OK;
    }

    // the truncated SVDs of [U_M | V_p] diag(s_M ; -H) [V_M | V_q]^T for the
    // blocks M of one level, on the next update stream once H is ready
    int svd_batch(const std::vector<int> &grp, const T *H, const T *Vk, int r, int64_t n2, int64_t b0,
                  cudaEvent_t eh)
    {
        const int np = (int)grp.size();
        std::vector<LrJob> jobs(np);
        for (int k = 0; k < np; ++k) {
            const int M = grp[k];
            const hm_hchol_node &gm = in[M];
            const int64_t m1 = gm.n1, m2 = gm.n - gm.n1;
            const int rm = nd[M].r;
            const int cap = (int)std::min<int64_t>(std::min(m1, m2), rm + r);
            T *Un = nullptr, *sn = nullptr, *Vn = nullptr;
            ALG_TRY(temp.get((size_t)(m1 * cap), &Un));
            ALG_TRY(temp.get((size_t)cap, &sn));
            ALG_TRY(temp.get((size_t)(m2 * cap), &Vn));
            hm_lr_problem p{};
            p.m = m1; p.n = m2;
            p.a1 = rm; p.a2 = r; p.b1 = rm; p.b2 = r;
            p.qr_left = 1; p.qr_right = 1;
            p.P1 = rm ? nd[M].U : nullptr; p.ldp1 = nd[M].ldu;
            p.P2 = Vk + (nd[M].off - b0); p.ldp2 = n2;
            p.Q1 = rm ? nd[M].V : nullptr; p.ldq1 = nd[M].ldv;
            p.Q2 = Vk + (nd[M].off + m1 - b0); p.ldq2 = n2;
            p.s1 = rm ? nd[M].s : nullptr;
            p.sign2 = -1.0;
            p.U = Un; p.s = sn; p.V = Vn;
            jobs[k] = LrJob{p, H, r};
            nd[M].U = Un; nd[M].ldu = std::max<int64_t>(m1, 1);
            nd[M].s = sn;
            nd[M].V = Vn; nd[M].ldv = std::max<int64_t>(m2, 1);
        }
        LrPlan pl;
        ALG_TRY(lr_svd_plan<T>(np, jobs.data(), pl));
        // blocks of one depth (one size) share a stream: their updates run in the
        // order the factorisation needs them, never behind a larger block's
        cudaStream_t sx = sup[nd[grp[0]].depth % kUpdStreams];
        cudaEvent_t es = nullptr;
        ALG_TRY(new_event(&es));
        ALG_CK(cudaStreamWaitEvent(sx, eh, 0));
        LrJob *dj = nullptr;
        int64_t *doff = nullptr, *dcoff = nullptr;
        T *dws = nullptr;
        int *dr = nullptr;
        S.st = sx;
        int rc = S.put(jobs.data(), (size_t)np, &dj);
        if (!rc) rc = S.put(pl.off.data(), pl.off.size(), &doff);
        if (!rc) rc = S.put(pl.coff.data(), pl.coff.size(), &dcoff);
        S.st = st;
        ALG_TRY(rc);
        ALG_TRY(S.zeros((size_t)pl.ws, &dws));
        ALG_TRY(S.zeros((size_t)np, &dr));
        lr_svd_kernel<T><<<np, kThreads, pl.smem, sx>>>(dj, doff, dcoff, dws, dr, pl.dmax, pl.xoff);
        ALG_CK(cudaGetLastError());
        int32_t *slot = nullptr;
        ALG_TRY(pinned_words(np, &slot));
        ALG_CK(cudaMemcpyAsync(slot, dr, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, sx));
        ALG_CK(cudaEventRecord(es, sx));
        for (int k = 0; k < np; ++k) {
            nd[grp[k]].ev = es;
            nd[grp[k]].slot = slot + k;
        }
        return HM_OK;
    }

    int node(int i)
    {
        const hm_hchol_node &g = in[i];
        if (is_leaf(g)) return leaf(i);
        ALG_TRY(node(g.left));
        ALG_TRY(resolve(i));
        Node &N = nd[i];
        const int r = N.r;
        const int64_t n1 = g.n1, n2 = g.n - g.n1;
        T *X = nullptr, *sk = nullptr, *Vk = nullptr;
        ALG_TRY(res->keep.get((size_t)(n1 * r), &X));
        ALG_TRY(res->keep.get((size_t)r, &sk));
        ALG_TRY(res->keep.get((size_t)(n2 * r), &Vk));
        if (r > 0) {
            ALG_CK(cudaMemcpy2DAsync(X, n1 * sizeof(T), N.U, N.ldu * sizeof(T), n1 * sizeof(T), r,
                                     cudaMemcpyDeviceToDevice, st));
            ALG_CK(cudaMemcpyAsync(sk, N.s, r * sizeof(T), cudaMemcpyDeviceToDevice, st));
            ALG_CK(cudaMemcpy2DAsync(Vk, n2 * sizeof(T), N.V, N.ldv * sizeof(T), n2 * sizeof(T), r,
                                     cudaMemcpyDeviceToDevice, st));
            const Node &L = nd[g.left];
            hm_solve_op *dops = nullptr;
            ALG_TRY(schedule(g.left, &dops));
            solve_schedule<T><<<(unsigned)r, kThreads, 0, st>>>(dops, L.oe - L.ob, X, n1, L.off);
            ALG_CK(cudaGetLastError());
        }
        hm_hchol_out &o = res->out[i];
        o.r = r;
        o.U = X; o.ldu = std::max<int64_t>(n1, 1);
        o.s = sk;
        o.V = Vk; o.ldv = std::max<int64_t>(n2, 1);
        hm_solve_op &op = h_ops[N.inord];
        op.r = r;
        if (r > 0) {
            op.A = X;
            op.s = sk;
            op.B = Vk;
            ALG_TRY(update(i, X, sk, Vk, r));
        }
        return node(g.right);
    }

    // returns HM_OK, or HM_ERR_NOT_POSDEF with (node, pivot) of the first
    // failing leaf in the reference's order
    int run(int root, int32_t *fail)
    {
        ALG_TRY(setup(root));
        ALG_TRY(node(root));
        ALG_CK(cudaMemcpyAsync(h_small, d_info, sizeof(int32_t) * nleaves, cudaMemcpyDeviceToHost, st));
        for (cudaStream_t x : sup) ALG_CK(cudaStreamSynchronize(x));
        ALG_CK(cudaStreamSynchronize(sw));
        ALG_CK(cudaStreamSynchronize(st));
        S.drained();
        for (int i : inorder) {
            if (!is_leaf(in[i])) continue;
            const int w = h_small[nd[i].leaf];
            if (w) {
                if (fail) { fail[0] = i; fail[1] = w; }
                set_last_error("PosDefException: leaf %d is not positive definite (pivot %d)", i, w);
                return HM_ERR_NOT_POSDEF;
            }
        }
        return HM_OK;
    }
};

template <typename T>
int hchol_factor(int nnodes, const hm_hchol_node *nodes, int32_t root, void **ctx, int32_t *fail, cudaStream_t st)
{
    HCholResult *res = new HCholResult();
    int rc;
    {
        HChol<T> h(nodes, nnodes, st, res);
        rc = h.run(root, fail);
        if (rc) cudaStreamSynchronize(st);       // nothing in flight reads memory freed below
    }
    if (rc) {
        delete res;
        return rc;
    }
    *ctx = res;
    return HM_OK;
}

}  // namespace
}  // namespace hm

using namespace hm;

extern "C" {

int hm_lr_svd(int dtype, int nprob, const hm_lr_problem *probs, int32_t *ranks, void *stream)
{
    clear_last_error();
    if (nprob < 0 || (nprob && (!probs || !ranks))) { set_last_error("bad problem list"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return lr_svd_run<double>(nprob, probs, ranks, st);
    if (dtype == HM_F32) return lr_svd_run<float>(nprob, probs, ranks, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_gemm_batched(int dtype, int nprob, const hm_gemm_problem *probs, void *stream)
{
    clear_last_error();
    if (nprob < 0 || (nprob && !probs)) { set_last_error("bad problem list"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return gemm_run<double>(nprob, probs, st);
    if (dtype == HM_F32) return gemm_run<float>(nprob, probs, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_axpby_batched(int dtype, int nprob, const hm_axpby_problem *probs, void *stream)
{
    clear_last_error();
    if (nprob < 0 || (nprob && !probs)) { set_last_error("bad problem list"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return axpby_run<double>(nprob, probs, st);
    if (dtype == HM_F32) return axpby_run<float>(nprob, probs, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_potrf_batched(int dtype, int nprob, const hm_potrf_problem *probs, int32_t *info, void *stream)
{
    clear_last_error();
    if (nprob < 0 || (nprob && !probs)) { set_last_error("bad problem list"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return potrf_run<double>(nprob, probs, info, st);
    if (dtype == HM_F32) return potrf_run<float>(nprob, probs, info, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_potrf_batched_async(int dtype, int nprob, const hm_potrf_problem *probs, int32_t *d_info, void *stream)
{
    clear_last_error();
    if (nprob < 0 || (nprob && (!probs || !d_info))) { set_last_error("bad problem list"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return potrf_run<double>(nprob, probs, nullptr, st, d_info);
    if (dtype == HM_F32) return potrf_run<float>(nprob, probs, nullptr, st, d_info);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_trtri_batched(int dtype, int nprob, const hm_trtri_problem *probs, void *stream)
{
    clear_last_error();
    if (nprob < 0 || (nprob && !probs)) { set_last_error("bad problem list"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return trtri_run<double>(nprob, probs, st);
    if (dtype == HM_F32) return trtri_run<float>(nprob, probs, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_hchol_factor(int dtype, int nnodes, const hm_hchol_node *nodes, int32_t root, void **ctx, int32_t *fail,
                    void *stream)
{
    clear_last_error();
    if (!ctx || nnodes < 1 || !nodes) { set_last_error("bad node list"); return HM_ERR_INVALID_ARG; }
    *ctx = nullptr;
    if (fail) fail[0] = fail[1] = -1;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return hchol_factor<double>(nnodes, nodes, root, ctx, fail, st);
    if (dtype == HM_F32) return hchol_factor<float>(nnodes, nodes, root, ctx, fail, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

int hm_hchol_result(void *ctx, int32_t node, hm_hchol_out *out)
{
    clear_last_error();
    HCholResult *res = static_cast<HCholResult *>(ctx);
    if (!res || !out || node < 0 || node >= (int32_t)res->out.size()) {
        set_last_error("bad context or node");
        return HM_ERR_INVALID_ARG;
    }
    *out = res->out[node];
    return HM_OK;
}

int hm_hchol_free(void *ctx)
{
    clear_last_error();
    delete static_cast<HCholResult *>(ctx);
    return HM_OK;
}

int hm_solve_transposed(int dtype, int nops, const hm_solve_op *ops, void *B, int64_t ldb, int64_t ncols, void *stream)
{
    clear_last_error();
    if (nops < 0 || (nops && !ops)) { set_last_error("bad schedule"); return HM_ERR_INVALID_ARG; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == HM_F64) return solve_run<double>(nops, ops, B, ldb, ncols, st);
    if (dtype == HM_F32) return solve_run<float>(nops, ops, B, ldb, ncols, st);
    set_last_error("unknown dtype %d", dtype);
    return HM_ERR_UNSUPPORTED;
}

}  // extern "C"
