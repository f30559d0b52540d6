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
constexpr int kInvMax = 256;        // largest block of an HM_SOLVE_INV op

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

// Core storage of lr_svd: D (p x q core, ld p), then J (q x q right
// rotations, before that the staging area of the Xm^T Ym product), sigma (q)
// and the sort order (q ints).  In shared memory (D takes d_elems values)
// when core_off < 0, else at ws + core_off for cores too large for it.
template <typename T>
__global__ void __launch_bounds__(kThreads) lr_svd_kernel(const hm_lr_problem *probs, const int64_t *ws_off,
                                                          const int64_t *core_off, T *ws, int *ranks, int64_t d_elems)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const hm_lr_problem pr = probs[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int a = pr.a1 + pr.a2, b = pr.b1 + pr.b2;
    const int64_t m = pr.m, n = pr.n;
    const int ka = pr.qr_left ? (int)(m < a ? m : a) : a;
    const int kb = pr.qr_right ? (int)(n < b ? n : b) : b;
    const bool tr = kb > ka;
    const int p = tr ? kb : ka, q = tr ? ka : kb;
    __shared__ int s_flag, s_rank;
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

    // 3. one-sided Jacobi on the columns of D (p x q, q <= p)
    const int qq = (q + 1) & ~1;
    for (int sweep = 0; sweep < kJacobiSweeps; ++sweep) {
        if (tid == 0) s_flag = 0;
        __syncthreads();
        for (int round = 0; round < qq - 1; ++round) {
            for (int pi = warp; pi < qq / 2; pi += kWarps) {
                int i, j;
                if (pi == 0) { i = round; j = qq - 1; }
                else { i = (round + pi) % (qq - 1); j = (round - pi + qq - 1) % (qq - 1); }
                if (i > j) { const int tmp = i; i = j; j = tmp; }
                if (j >= q) continue;
                T *di = D + (int64_t)p * i, *dj = D + (int64_t)p * j;
                T al = 0, be = 0, ga = 0;
                for (int r = lane; r < p; r += 32) {
                    const T u = di[r], v = dj[r];
                    al = fma(u, u, al); be = fma(v, v, be); ga = fma(u, v, ga);
                }
                al = warp_sum(al); be = warp_sum(be); ga = warp_sum(ga);
                if (al == T(0) || be == T(0) || !(fabs(ga) > Lim<T>::eps * sqrt(al) * sqrt(be))) continue;
                const T zeta = (be - al) / (2 * ga);
                const T az = fabs(zeta);
                const T t = az > Lim<T>::big ? T(0.5) / zeta : copysign(T(1) / (az + sqrt(fma(zeta, zeta, T(1)))), zeta);
                const T c = T(1) / sqrt(fma(t, t, T(1))), s = c * t;
                for (int r = lane; r < p; r += 32) {
                    const T u = di[r], v = dj[r];
                    di[r] = c * u - s * v;
                    dj[r] = s * u + c * v;
                }
                T *ji = J + (int64_t)q * i, *jj = J + (int64_t)q * j;
                for (int r = lane; r < q; r += 32) {
                    const T u = ji[r], v = jj[r];
                    ji[r] = c * u - s * v;
                    jj[r] = s * u + c * v;
                }
                if (lane == 0) s_flag = 1;
            }
            __syncthreads();
        }
        const int any = s_flag;
        __syncthreads();
        if (!any) break;
    }

    // 4. singular values, descending order, getrank
    T *sig = J + (int64_t)q * q;
    int *perm = reinterpret_cast<int *>(sig + q);
    for (int j = warp; j < q; j += kWarps) {
        T *dj = D + (int64_t)p * j;
        T ss = 0;
        for (int r = lane; r < p; r += 32) ss = fma(dj[r], dj[r], ss);
        const T sv = sqrt(warp_sum(ss));
        if (sv > T(0)) {
            const T inv = T(1) / sv;
            for (int r = lane; r < p; r += 32) dj[r] *= inv;
        }
        if (lane == 0) sig[j] = sv;
    }
    __syncthreads();
    for (int j = tid; j < q; j += kThreads) {
        int pos = 0;
        const T sj = sig[j];
        for (int l = 0; l < q; ++l) pos += (sig[l] > sj) || (sig[l] == sj && l < j);
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
        if (threadIdx.x == 0) {
            const T d = S[j + ld * j];
            if (!(d > T(0))) s_fail = (int)(j + 1);
            else S[j + ld * j] = sqrt(d);
        }
        __syncthreads();
        if (s_fail) break;
        const T inv = T(1) / S[j + ld * j];
        for (int64_t i = j + 1 + threadIdx.x; i < n; i += kThreads) S[j + ld * i] *= inv;
        __syncthreads();
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
__global__ void __launch_bounds__(kThreads) solve_schedule(const hm_solve_op *ops, int nops, T *B, int64_t ldb)
{
    __shared__ T tk[kTkChunk];
    __shared__ T xs[kInvMax];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T *x = B + ldb * (int64_t)blockIdx.x;
    for (int o = 0; o < nops; ++o) {
        const hm_solve_op op = ops[o];
        const T *A = static_cast<const T *>(op.A);
        if (op.kind == HM_SOLVE_TRSM) {
            if (warp == 0) trsm_t_warp(A, op.ld, op.n1, x + op.o1);
        } else if (op.kind == HM_SOLVE_INV) {
            // x1 <- W^T x1, W = R^{-1} upper: four lanes per output, all warps
            T *x1 = x + op.o1;
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
            const T *x1 = x + op.o1;
            T *x2 = x + op.o2;
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
            const T *x1 = x + op.o1;
            for (int64_t j = warp; j < op.n2; j += kWarps) {
                const T *col = A + op.ld * j;
                T part = 0;
                for (int64_t i = lane; i < op.n1; i += 32) part = fma(col[i], x1[i], part);
                part = warp_sum(part);
                if (lane == 0) x[op.o2 + j] -= part;
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
        ALG_CK(device_malloc_async(&p, std::max<size_t>(count, 1) * sizeof(T), st));
        ptrs.push_back(p);
        if (count) ALG_CK(cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, st));
        *dev = static_cast<T *>(p);
        return HM_OK;
    }
    template <typename T>
    int zeros(size_t count, T **dev)
    {
        void *p = nullptr;
        ALG_CK(device_malloc_async(&p, std::max<size_t>(count, 1) * sizeof(T), st));
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

template <typename T>
int lr_svd_run(int nprob, const hm_lr_problem *probs, int32_t *ranks, cudaStream_t st)
{
    std::vector<int64_t> off(nprob), coff(nprob, -1);
    int64_t ws = 0, dmax = 1, jmax = 1;
    int qmax = 1;
    for (int i = 0; i < nprob; ++i) {
        const hm_lr_problem &p = probs[i];
        const int a = p.a1 + p.a2, b = p.b1 + p.b2;
        if (p.m < 0 || p.n < 0 || p.a1 < 0 || p.a2 < 0 || p.b1 < 0 || p.b2 < 0) {
            set_last_error("problem %d: negative size", i);
            return HM_ERR_INVALID_ARG;
        }
        if (p.Xm) {
            if (p.a2 || p.b2 || p.qr_left || p.qr_right || p.t < 0 || (p.t > 0 && !p.Ym) || (p.a1 && !p.s1) ||
                (p.b1 && !p.s2)) {
                set_last_error("problem %d: the Xm^T Ym core takes one part per side, no QR", i);
                return HM_ERR_INVALID_ARG;
            }
        } else if (a != b || (p.a1 && !p.s1) || (p.a2 && !p.s2)) {
            set_last_error("problem %d: a diagonal middle needs a1 + a2 == b1 + b2 and its values", i);
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
        off[i] = ws;
        ws += (p.qr_left ? p.m * a : 0) + (p.qr_right ? p.n * b : 0) + a + b;
        ws = (ws + 31) / 32 * 32;
        const int64_t jn = std::max(q * q, p.Xm ? (int64_t)32 * (a + b) : 0);
        const size_t need = (size_t)(pp * q + jn + q) * sizeof(T) + (size_t)q * sizeof(int) + 64;
        if (need <= kCoreSmemBytes) {
            dmax = std::max(dmax, pp * q);
            jmax = std::max(jmax, jn);
            qmax = std::max<int>(qmax, (int)q);
        } else {
            coff[i] = ws;
            ws += pp * q + jn + 2 * q;          // sigma (q values) and the order (q ints) after J
            ws = (ws + 31) / 32 * 32;
        }
    }
    if (nprob == 0) return HM_OK;
    // J also holds sigma (q values) and the sort order (q ints) after it
    const size_t smem = (size_t)(dmax + jmax + qmax) * sizeof(T) + (size_t)qmax * sizeof(int) + 64;
    ALG_TRY(set_smem(lr_svd_kernel<T>, smem));
    Staged S(st);
    hm_lr_problem *d_probs = nullptr;
    int64_t *d_off = nullptr, *d_coff = nullptr;
    T *d_ws = nullptr;
    int *d_ranks = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    ALG_TRY(S.put(off.data(), off.size(), &d_off));
    ALG_TRY(S.put(coff.data(), coff.size(), &d_coff));
    ALG_TRY(S.zeros((size_t)std::max<int64_t>(ws, 1), &d_ws));
    ALG_TRY(S.zeros((size_t)nprob, &d_ranks));
    lr_svd_kernel<T><<<nprob, kThreads, smem, st>>>(d_probs, d_off, d_coff, d_ws, d_ranks, dmax);
    ALG_CK(cudaGetLastError());
    std::vector<int> hr(nprob);
    ALG_CK(cudaMemcpyAsync(hr.data(), d_ranks, nprob * sizeof(int), cudaMemcpyDeviceToHost, st));
    ALG_CK(cudaStreamSynchronize(st));
    for (int i = 0; i < nprob; ++i) ranks[i] = hr[i];
    return HM_OK;
}

template <typename T>
int gemm_run(int nprob, const hm_gemm_problem *probs, cudaStream_t st)
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
    Staged S(st);
    hm_gemm_problem *d_probs = nullptr;
    int64_t *d_tile0 = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    ALG_TRY(S.put(tile0.data(), tile0.size(), &d_tile0));
    gemm_batched<T><<<(unsigned)tiles, 256, 0, st>>>(d_probs, d_tile0, nprob);
    ALG_CK(cudaGetLastError());
    return HM_OK;
}

template <typename T>
int axpby_run(int nprob, const hm_axpby_problem *probs, cudaStream_t st)
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
    Staged S(st);
    hm_axpby_problem *d_probs = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    const unsigned bx = (unsigned)std::min<int64_t>((most + 255) / 256, 1024);
    axpby_batched<T><<<dim3(bx, nprob), 256, 0, st>>>(d_probs);
    ALG_CK(cudaGetLastError());
    return HM_OK;
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

template <typename T>
int trtri_run(int nprob, const hm_trtri_problem *probs, cudaStream_t st)
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
    Staged S(st);
    hm_trtri_problem *d_probs = nullptr;
    ALG_TRY(S.put(probs, (size_t)nprob, &d_probs));
    trtri_batched<T><<<nprob, kThreads, smem, st>>>(d_probs, nmax);
    ALG_CK(cudaGetLastError());
    return HM_OK;
}

template <typename T>
int solve_run(int nops, const hm_solve_op *ops, void *B, int64_t ldb, int64_t ncols, cudaStream_t st)
{
    int64_t extent = 0;
    for (int i = 0; i < nops; ++i) {
        const hm_solve_op &o = ops[i];
        if (o.kind < HM_SOLVE_TRSM || o.kind > HM_SOLVE_INV || (o.kind == HM_SOLVE_INV && o.n1 > kInvMax) || o.n1 < 0 || o.n2 < 0 || o.o1 < 0 || o.o2 < 0 ||
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
    solve_schedule<T><<<(unsigned)ncols, kThreads, 0, st>>>(d_ops, nops, static_cast<T *>(B), ldb);
    ALG_CK(cudaGetLastError());
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
