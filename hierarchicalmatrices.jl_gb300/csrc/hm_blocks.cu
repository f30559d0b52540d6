// Block-level kernels: the strided leaf-block products of src/algebra.jl and
// the BarycentricMatrix2D factors of src/BarycentricMatrix.jl, as standalone
// GPU calls on device arrays.
#include <cuda_runtime.h>

#include "hm_kernels.cuh"

namespace hm {

// y[ib + i*incy] += sum_j A[i + lda j] x[jb + j*incx]   (src/algebra.jl:37-48)
// One thread per row; consecutive threads read consecutive rows of a column.
template <typename T>
__global__ void gemv_n(const T *A, int64_t m, int64_t n, int64_t lda, const T *x, int64_t incx, T *y, int64_t incy)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    T acc = 0;
    for (int64_t j = 0; j < n; ++j) acc = fma(A[i + lda * j], x[j * incx], acc);
    y[i * incy] += acc;
}

// y[ib + i*incy] += sum_j A[j + lda i] x[jb + j*incx]   (src/algebra.jl:52-65)
// One warp per output; lanes stride the column, then a shuffle reduction.
template <typename T>
__global__ void gemv_t(const T *A, int64_t m, int64_t n, int64_t lda, const T *x, int64_t incx, T *y, int64_t incy)
{
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    T acc = 0;
    for (int64_t j = lane; j < m; j += 32) acc = fma(A[j + lda * i], x[j * incx], acc);
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) y[i * incy] += acc;
}

// Low-rank block, first stage: t[k] = sum_j W[j + ldw k] x[j*incx] for k < r
// (W = V for the product, U for the adjoint).  One warp per k.
template <typename T>
__global__ void lr_project(const T *W, int64_t rows, int64_t ldw, int64_t r, const T *x, int64_t incx, T *t)
{
    const int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= r) return;
    T acc = 0;
    for (int64_t j = lane; j < rows; j += 32) acc = fma(W[j + ldw * k], x[j * incx], acc);
    for (int o = 16; o; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) t[k] = acc;
}

// Low-rank block, second stage: y[i*incy] += sum_k W[i + ldw k] (C t)[k] with
// C = diag(core) (core_diag) or the r x r core (column-major, transposed for
// the adjoint).  Each CTA forms C t in shared memory first.
template <typename T>
__global__ void lr_expand(const T *W, int64_t rows, int64_t ldw, int64_t r, const T *core, int core_diag,
                          int core_trans, const T *t, T *y, int64_t incy)
{
    extern __shared__ unsigned char smem_raw[];
    T *ct = reinterpret_cast<T *>(smem_raw);
    for (int64_t k = threadIdx.x; k < r; k += blockDim.x) {
        T v = 0;
        if (core_diag) {
            v = core[k] * t[k];
        } else {
            for (int64_t l = 0; l < r; ++l) v = fma(core_trans ? core[l + r * k] : core[k + r * l], t[l], v);
        }
        ct[k] = v;
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    T acc = 0;
    for (int64_t k = 0; k < r; ++k) acc = fma(W[i + ldw * k], ct[k], acc);
    y[i * incy] += acc;
}

// BarycentricMatrix2D factors on the boxes [a, b] x [c, d]
// (src/BarycentricMatrix.jl:147-178, 248-297): F[m + r n] = f(xh_m, yh_n),
// U[i + rows m] = Lagrange basis of the row box at x_i (column-major), and V
// likewise for the columns.  One thread per point (or per F entry).
template <typename T>
__global__ void bary_factors(int kernel, int r, double a, double b, double c, double d, const double *cheb,
                             const double *lam, const double *x, int64_t nx, const double *y, int64_t ny, T *U, T *F,
                             T *V)
{
    __shared__ double xh[HM_RMAX], yh[HM_RMAX], lm[HM_RMAX];
    if (threadIdx.x < r) {
        xh[threadIdx.x] = box_node(a, b, cheb[threadIdx.x]);
        yh[threadIdx.x] = box_node(c, d, cheb[threadIdx.x]);
        lm[threadIdx.x] = lam[threadIdx.x];
    }
    __syncthreads();
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < (int64_t)r * r) F[g] = (T)kernel_eval(kernel, xh[g % r], yh[g / r]);
    for (int side = 0; side < 2; ++side) {
        const int64_t n = side ? ny : nx;
        const double *p = side ? y : x;
        const double *nd = side ? yh : xh;
        T *out = side ? V : U;
        if (g >= n) continue;
        double w[HM_RMAX], sum = 0.0;
#pragma unroll
        for (int m = 0; m < HM_RMAX; ++m)
            if (m < r) { w[m] = __dmul_rn(lm[m], 1.0 / __dsub_rn(p[g], nd[m])); sum = __dadd_rn(sum, w[m]); }
#pragma unroll
        for (int m = 0; m < HM_RMAX; ++m)
            if (m < r) out[g + n * m] = (T)(w[m] / sum);
    }
}

template __global__ void gemv_n<double>(const double *, int64_t, int64_t, int64_t, const double *, int64_t, double *, int64_t);
template __global__ void gemv_n<float>(const float *, int64_t, int64_t, int64_t, const float *, int64_t, float *, int64_t);
template __global__ void gemv_t<double>(const double *, int64_t, int64_t, int64_t, const double *, int64_t, double *, int64_t);
template __global__ void gemv_t<float>(const float *, int64_t, int64_t, int64_t, const float *, int64_t, float *, int64_t);
template __global__ void lr_project<double>(const double *, int64_t, int64_t, int64_t, const double *, int64_t, double *);
template __global__ void lr_project<float>(const float *, int64_t, int64_t, int64_t, const float *, int64_t, float *);
template __global__ void lr_expand<double>(const double *, int64_t, int64_t, int64_t, const double *, int, int, const double *, double *, int64_t);
template __global__ void lr_expand<float>(const float *, int64_t, int64_t, int64_t, const float *, int, int, const float *, float *, int64_t);
template __global__ void bary_factors<double>(int, int, double, double, double, double, const double *, const double *, const double *, int64_t, const double *, int64_t, double *, double *, double *);
template __global__ void bary_factors<float>(int, int, double, double, double, double, const double *, const double *, const double *, int64_t, const double *, int64_t, float *, float *, float *);

}  // namespace hm
