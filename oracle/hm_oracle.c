/*
 * hm_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C CPU restatement of the hot path of HierarchicalMatrices.jl v0.2.2
 * (Julia): the KernelMatrix block tree, its Chebyshev/barycentric compression
 * and its matrix-vector product, plus the generic strided block kernels the
 * reference's own tests pin.  Only the test suite, the smoke check and the CPU
 * baseline leg of the benchmark load this library, and only as the checker or
 * as the timed CPU reference; the product never links or calls it.
 *
 * Every function follows one reference function and keeps its loop order and
 * its rounding steps (no FMA contraction: build with -ffp-contract=off), so
 * that results agree with the Julia code to the last few ulps:
 *   - chebyshev nodes / weights        src/BarycentricMatrix.jl:92-136
 *   - BarycentricPoly2D (F samples)    src/BarycentricMatrix.jl:147-178
 *   - BarycentricMatrix2D + update!    src/BarycentricMatrix.jl:236-297
 *   - indsplit                         src/BarycentricMatrix.jl:299-307
 *   - KernelMatrix / 1 / 2             src/KernelMatrix.jl:47-116
 *   - KernelMatrix mul! (block walk)   src/KernelMatrix.jl:14-45
 *   - BarycentricMatrix2D mul!         src/algebra.jl:243-277
 *   - dense / transposed mul!          src/algebra.jl:37-82
 *   - LowRankMatrix mul! / adjoint     src/algebra.jl:110-159
 *   - BLOCKRANK                        src/HierarchicalMatrices.jl:5-7
 *
 * Parity of the KernelMatrix matvec is pinned against dense FP64 products
 * (the reference's own check in examples/Kernel.jl:73-78) and, for the
 * strided block kernels, against the known answers of test/runtests.jl:15-52.
 * Julia is not available to run the reference itself.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_OK 0
#define OR_ERR_BOUNDS 1
#define OR_ERR_ALLOC 2
#define OR_ERR_ARG 3

enum { OR_TAG_KMAT = 1, OR_TAG_BARY = 2, OR_TAG_DENSE = 3 };
enum { OR_CAUCHY = 0, OR_COULOMB = 1, OR_COULOMB_PRIME = 2, OR_LOG = 3 };

/* BLOCKRANK(T) = 2*round(0.5*log_{3+sqrt 8}(1/eps(T)))  (src/HierarchicalMatrices.jl:5) */
int or_blockrank(double eps)
{
    double v = 0.5 * (log(1.0 / eps) / log(3.0 + sqrt(8.0)));
    return 2 * (int)llround(v);
}

static double or_sinpi(double t)
{
    /* sin(pi t) evaluated in extended precision and rounded once. */
    long double pi = 3.141592653589793238462643383279502884L;
    return (double)sinl(pi * (long double)t);
}

/* chebyshevpoints(T, n; kind)  src/BarycentricMatrix.jl:92-111 */
void or_chebyshevpoints(int n, int kind, double *x)
{
    int nd2 = n / 2;
    for (int k = 0; k < n; ++k) x[k] = 0.0;
    for (int k = 1; k <= nd2; ++k) {
        double num = (double)(n - 2 * k) + 1.0;
        double den = (kind == 1) ? (double)(2 * n) : (double)(2 * (n - 1));
        x[k - 1] = or_sinpi(num / den);
    }
    for (int k = 1; k <= nd2; ++k) x[n - k] = -x[k - 1];
}

/* chebyshevbarycentricweights(T, n; kind)  src/BarycentricMatrix.jl:114-136 */
void or_chebyshevweights(int n, int kind, double *w)
{
    int nd2 = n / 2;
    for (int k = 0; k < n; ++k) w[k] = 0.0;
    if (kind == 1) {
        for (int k = 1; k <= nd2 + 1 && k <= n; ++k)
            w[k - 1] = or_sinpi(((double)(2 * k) - 1.0) / (double)(2 * n));
        for (int k = 1; k <= nd2; ++k) w[n - k] = w[k - 1];
        for (int k = 2; k <= n; k += 2) w[k - 1] *= -1.0;
    } else {
        for (int k = 0; k < n; ++k) w[k] = 1.0;
        for (int k = 2; k <= n; k += 2) w[k - 1] *= -1.0;
        w[0] *= 0.5;
        w[n - 1] *= 0.5;
    }
}

/* The kernels of examples/Kernel.jl:34-37. */
static double or_kernel(int id, double x, double y)
{
    double d = x - y;
    switch (id) {
    case OR_CAUCHY: return 1.0 / d;
    case OR_COULOMB: return 1.0 / (d * d);
    case OR_COULOMB_PRIME: return 1.0 / ((d * d) * d);
    default: return log(fabs(d));
    }
}

double or_kernel_eval(int id, double x, double y) { return or_kernel(id, x, y); }

/* A contiguous index range (0-based start, length >= 0): a Julia UnitRange. */
typedef struct { int64_t s, l; } or_range;

/*
 * indsplit  src/BarycentricMatrix.jl:299-307.  Scans from first(ir) while
 * x[i] >= (a+b)/2.  The first element is read even for an empty range, as in
 * the reference (a read past the end is the reference's BoundsError).
 */
static int or_indsplit(const double *x, int64_t nx, or_range ir, double a, double b,
                       or_range *r1, or_range *r2)
{
    double ab2 = 0.5 * (a + b);
    int64_t i = ir.s;
    for (;;) {
        if (i < 0 || i >= nx) return OR_ERR_BOUNDS;
        if (!(x[i] >= ab2)) break;
        i += 1;
        if (i > ir.s + ir.l - 1) break;
    }
    r1->s = ir.s; r1->l = i - ir.s;
    r2->s = i;
    r2->l = ir.s + ir.l - i; if (r2->l < 0) r2->l = 0;
    return OR_OK;
}

int or_indsplit_api(const double *x, int64_t nx, int64_t s, int64_t l, double a, double b,
                    int64_t *out4)
{
    or_range ir = {s, l}, r1, r2;
    int st = or_indsplit(x, nx, ir, a, b, &r1, &r2);
    if (st) return st;
    out4[0] = r1.s; out4[1] = r1.l; out4[2] = r2.s; out4[3] = r2.l;
    return OR_OK;
}

typedef struct or_block {
    int tag;
    int64_t m, n;           /* size(block) */
    int64_t i0, j0;         /* first row / column (0-based) in x / y */
    int level;              /* depth in the block tree (root KernelMatrix = 0) */
    struct or_block *child[4];  /* KernelMatrix: blocks (1,1),(1,2),(2,1),(2,2) */
    int r;                  /* BarycentricMatrix2D rank */
    double box[4];          /* a, b, c, d of a BarycentricMatrix2D */
    double *U, *V, *F;      /* column-major m x r, n x r, r x r */
    double *A;              /* dense leaf, column-major m x n */
} or_block;

typedef struct {
    int kernel, r;
    int64_t leaf;          /* BLOCKSIZE */
    const double *x, *y;
    int64_t nx, ny;
    double *cheb, *lam;    /* r nodes / weights of the first kind */
    int err;
} or_ctx;

static or_block *or_new(int tag)
{
    or_block *b = (or_block *)calloc(1, sizeof(or_block));
    if (b) b->tag = tag;
    return b;
}

void or_free(or_block *b)
{
    if (!b) return;
    for (int k = 0; k < 4; ++k) or_free(b->child[k]);
    free(b->U); free(b->V); free(b->F); free(b->A);
    free(b);
}

/* T[f(x[i], y[j]) for i in ir, j in jr]  src/KernelMatrix.jl:57-60 */
static or_block *or_dense(or_ctx *c, or_range ir, or_range jr, int level)
{
    or_block *b = or_new(OR_TAG_DENSE);
    if (!b) { c->err = OR_ERR_ALLOC; return NULL; }
    b->m = ir.l; b->n = jr.l; b->i0 = ir.s; b->j0 = jr.s; b->level = level;
    b->A = (double *)malloc(sizeof(double) * (size_t)(ir.l * jr.l + 1));
    if (!b->A) { c->err = OR_ERR_ALLOC; free(b); return NULL; }
    for (int64_t j = 0; j < jr.l; ++j)
        for (int64_t i = 0; i < ir.l; ++i) {
            int64_t gi = ir.s + i, gj = jr.s + j;
            if (gi >= c->nx || gj >= c->ny) { c->err = OR_ERR_BOUNDS; b->A[i + ir.l * j] = 0; continue; }
            b->A[i + ir.l * j] = or_kernel(c->kernel, c->x[gi], c->y[gj]);
        }
    return b;
}

/*
 * BarycentricMatrix2D(T, f, a, b, c, d, x, y, ir, jr): BarycentricPoly2D
 * (src/BarycentricMatrix.jl:147-178) followed by update!
 * (src/BarycentricMatrix.jl:248-297).
 */
static or_block *or_bary(or_ctx *c, double a, double b, double cc, double d,
                         or_range ir, or_range jr, int level)
{
    int r = c->r;
    or_block *B = or_new(OR_TAG_BARY);
    if (!B) { c->err = OR_ERR_ALLOC; return NULL; }
    B->m = ir.l; B->n = jr.l; B->i0 = ir.s; B->j0 = jr.s; B->r = r; B->level = level;
    B->box[0] = a; B->box[1] = b; B->box[2] = cc; B->box[3] = d;
    B->U = (double *)malloc(sizeof(double) * (size_t)(ir.l * r + 1));
    B->V = (double *)malloc(sizeof(double) * (size_t)(jr.l * r + 1));
    B->F = (double *)malloc(sizeof(double) * (size_t)(r * r));
    if (!B->U || !B->V || !B->F) { c->err = OR_ERR_ALLOC; or_free(B); return NULL; }
    double xh[64], yh[64];
    double ab2 = 0.5 * (a + b), ba2 = 0.5 * (b - a);
    double cd2 = 0.5 * (cc + d), dc2 = 0.5 * (d - cc);
    for (int p = 0; p < r; ++p) xh[p] = ab2 + ba2 * c->cheb[p];
    for (int q = 0; q < r; ++q) yh[q] = cd2 + dc2 * c->cheb[q];
    for (int n = 0; n < r; ++n)
        for (int m = 0; m < r; ++m) B->F[m + r * n] = or_kernel(c->kernel, xh[m], yh[n]);
    /* update!: U[i,m] = lam_m * inv(x_i - xh_m), normalised by the row sum */
    for (int m = 0; m < r; ++m)
        for (int64_t i = 0; i < ir.l; ++i) {
            int64_t gi = ir.s + i;
            if (gi >= c->nx) { c->err = OR_ERR_BOUNDS; B->U[i + ir.l * m] = 0; continue; }
            B->U[i + ir.l * m] = c->lam[m] * (1.0 / (c->x[gi] - xh[m]));
        }
    for (int64_t i = 0; i < ir.l; ++i) {
        double t = 0.0;
        for (int m = 0; m < r; ++m) t += B->U[i + ir.l * m];
        for (int m = 0; m < r; ++m) B->U[i + ir.l * m] /= t;
    }
    for (int n = 0; n < r; ++n)
        for (int64_t j = 0; j < jr.l; ++j) {
            int64_t gj = jr.s + j;
            if (gj >= c->ny) { c->err = OR_ERR_BOUNDS; B->V[j + jr.l * n] = 0; continue; }
            B->V[j + jr.l * n] = c->lam[n] * (1.0 / (c->y[gj] - yh[n]));
        }
    for (int64_t j = 0; j < jr.l; ++j) {
        double t = 0.0;
        for (int n = 0; n < r; ++n) t += B->V[j + jr.l * n];
        for (int n = 0; n < r; ++n) B->V[j + jr.l * n] /= t;
    }
    return B;
}

static void or_kmat_size(or_block *H)
{
    /* size(H): rows from block column N=2, columns from block row 1
       (src/hierarchical.jl:33-47) */
    H->m = H->child[1]->m + H->child[3]->m;
    H->n = H->child[0]->n + H->child[1]->n;
    H->i0 = H->child[0]->i0; H->j0 = H->child[0]->j0;
}

/* kind: 0 = KernelMatrix, 1 = KernelMatrix1, 2 = KernelMatrix2
   (src/KernelMatrix.jl:49-70, 72-93, 95-116) */
static or_block *or_kmat_rec(or_ctx *c, int kind, or_range ir, or_range jr,
                             double a, double b, double cc, double d, int level)
{
    or_range ir1, ir2, jr1, jr2;
    int st = or_indsplit(c->x, c->nx, ir, a, b, &ir1, &ir2);
    if (!st) st = or_indsplit(c->y, c->ny, jr, cc, d, &jr1, &jr2);
    if (st) { c->err = st; return NULL; }
    double ab2 = 0.5 * (a + b), cd2 = 0.5 * (cc + d);
    int leaf = ir1.l < c->leaf && ir2.l < c->leaf && jr1.l < c->leaf && jr2.l < c->leaf;
    or_block *H = or_new(OR_TAG_KMAT);
    if (!H) { c->err = OR_ERR_ALLOC; return NULL; }
    H->level = level;
    int L = level + 1;
    if (kind == 0) {
        if (leaf) {
            H->child[0] = or_dense(c, ir1, jr1, L);
            H->child[1] = or_dense(c, ir1, jr2, L);
            H->child[2] = or_dense(c, ir2, jr1, L);
            H->child[3] = or_dense(c, ir2, jr2, L);
        } else {
#ifdef _OPENMP
#pragma omp task shared(H) if (level < 6)
#endif
            H->child[0] = or_kmat_rec(c, 0, ir1, jr1, a, ab2, cc, cd2, L);
#ifdef _OPENMP
#pragma omp task shared(H) if (level < 6)
#endif
            H->child[1] = or_kmat_rec(c, 1, ir1, jr2, a, ab2, cd2, d, L);
#ifdef _OPENMP
#pragma omp task shared(H) if (level < 6)
#endif
            H->child[2] = or_kmat_rec(c, 2, ir2, jr1, ab2, b, cc, cd2, L);
            H->child[3] = or_kmat_rec(c, 0, ir2, jr2, ab2, b, cd2, d, L);
#ifdef _OPENMP
#pragma omp taskwait
#endif
        }
    } else if (kind == 1) {
        H->child[0] = or_bary(c, a, ab2, cc, cd2, ir1, jr1, L);
        H->child[1] = or_bary(c, a, ab2, cd2, d, ir1, jr2, L);
        H->child[2] = leaf ? or_dense(c, ir2, jr1, L)
                           : or_kmat_rec(c, 1, ir2, jr1, ab2, b, cc, cd2, L);
        H->child[3] = or_bary(c, ab2, b, cd2, d, ir2, jr2, L);
    } else {
        H->child[0] = or_bary(c, a, ab2, cc, cd2, ir1, jr1, L);
        H->child[1] = leaf ? or_dense(c, ir1, jr2, L)
                           : or_kmat_rec(c, 2, ir1, jr2, a, ab2, cd2, d, L);
        H->child[2] = or_bary(c, ab2, b, cc, cd2, ir2, jr1, L);
        H->child[3] = or_bary(c, ab2, b, cd2, d, ir2, jr2, L);
    }
    for (int k = 0; k < 4; ++k)
        if (!H->child[k]) { if (!c->err) c->err = OR_ERR_ALLOC; or_free(H); return NULL; }
    or_kmat_size(H);
    return H;
}

/* KernelMatrix(f, x, y, a, b, c, d)  src/KernelMatrix.jl:47 */
int or_kernelmatrix(int kernel, const double *x, int64_t nx, const double *y, int64_t ny,
                    double a, double b, double c, double d, int r, int64_t leaf, int nthreads,
                    or_block **out)
{
    if (r < 1 || r > 64 || nx < 1 || ny < 1) return OR_ERR_ARG;
    or_ctx ctx;
    memset(&ctx, 0, sizeof(ctx));
    ctx.kernel = kernel; ctx.r = r; ctx.leaf = leaf;
    ctx.x = x; ctx.y = y; ctx.nx = nx; ctx.ny = ny;
    double cheb[64], lam[64];
    or_chebyshevpoints(r, 1, cheb);
    or_chebyshevweights(r, 1, lam);
    ctx.cheb = cheb; ctx.lam = lam;
    or_range ir = {0, nx}, jr = {0, ny};
    or_block *H = NULL;
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel num_threads(nthreads)
#pragma omp single
        H = or_kmat_rec(&ctx, 0, ir, jr, a, b, c, d, 0);
    } else
#endif
    {
        (void)nthreads;
        H = or_kmat_rec(&ctx, 0, ir, jr, a, b, c, d, 0);
    }
    if (ctx.err) { or_free(H); return ctx.err; }
    *out = H;
    return OR_OK;
}

/* --- block matvecs ------------------------------------------------------ */

/* mul!(u, B::BarycentricMatrix2D, v, istart, jstart)  src/algebra.jl:243-277
   (istart/jstart are 1-based, as in Julia) */
static void or_bary_mul(double *u, const or_block *B, const double *v, int64_t istart, int64_t jstart)
{
    int r = B->r;
    double t1[64], t2[64];
    int64_t ishift = istart - 1, jshift = jstart - 1;
    for (int k = 0; k < r; ++k) {
        double s = 0.0;
        for (int64_t j = 1; j <= B->n; ++j) s += B->V[(j - 1) + B->n * k] * v[jshift + j - 1];
        t1[k] = s;
        t2[k] = 0.0;
    }
    for (int l = 0; l < r; ++l) {
        double t = t1[l];
        for (int k = 0; k < r; ++k) t2[k] += B->F[k + r * l] * t;
    }
    for (int k = 0; k < r; ++k) {
        double t = t2[k];
        for (int64_t i = 1; i <= B->m; ++i) u[ishift + i - 1] += B->U[(i - 1) + B->m * k] * t;
    }
}

/* mul!(y, A::Matrix, x, istart, jstart, INCX, INCY)  src/algebra.jl:37-48 */
void or_dense_mul(double *y, const double *A, int64_t m, int64_t n, const double *x,
                  int64_t istart, int64_t jstart, int64_t incx, int64_t incy)
{
    int64_t ishift = istart - incy, jshift = jstart - incx;
    for (int64_t j = 1; j <= n; ++j) {
        double xj = x[jshift + j * incx - 1];
        for (int64_t i = 1; i <= m; ++i) y[ishift + i * incy - 1] += A[(i - 1) + m * (j - 1)] * xj;
    }
}

/* mul!(y, transpose(A), x, istart, jstart, INCX, INCY)  src/algebra.jl:52-65;
   the adjoint (src/algebra.jl:69-82) is the same for real data */
void or_dense_mul_t(double *y, const double *A, int64_t m, int64_t n, const double *x,
                    int64_t istart, int64_t jstart, int64_t incx, int64_t incy)
{
    int64_t ishift = istart - incy, jshift = jstart - incx;
    for (int64_t i = 1; i <= n; ++i) {
        double yi = 0.0;
        for (int64_t j = 1; j <= m; ++j) yi += A[(j - 1) + m * (i - 1)] * x[jshift + j * incx - 1];
        y[ishift + i * incy - 1] += yi;
    }
}

/* mul!(y, L::LowRankMatrix, x, istart, jstart, INCX, INCY)  src/algebra.jl:110-131
   U is m x r, V is n x r (column-major), sigma = diag(Sigma). */
void or_lowrank_mul(double *y, const double *U, const double *sigma, const double *V,
                    int64_t m, int64_t n, int64_t r, const double *x,
                    int64_t istart, int64_t jstart, int64_t incx, int64_t incy)
{
    int64_t ishift = istart - incy, jshift = jstart - incx;
    double *temp = (double *)malloc(sizeof(double) * (size_t)(r + 1));
    for (int64_t k = 0; k < r; ++k) {
        double t = 0.0;
        for (int64_t j = 1; j <= n; ++j) t += V[(j - 1) + n * k] * x[jshift + j * incx - 1];
        temp[k] = t * sigma[k];
    }
    for (int64_t k = 0; k < r; ++k) {
        double tk = temp[k];
        for (int64_t i = 1; i <= m; ++i) y[ishift + i * incy - 1] += U[(i - 1) + m * k] * tk;
    }
    free(temp);
}

/* mul!(y, L', x, istart, jstart, INCX, INCY)  src/algebra.jl:137-159 */
void or_lowrank_mul_t(double *y, const double *U, const double *sigma, const double *V,
                      int64_t m, int64_t n, int64_t r, const double *x,
                      int64_t istart, int64_t jstart, int64_t incx, int64_t incy)
{
    int64_t ishift = istart - incy, jshift = jstart - incx;
    double *temp = (double *)malloc(sizeof(double) * (size_t)(r + 1));
    for (int64_t k = 0; k < r; ++k) {
        double t = 0.0;
        for (int64_t j = 1; j <= m; ++j) t += U[(j - 1) + m * k] * x[jshift + j * incx - 1];
        temp[k] = t * sigma[k];
    }
    for (int64_t k = 0; k < r; ++k) {
        double tk = temp[k];
        for (int64_t i = 1; i <= n; ++i) y[ishift + i * incy - 1] += V[(i - 1) + n * k] * tk;
    }
    free(temp);
}

/* Block walk of the generated mul!(u, H::KernelMatrix, v, istart, jstart)
   src/KernelMatrix.jl:17-45.  The two block rows write disjoint parts of u, so
   they may run as parallel tasks without changing any summation order. */
static void or_kmat_mul_rec(double *u, const or_block *H, const double *v, int64_t istart, int64_t jstart)
{
    if (H->tag == OR_TAG_BARY) { or_bary_mul(u, H, v, istart, jstart); return; }
    if (H->tag == OR_TAG_DENSE) { or_dense_mul(u, H->A, H->m, H->n, v, istart, jstart, 1, 1); return; }
    int64_t p = 0;
    for (int m = 0; m < 2; ++m) {
        int64_t pm = p;
#ifdef _OPENMP
#pragma omp task if (H->level < 6) firstprivate(pm, m)
#endif
        {
            int64_t q = 0;
            for (int n = 0; n < 2; ++n) {
                or_kmat_mul_rec(u, H->child[2 * m + n], v, istart + pm, jstart + q);
                q += H->child[n]->n;   /* blocksize(H, 1, n, 2) */
            }
        }
        p += H->child[2 * m + 1]->m;   /* blocksize(H, m, N, 1) */
    }
#ifdef _OPENMP
#pragma omp taskwait
#endif
}

/* LinearAlgebra.mul!(u, H, v) = mul!(u, H, v, 1, 1): accumulates into u. */
int or_kernelmatrix_mul(const or_block *H, double *u, int64_t nu, const double *v, int64_t nv,
                        int nthreads)
{
    if (nu < H->m || nv < H->n) return OR_ERR_BOUNDS;
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel num_threads(nthreads)
#pragma omp single
        or_kmat_mul_rec(u, H, v, 1, 1);
        return OR_OK;
    }
#endif
    (void)nthreads;
    or_kmat_mul_rec(u, H, v, 1, 1);
    return OR_OK;
}

void or_kernelmatrix_size(const or_block *H, int64_t *mn) { mn[0] = H->m; mn[1] = H->n; }

/* --- tree statistics and leaf-block export ---------------------------------- */

static void or_walk(const or_block *H, int64_t *st)
{
    /* st: [0] barycentric count, [1] dense count, [2] max depth,
       [3] sum of bary rows+cols, [4] dense values, [5] stored values (reference layout) */
    if (H->tag == OR_TAG_KMAT && H->level > st[2]) st[2] = H->level;
    if (H->tag == OR_TAG_BARY) {
        st[0] += 1; st[3] += H->m + H->n;
        st[5] += (H->m + H->n) * H->r + (int64_t)H->r * H->r;
    } else if (H->tag == OR_TAG_DENSE) {
        st[1] += 1; st[4] += H->m * H->n; st[5] += H->m * H->n;
    } else {
        for (int k = 0; k < 4; ++k) or_walk(H->child[k], st);
    }
}

void or_kernelmatrix_stats(const or_block *H, int64_t *st6)
{
    for (int k = 0; k < 6; ++k) st6[k] = 0;
    or_walk(H, st6);
}

typedef struct { int64_t k, cap; int64_t *meta; double *box; } or_export;

static void or_collect(const or_block *H, or_export *e)
{
    if (H->tag == OR_TAG_KMAT) { for (int k = 0; k < 4; ++k) or_collect(H->child[k], e); return; }
    if (e->k < e->cap) {
        int64_t *m = e->meta + 6 * e->k;
        m[0] = H->tag; m[1] = H->i0; m[2] = H->m; m[3] = H->j0; m[4] = H->n; m[5] = H->level;
        for (int q = 0; q < 4; ++q) e->box[4 * e->k + q] = H->box[q];
    }
    e->k += 1;
}

/* Leaf blocks in block-walk order: meta = (tag, i0, m, j0, n, level) per block,
   box = (a, b, c, d) for barycentric blocks.  Returns the number of blocks. */
int64_t or_kernelmatrix_leaves(const or_block *H, int64_t cap, int64_t *meta, double *box)
{
    or_export e = {0, cap, meta, box};
    or_collect(H, &e);
    return e.k;
}

static const or_block *or_find(const or_block *H, int64_t *k)
{
    if (H->tag != OR_TAG_KMAT) { if (*k == 0) return H; *k -= 1; return NULL; }
    for (int q = 0; q < 4; ++q) { const or_block *b = or_find(H->child[q], k); if (b) return b; }
    return NULL;
}

/* Copy the factors of leaf block idx (block-walk order): which = 0 U, 1 V, 2 F, 3 dense A. */
int or_kernelmatrix_block_data(const or_block *H, int64_t idx, int which, double *out)
{
    int64_t k = idx;
    const or_block *b = or_find(H, &k);
    if (!b) return OR_ERR_ARG;
    if (b->tag == OR_TAG_BARY) {
        if (which == 0) memcpy(out, b->U, sizeof(double) * (size_t)(b->m * b->r));
        else if (which == 1) memcpy(out, b->V, sizeof(double) * (size_t)(b->n * b->r));
        else if (which == 2) memcpy(out, b->F, sizeof(double) * (size_t)(b->r * b->r));
        else return OR_ERR_ARG;
    } else {
        if (which != 3) return OR_ERR_ARG;
        memcpy(out, b->A, sizeof(double) * (size_t)(b->m * b->n));
    }
    return OR_OK;
}

/* --- dense FP64 reference with compensated summation ---------------------- */

/* out[q] = sum_j f(x[rows[q]], y[j]) * b[j], products and sums carried in
   double-double (TwoProd via fma, TwoSum), rounded once at the end. */
void or_dense_rows(int kernel, const double *x, const double *y, int64_t ny, const double *b,
                   const int64_t *rows, int64_t nrows, double *out, int nthreads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int64_t q = 0; q < nrows; ++q) {
        double xi = x[rows[q]];
        double s = 0.0, c = 0.0;
        for (int64_t j = 0; j < ny; ++j) {
            double f = or_kernel(kernel, xi, y[j]);
            double p = f * b[j];
            double pe = fma(f, b[j], -p);
            double t = s + p;
            double bp = t - s;
            double se = (s - (t - bp)) + (p - bp);
            s = t;
            c += se + pe;
        }
        out[q] = s + c;
    }
    (void)nthreads;
}
