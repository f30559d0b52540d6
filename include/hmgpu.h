/*
 * hmgpu.h -- C ABI of the GB300-native hierarchical-matrix library (libhmgpu.so).
 *
 * Drop-in boundary for the hot path of HierarchicalMatrices.jl v0.2.2: the
 * KernelMatrix compression of Cauchy-type kernels and the hierarchical
 * matrix-vector product.  Plain pointers and sizes only; every call returns a
 * status code (HM_OK = 0) and never falls back to the CPU.  "device" pointers
 * are CUDA device memory of the current device; "host" pointers are ordinary
 * process memory.  Streams are cudaStream_t passed as void* (NULL = legacy
 * default stream).
 *
 * Each entry point names the reference function it stands in for
 * (file:line within HierarchicalMatrices.jl).
 */
#ifndef HMGPU_H
#define HMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hm_handle hm_handle;

/* Status codes.  The reference reports failures as Julia exceptions; the
   mapping is given per code. */
enum {
    HM_OK = 0,
    HM_ERR_INVALID_ARG = 1,   /* ArgumentError / DimensionMismatch */
    HM_ERR_UNSORTED = 2,      /* points not non-increasing (the reference needs descending order) */
    HM_ERR_BOUNDS = 3,        /* BoundsError (indsplit past the end, vector too short) */
    HM_ERR_NAN = 4,           /* NaN point or box end */
    HM_ERR_CUDA = 5,          /* a CUDA runtime call failed (see hm_last_error) */
    HM_ERR_ALLOC = 6,         /* device allocation failed */
    HM_ERR_UNSUPPORTED = 7,   /* rank above 32, unknown kernel or storage type */
    HM_ERR_BOX = 8,           /* box ends not strictly decreasing (a > b, c > d) */
    HM_ERR_DEGENERATE = 9,    /* a partition the reference itself builds inconsistently */
    HM_ERR_NOT_POSDEF = 10    /* PosDefException: a Cholesky pivot is not positive */
};

/* Kernels of examples/Kernel.jl:34-37. */
enum {
    HM_KERNEL_CAUCHY = 0,         /* 1/(x-y) */
    HM_KERNEL_COULOMB = 1,        /* 1/(x-y)^2 */
    HM_KERNEL_COULOMB_PRIME = 2,  /* 1/(x-y)^3 */
    HM_KERNEL_LOG = 3             /* log|x-y| */
};

/* Storage / arithmetic type of factors, leaves and vectors. */
/* Storage types.  HM_F64 and HM_F32: factors and leaves in FP64 / FP32.
   HM_DF64 (no reference counterpart): the FP64 product with its row-segment
   panels (near-field leaves and row bases, the bulk of the stored values) kept
   as pairs of FP32 values (h, l), h + l within 2^-48 relative of the FP64
   value, and multiplied in double-float arithmetic on the FP32 pipes (GB300's
   FP64 pipe is about 1/56 of its FP32 rate); vectors, the column bases, the
   far-field blocks and the tree passes stay FP64.  Same bytes as HM_F64;
   products agree with HM_F64 to about 1e-14 relative.  Building fails with
   HM_ERR_UNSUPPORTED when a panel value's magnitude reaches 2^127.
   KernelMatrix builds only (not hm_hier_build). */
enum { HM_F64 = 0, HM_F32 = 1, HM_DF64 = 2 };

/* Error reporting (the reference raises Julia exceptions instead: BoundsError
   from indsplit, src/BarycentricMatrix.jl:299-307, and AssertionError from
   update!, :249-250).  Name of a status code. */
const char *hm_status_string(int status);
/* Message of the last failing call on this thread ("" if none). */
const char *hm_last_error(void);
/* Library version number (no reference counterpart). */
int hm_version(void);

/* BLOCKRANK(T) (src/HierarchicalMatrices.jl:5): rank for machine epsilon eps. */
int hm_blockrank(double eps);

/* indsplit(x, ir, a, b) (src/BarycentricMatrix.jl:299-307) on a host point
   list: splits the 0-based range [start, start+len) at the first point below
   (a+b)/2.  out4 = (start1, len1, start2, len2). */
int hm_indsplit(const double *x, int64_t n, int64_t start, int64_t len, double a, double b,
                int64_t *out4);

/* KernelMatrix(f, x, y, a, b, c, d) (src/KernelMatrix.jl:47-116).
   x (nx) and y (ny) are HOST arrays in non-increasing order with a > b, c > d,
   as the reference requires.  rank = BLOCKRANK (0 selects 20), blocksize =
   BLOCKSIZE leaf threshold (0 selects 4*rank).  Compression runs on the GPU in
   FP64; factors and leaves are stored as `storage` (HM_F64, HM_F32 or HM_DF64). */
int hm_kernelmatrix_build(int kernel, const double *x, int64_t nx, const double *y, int64_t ny,
                          double a, double b, double c, double d, int rank, int64_t blocksize,
                          int storage, void *stream, hm_handle **out);

/* Many independent KernelMatrices as one block-diagonal handle (no
   counterpart in the reference, which builds one matrix per call).
   Instance i has nx[i] rows and ny[i] columns; x (sum nx) and y (sum ny) are
   the instances' HOST point lists concatenated, each non-increasing, and
   boxes holds (a, b, c, d) per instance.  hm_mul on the handle multiplies
   every instance at once: rows and columns of instance i follow those of
   instances 0..i-1 in u and v.  Planning runs on all host cores. */
int hm_kernelmatrix_batch_build(int kernel, int ninst, const int64_t *nx, const int64_t *ny,
                                const double *x, const double *y, const double *boxes, int rank,
                                int64_t blocksize, int storage, void *stream, hm_handle **out);

/* A user-assembled HierarchicalMatrix (src/HierarchicalMatrix.jl:1, built with
   H[Block(m), Block(n)] = ..., src/hierarchical.jl:149-172), flattened to its
   nblocks leaf blocks.  Block i occupies rows [row0, row0+rows) and columns
   [col0, col0+cols) -- the offsets of the reference's block walk
   (src/HierarchicalMatrix.jl:24-52) -- and its FP64 data starts at
   values + offsets[i] (HOST memory):
     kind 0 Matrix:              A, rows x cols, column-major
     kind 1 LowRankMatrix:       U (rows x r), sigma (r), V (cols x r)   (src/LowRankMatrix.jl:28-33)
     kind 2 BarycentricMatrix2D: U (rows x r), F (r x r), V (cols x r)   (src/BarycentricMatrix.jl:208-218)
   ranks[i] = r (ignored for kind 0).  Blocks may overlap; their products add
   up like the reference's walk.  hm_mul / hm_mul_strided then run the
   product y += H x; transposed and derivative products are not available. */
int hm_hier_build(int storage, int64_t m, int64_t n, int nblocks, const int32_t *kinds,
                  const int64_t *row0, const int64_t *rows, const int64_t *col0, const int64_t *cols,
                  const int64_t *ranks, const double *values, const int64_t *offsets, void *stream,
                  hm_handle **out);

/* Block-level products on DEVICE arrays of type dtype (HM_F64 / HM_F32),
   1-based starts and positive increments like the reference; x and y
   lengths are checked (HM_ERR_BOUNDS).  All accumulate into y.
   hm_dense_mul: trans = 0: mul!(y, A, x, istart, jstart, INCX, INCY)
   (src/algebra.jl:37-48); trans = 1: mul!(y, transpose(A), ...)
   (src/algebra.jl:52-65; the adjoint of real data, :69-82, is the same).
   A is m x n column-major with leading dimension lda. */
int hm_dense_mul(int trans, int dtype, const void *A, int64_t m, int64_t n, int64_t lda,
                 const void *x, int64_t lenx, int64_t jstart, int64_t incx, void *y, int64_t leny,
                 int64_t istart, int64_t incy, void *stream);

/* chebyshevpoints(T, n) and chebyshevbarycentricweights(T, n), first kind,
   in FP64 (src/BarycentricMatrix.jl:92-136): the nodes and weights of every
   barycentric factor the library builds. */
int hm_chebyshev(int n, double *x, double *lambda);

/* y += U C V^T x (adjoint = 0) or y += V C^T U^T x (adjoint = 1) with U m x r
   and V n x r column-major; C = diag(core) when core_diag (LowRankMatrix
   mul! and its adjoint, src/algebra.jl:110-131, 137-159) or the r x r
   column-major core (BarycentricMatrix2D mul!, src/algebra.jl:243-277). */
int hm_lowrank_mul(int adjoint, int dtype, const void *U, const void *core, int core_diag,
                   const void *V, int64_t m, int64_t n, int64_t r, const void *x, int64_t lenx,
                   int64_t jstart, int64_t incx, void *y, int64_t leny, int64_t istart, int64_t incy,
                   void *stream);

/* BarycentricMatrix2D(T, f, a, b, c, d, x, y, ir, jr) factors
   (src/BarycentricMatrix.jl:147-178, 236-297) for the HOST points x (nx) and
   y (ny) of the block: U (nx x rank), F (rank x rank), V (ny x rank), all
   column-major DEVICE arrays of type dtype, computed in FP64.  Synchronous. */
int hm_bary_factors(int kernel, int rank, double a, double b, double c, double d, const double *x,
                    int64_t nx, const double *y, int64_t ny, int dtype, void *U, void *F, void *V,
                    void *stream);

/* size(H) (src/hierarchical.jl:33-47). */
int hm_size(const hm_handle *h, int64_t *m, int64_t *n);
/* Storage type of h (HM_F64 / HM_F32 / HM_DF64): the element type T of the
   KernelMatrix{T} type of src/KernelMatrix.jl:1, plus the DF64 form. */
int hm_storage(const hm_handle *h);

/* Statistics (no reference counterpart; the block counts are those of the
   tree src/KernelMatrix.jl:47-116 builds):
   out[0..] = barycentric blocks, dense blocks, tree depth, row slots,
   column slots, canonical stored values, reference-layout values, values this
   build stores, dense values, row segments, max panel width, device bytes,
   kernel launches per single-RHS hm_mul with the side stream on (the default).
   Returns the number of values written (<= nout). */
int hm_stats(const hm_handle *h, int64_t *out, int nout);

/* Device-side status of h's kernels (and of its transpose, once built):
   0 when clean, 1 (HM_DEV_WAIT_TIMEOUT) when a streaming kernel gave up
   waiting for a shared-memory stage copy (its products are then invalid).
   Synchronises the device; reset != 0 clears the word.  No reference
   counterpart (Julia raises inside mul!). */
int hm_device_status(hm_handle *h, int *code, int reset);

/* mul!(u, H, v, istart, jstart) (src/KernelMatrix.jl:14-45), generalised to
   nrhs right-hand sides: for q < nrhs,
     u[:, q] += H * v[:, q]   (accumulate = 1, the reference's semantics)
     u[:, q]  = H * v[:, q]   (accumulate = 0)
   u, v are DEVICE arrays of the handle's storage type, column q at u + q*ldu.
   Stream-ordered; returns before the work completes.  Internally the tree
   passes run on a side stream forked from and joined back into `stream`.
   nrhs = 0 reads and writes nothing (u and v may then be NULL), here and in
   hm_mul_t, hm_mul_drow and hm_mul_host. */
int hm_mul(hm_handle *h, const void *v, int64_t ldv, void *u, int64_t ldu, int nrhs,
           int accumulate, void *stream);

/* u (+)= H^T v: the transposed product (the role of the Transpose/Adjoint
   block mul! of src/algebra.jl:50-82 and :133-159 for the whole KernelMatrix;
   the reference itself has no transposed KernelMatrix product).  Same
   arguments as hm_mul with u of length ny and v of length nx.  The first
   call builds the transposed plan (the reference's tree of (y, x) is the
   transpose of the tree of (x, y)) and keeps it with the handle. */
int hm_mul_t(hm_handle *h, const void *v, int64_t ldv, void *u, int64_t ldu, int nrhs,
             int accumulate, void *stream);

/* Row-derivative product (no counterpart in the reference; the building
   block of the gradients of L(x, y, w) through the kernel and the
   barycentric factors, with the block tree held fixed):
     transposed = 0:  u (+)= D_x v,    D_x[i, j] = d H[i, j] / d x_i
     transposed = 1:  u (+)= D_y^T v,  D_y[i, j] = d H[i, j] / d y_j
   Near-field entries differentiate the kernel, far-field rows the
   barycentric basis U(x_i) (U_m' = U_m (sum_k U_k/(x - xh_k) - 1/(x - xh_m))).
   For L = 1/2 |H w - t|^2 with r = H w - t:  dL/dx = r .* (D_x w),
   dL/dy = w .* (D_y^T r), dL/dw = H^T r.  The derivative panels are filled
   on the first call and kept (the same device memory as the panels). */
int hm_mul_drow(hm_handle *h, int transposed, const void *v, int64_t ldv, void *u, int64_t ldu,
                int nrhs, int accumulate, void *stream);

/* mul!(y, H, x, istart, jstart, INCX, INCY) (src/HierarchicalMatrix.jl:24-52):
   y[istart-1 + i*incy] += (H x)[i] with x read at x[jstart-1 + j*incx]
   (1-based istart/jstart, positive strides).  lenx/leny are the array
   lengths, checked like the reference's BoundsError.  DEVICE arrays. */
int hm_mul_strided(hm_handle *h, const void *x, int64_t lenx, int64_t jstart, int64_t incx,
                   void *y, int64_t leny, int64_t istart, int64_t incy, void *stream);

/* H * v with HOST arrays (u = H v or u += H v; the reference's
   mul!(u, K, v) and K * v on Julia arrays, src/KernelMatrix.jl:5-45):
   copies v to the device, runs hm_mul and brings the result back;
   synchronous.  When u is page-locked (cudaHostAlloc / cudaHostRegister)
   and the product ends by combining its near and far fields, that last
   kernel writes u directly; otherwise the result is copied back.  When v is
   page-locked, the leaf panels cover every row of v once and the near field
   starts after the leaf stage, the leaf stage reads v from the host and
   stores it on the device as it goes, instead of a copy before the product.
   The launches are replayed from a CUDA graph from the second call with the
   same right-hand-side count, accumulate flag and destination. */
int hm_mul_host(hm_handle *h, const void *v, void *u, int nrhs, int accumulate);

/* Exact dense rows: out[q] = sum_j f(x[rows[q]], y[j]) b[j] evaluated in FP64
   with double-double accumulation, on the handle's points (DEVICE b, rows,
   out).  Used to state the error of a compressed product (the reference's
   own check multiplies the dense Matrix(K), examples/Kernel.jl:73-78). */
int hm_direct_rows(hm_handle *h, const double *b, const int64_t *rows, int64_t nrows, double *out,
                   void *stream);

/* Handle options.  HM_OPT_OVERLAP (default 2): 1 runs the tree passes of
   hm_mul on a side stream concurrently with the near-field panels from the
   start, 2 starts the near field after the upward pass, 3 after the
   far-field (M2L) stage, 4 after the leaf-basis stage of the upward pass; 0
   runs every stage in order on the caller's stream. */
enum {
    HM_OPT_OVERLAP = 1,
    /* HM_OPT_NEAR_STAGES (default 4, 2..16): shared-memory stages (8 KB each)
       of the near-field streaming kernel.  Values whose shared memory does
       not fit the kernel's CTAs per SM fall back to the largest that does. */
    HM_OPT_NEAR_STAGES = 2,
    /* HM_OPT_TENSOR_CORES (default 1): FP32 products with 16 or more
       right-hand sides run their row-segment panels on the tensor cores
       (every FP32 value split exactly into three BF16 pieces, six products
       per step, FP32 accumulation); 0 keeps them on the FP32 pipes. */
    HM_OPT_TENSOR_CORES = 3,
    /* HM_OPT_NEAR_KERNEL (default 0): near-field and far-field panels with up
       to 8 right-hand sides on 0 = per-warp rings for 3-8 FP32 right-hand
       sides and one warp per row segment otherwise, 1 = one warp per row
       segment, 2 = CTAs streaming runs of segments through shared memory
       (cp.async.bulk), 3 = per-warp rings (warps streaming runs of segments
       through shared-memory stages with cp.async; FP32 with 3-8 right-hand
       sides, otherwise as 0). */
    HM_OPT_NEAR_KERNEL = 4,
    /* HM_OPT_AUTOTUNED: value 0 forgets the schedules hm_autotune chose, so
       every product runs with the options above again.  Setting any other
       option forgets them too. */
    HM_OPT_AUTOTUNED = 5,
    /* HM_OPT_PDL (default 1 for FP32 storage, 0 for FP64): the kernels of the tree passes (and the
       far-field rows after them) are launched as programmatic dependents of
       the kernel before them on the stream, so that each is scheduled while
       its predecessor finishes and stages its constant inputs before it waits
       for the predecessor's results; 0 launches them plainly. */
    HM_OPT_PDL = 6,
    /* HM_OPT_WAIT_LIMIT_NS (default 2e9, 1..2e9): nanoseconds after which a
       wait of the streamed near-field kernel (HM_OPT_NEAR_KERNEL 2) or of the
       tensor-core panel kernel on its copies or MMAs gives up: the CTA
       records HM_DEV_WAIT_TIMEOUT (hm_device_status), lets what it has in
       flight land (bounded by 0.2 s), releases its tensor memory and returns;
       the product's output is then invalid.  Keeps autotuned schedules.
       No reference counterpart. */
    HM_OPT_WAIT_LIMIT_NS = 7,
    /* HM_OPT_TEST_STALL (default 0): test hook for that give-up path.  With 1,
       the first wait of every CTA of those two kernels waits on a barrier
       nothing arrives on, so it runs out after HM_OPT_WAIT_LIMIT_NS.  Keeps
       autotuned schedules.  No reference counterpart. */
    HM_OPT_TEST_STALL = 8,
    /* HM_OPT_WIDE_TREE (default 1): products with 32 or more right-hand sides
       (rank 20) run the tree passes (leaf bases, transfers, far-field blocks)
       on kernels that give each lane one right-hand side and all 20
       coefficients of it (a warp of 32, or 2 or 4 groups of 16 or 8 lanes);
       2 uses them from 2 right-hand sides on; 0 keeps the kernels with the
       coefficients on the lanes and chunks of 8 right-hand sides.  Applies to
       the autotuned schedules too (it overrides their choice; the autotuner
       tries 1 and 2 for 2-31 right-hand sides, 1 and 0 from 32).  No reference
       counterpart. */
    HM_OPT_WIDE_TREE = 9,
    /* HM_OPT_RING_TILE (default 0): the per-warp rings' tile for 3-8 FP32
       right-hand sides: 0 = up to 768 panel values x 3 stages per warp,
       1 = 512 x 4, 2 = 1024 x 3.  No reference counterpart. */
    HM_OPT_RING_TILE = 10
};
int hm_configure(hm_handle *h, int option, int64_t value);

/* Autotuner (no counterpart in the reference, which has one serial loop).
   Times every candidate schedule of a product with nrhs right-hand sides
   on `stream` (reps products each, CUDA events, after two warm-up products,
   two rounds with the better time kept) and keeps the fastest for nrhs's
   bucket (1, 2, 3-4, 5-8, 9-16, 17-32, 33-64, 65-128, 129+): later hm_mul,
   hm_mul_strided, hm_mul_host and hm_mul_drow calls of that bucket run with
   it, including inside stream capture.  Candidates: HM_OPT_OVERLAP 0..4
   (0..1 above 8 right-hand sides), HM_OPT_NEAR_KERNEL 0 (with each of the
   three ring tiles for 3-8 FP32 right-hand sides), 1 (FP32 with 3-8
   right-hand sides) or 2 with HM_OPT_NEAR_STAGES 3, 4 or 6 (up to 8
   right-hand sides), HM_OPT_WIDE_TREE on or off (32 or more),
   HM_OPT_TENSOR_CORES
   on or off (FP32, 16 or more), HM_OPT_PDL on or off.  Inputs are scratch vectors allocated on
   `stream` and freed before return; synchronous; not allowed while `stream`
   is being captured.  choice (host, 5 values, may be NULL) receives the
   chosen overlap, near kernel, near stages, tensor-core flag and PDL flag; ms (host, 2
   values, may be NULL) the chosen schedule's time per product and that of
   the configured options.  Like hm_configure, it changes the handle: do not
   call it while products on the same handle are being issued from other
   host threads. */
int hm_autotune(hm_handle *h, int nrhs, int reps, void *stream, int32_t *choice, double *ms);

/* The schedule products with nrhs right-hand sides run with (hm_autotune's
   choice for nrhs's bucket, else the configured options): out[0..6] =
   overlap, near kernel, near stages, tensor-core flag, PDL flag, ring tile
   (0: 768 panel values x 3 stages per warp, 1: 512 x 4, 2: 1024 x 3; for 3-8
   FP32 right-hand sides) and the lane-per-right-hand-side tree flag (32+).
   Returns the number of values written (<= nout), or minus a status.  No
   reference counterpart. */
int hm_autotune_choice(const hm_handle *h, int nrhs, int32_t *out, int nout);

/* Test hook for the allocation-failure paths (no reference counterpart: the
   reference allocates through Julia's GC).  after >= 0: the next `after`
   device allocations of the library (cudaMalloc / cudaMallocAsync, builds,
   per-stream scratch, staging, the autotuner's vectors, the algebra's
   workspaces) succeed and the one after them fails with HM_ERR_ALLOC without
   calling CUDA; the hook then disarms itself.  after = -1 disarms it.
   Process-wide.  Every entry point that allocates returns HM_ERR_ALLOC from
   such a failure and frees what it had allocated. */
int hm_debug_fail_alloc(int64_t after);

/* Allocation-free single right-hand-side product.  No counterpart in the
   reference: it is an addition for callers that cannot let a library
   allocate device memory while they run — processes whose GPU memory is
   claimed up front by another allocator (a framework memory pool), and
   loops that must not call cudaMalloc/cudaFree after start-up because those
   calls can synchronise the whole device.
     u (+)= H v   (accumulate = 1 adds, as the reference's mul!; 0 overwrites)
   u, v: DEVICE vectors of the handle's storage type (lengths nx, ny); all
   stages run in order on `stream`.
   Scratch: a 16 MiB array compiled into the library (a file-scope __device__
   array, held by every GPU that loads the library until the process exits).
   A matrix whose coefficients need more, (n_yslots + n_xslots) * rank
   elements with each part rounded up to 256 bytes, is rejected with
   HM_ERR_UNSUPPORTED (hm_mul has no such limit).  Each call writes every
   coefficient before reading it, so nothing has to start at zero, but all
   calls share the one array: calls that overlap on the GPU (other streams,
   or other handles, at the same time) race and give wrong results.
   The first call on each device looks up the array's device address with
   cudaGetSymbolAddress (that device current) and caches it for the life of
   the process; make that first call before any stream capture.  A device
   reset (cudaDeviceReset) can move the array: after one, load the library
   afresh before calling again.  The device current at the call must be the
   one the handle was built on (HM_ERR_INVALID_ARG otherwise).  The call runs
   the schedule hm_mul would pick for one right-hand side (hm_autotune's, when
   it ran) with every stage on `stream`.  It makes no cudaMalloc, cudaFree or
   other allocating call. */
int hm_mul_noalloc(hm_handle *h, const void *v, void *u, int accumulate, void *stream);

/* Per-stage timing of hm_mul (the reference prints @time per call,
   examples/Kernel.jl:73-76): for each stage whose bit is set in stage_mask
   (0 upward pass: leaf bases and transfers, 1 far field and downward
   transfers, 2 near-field panels, 3 far-field panel columns, 4 the whole
   product on the caller's stream), CUDA events are recorded on the stream
   that launches the stage, around its launches.  hm_profile_read synchronises on them and returns accumulated
   milliseconds and launch counts per stage; reset = 1 clears the totals.
   stage_mask = 0 turns timing off. */
int hm_profile(hm_handle *h, int stage_mask);
int hm_profile_read(hm_handle *h, double *ms, int64_t *launches, int n, int reset);
/* Timeline of the pending timed stages (consumed as by hm_profile_read):
   for each, in the order recorded, out[3i] = stage, out[3i+1] = start and
   out[3i+2] = end in ms from the earliest start.  Returns the number of
   records (only the first nmax are written), or a negative status. */
int hm_profile_timeline(hm_handle *h, double *out, int nmax);

/* Releases a handle (Julia's garbage collector, in the reference). */
void hm_free(hm_handle *h);

/* --- host planner (no GPU needed) ------------------------------------------
   The block tree of KernelMatrix (src/KernelMatrix.jl:47-116, split by
   indsplit, src/BarycentricMatrix.jl:299-307) and the flattened tables that
   hm_kernelmatrix_build uploads, for inspection and host-side tests.  Same validation and status codes as
   hm_kernelmatrix_build. */
typedef struct hm_plan hm_plan;
int hm_plan_create(const double *x, int64_t nx, const double *y, int64_t ny, double a, double b,
                   double c, double d, int rank, int64_t blocksize, hm_plan **out);
/* Table `which` (0 vpanels, 1 vpanel boxes, 2 upward steps, 3 upward level
   offsets, 4 far-field rows, 5 far-field entries, 6 F boxes, 7 downward steps,
   8 downward level offsets, 9 row segments, 10 pieces, 11 segment fill info,
   12 transfer matrices, 13 Chebyshev nodes, 14 barycentric weights,
   15-18 upward band records / steps / tasks / band offsets, 19-22 the same
   for the downward bands):
   pointer, element count and element size (records of hm_types.h). */
/* The merged plan of hm_kernelmatrix_batch_build (same arguments). */
int hm_batch_plan_create(int ninst, const int64_t *nx, const int64_t *ny, const double *x,
                         const double *y, const double *boxes, int rank, int64_t blocksize,
                         hm_plan **out);
int hm_plan_table(const hm_plan *p, int which, const void **data, int64_t *count, int64_t *elem_bytes);
/* r, nx, ny, row slots, column slots, V/F/panel store elements, max panel
   width, barycentric blocks, dense blocks, depth, canonical values,
   reference-layout values, stored values, dense values, row segments. */
int hm_plan_sizes(const hm_plan *p, int64_t *out, int nout);
void hm_plan_free(hm_plan *p);

/* ------------------------------------------------------------------------
   Low-rank arithmetic and the blockwise Cholesky (src/LowRankMatrix.jl:70-171,
   src/algebra.jl:394-524, src/hierarchical.jl:174-231, src/cholesky.jl).
   The recursion over blocks runs on the host (hierarchicalmatrices/algebra.py);
   these batched calls do the arithmetic on the GPU.  All matrices are
   column-major DEVICE arrays of type dtype (HM_F64 or HM_F32), descriptors
   and result arrays are HOST arrays.  Calls marked synchronous return after
   the stream has finished the work.
   ------------------------------------------------------------------------ */

/* One truncated SVD of a product  X = P M Q^T  (the common core of every
   LowRankMatrix operation of src/LowRankMatrix.jl:82-158):
     P = [P1 P2]  m x (a1 + a2)       Q = [Q1 Q2]  n x (b1 + b2)
     M = diag(s1 ; sign2 * s2)        when Xm == NULL (then a1 + a2 == b1 + b2)
     M = diag(s1) Xm^T Ym diag(s2)    otherwise (Xm t x a1, Ym t x b1; a2 = b2 = 0)
   qr_left / qr_right: orthonormalise P / Q by Householder QR first, as the
   reference's qr! does (the sum, A*L and L*A forms); without QR the factor is
   used as given (the L1*L2 and L1'*L2 forms).  Q1 == NULL stands for the
   identity (n == b1, b2 == 0, qr_right == 0: svdtrunc of a dense P).
   The core (R_P M R_Q^T, or M) is ka x kb with ka = qr_left ? min(m, a) : a
   and kb likewise; its singular values are q = min(ka, kb).  Cores up to
   about HM_LR_KMAX x HM_LR_KMAX are factored in shared memory, larger ones
   (up to 4096 x 4096) from a global-memory workspace.  Outputs: U (m x q, ld m), s (q) and V
   (n x q, ld n) receive the first r columns / values in descending order,
   r = getrank(sigma) = #{sigma_j > q * eps(sigma_1)} (src/LowRankMatrix.jl:70-80). */
#define HM_LR_KMAX 96
typedef struct {
    int64_t m, n, t;
    int32_t a1, a2, b1, b2;
    int32_t qr_left, qr_right;
    const void *P1, *P2, *Q1, *Q2;
    int64_t ldp1, ldp2, ldq1, ldq2;
    const void *s1, *s2;
    double sign2;
    const void *Xm, *Ym;
    int64_t ldx, ldy;
    void *U, *s, *V;
} hm_lr_problem;

/* Batched truncated SVDs (one CTA per problem).  ranks (host, nprob) receives
   r per problem.  Synchronous. */
int hm_lr_svd(int dtype, int nprob, const hm_lr_problem *probs, int32_t *ranks, void *stream);

/* D = beta C + alpha P diag(s) Q^T with P m x k (or its transpose stored k x m
   when transp), Q n x k (or k x n when transq), s = NULL for ones, C = NULL
   for C = D (C may also equal D); beta = 0 never reads C.  Covers Matrix -/+
   LowRankMatrix blocks of H -/+ L (src/algebra.jl:460-524), A22 - R12'R12
   for a dense R12 (src/cholesky.jl:40-56) and the dense products A*L.U,
   A'*L.V of src/LowRankMatrix.jl:128-142. */
typedef struct {
    int64_t m, n, k;
    const void *P; int64_t ldp; int32_t transp;
    const void *Q; int64_t ldq; int32_t transq;
    const void *s;
    double alpha, beta;
    const void *C; int64_t ldc;
    void *D; int64_t ldd;
} hm_gemm_problem;
int hm_gemm_batched(int dtype, int nprob, const hm_gemm_problem *probs, void *stream);

/* D[i, j] = alpha dr[i] A[i, j] dc[j] + beta B[i, j] (m x n blocks; dr, dc =
   NULL for ones; B = NULL when beta = 0): Matrix +/- Matrix of H +/- H
   (src/hierarchical.jl:174-231), Diagonal * L.U and L.V * Diagonal
   (src/LowRankMatrix.jl:144-158), scalar * L (:160-171) and block copies. */
typedef struct {
    int64_t m, n;
    const void *A; int64_t lda;
    const void *B; int64_t ldb;
    const void *dr, *dc;
    double alpha, beta;
    void *D; int64_t ldd;
} hm_axpby_problem;
int hm_axpby_batched(int dtype, int nprob, const hm_axpby_problem *probs, void *stream);

/* hierarchicalcholesky(A::Matrix) = Matrix(cholesky(Symmetric(A)).U)
   (src/cholesky.jl:16-18): R (n x n, ld ldr) = the upper Cholesky factor of
   the symmetric matrix whose upper triangle is A's (A n x n, ld lda), zeros
   below the diagonal; R may equal A.  info (host, nprob): 0, or j >= 1 when
   the j-th pivot is not positive (then the call returns HM_ERR_NOT_POSDEF).
   Synchronous. */
typedef struct {
    int64_t n;
    const void *A; int64_t lda;
    void *R; int64_t ldr;
} hm_potrf_problem;
int hm_potrf_batched(int dtype, int nprob, const hm_potrf_problem *probs, int32_t *info, void *stream);
/* The same without waiting: d_info is a DEVICE array (nprob values) that the
   kernel fills with 0 or the failing pivot j >= 1; the caller reads it later
   (hierarchicalcholesky reads the words of all its leaves once, at the end,
   and raises for the first failing leaf as src/cholesky.jl:16-18 would).
   Returns after the launch is queued. */
int hm_potrf_batched_async(int dtype, int nprob, const hm_potrf_problem *probs, int32_t *d_info, void *stream);

/* solvetransposed(R, B) (src/cholesky.jl:97-228): B <- R^{-T} B in place for
   the ncols columns of B (ld ldb), R an upper block-triangular hierarchical
   matrix given as its forward-substitution schedule, ops in the order of the
   reference's recursion:
     HM_SOLVE_TRSM   x[o1 : o1+n1) <- R^{-T} x[..]          (A = R, n1 x n1 upper, ld)
     HM_SOLVE_LR     x[o2 : o2+n2) -= V diag(s) U^T x[o1 : o1+n1)
                                                              (A = U n1 x r ld, B = V n2 x r ld2)
     HM_SOLVE_DENSE  x[o2 : o2+n2) -= M^T x[o1 : o1+n1)       (A = M n1 x n2, ld)
     HM_SOLVE_INV    x[o1 : o1+n1) <- W^T x[..], W = R^{-1}  (A = W, n1 x n1 upper, ld;
                                                              n1 <= 256; from hm_trtri_batched)
     HM_SOLVE_LTRSM  x[o1 : o1+n1) <- L^{-1} x[..], L = R^T  (A = L, n1 x n1 lower, ld;
                                                              n1 <= 256: forward substitution
                                                              reading L's columns contiguously)
   One CTA per column of B runs the ops in order.  HM_SOLVE_INV turns the
   serial forward substitution of a diagonal block into one parallel product
   (GB300's FP64 rate makes a one-warp substitution slow). */
enum { HM_SOLVE_TRSM = 0, HM_SOLVE_LR = 1, HM_SOLVE_DENSE = 2, HM_SOLVE_INV = 3, HM_SOLVE_LTRSM = 4 };
typedef struct {
    int32_t kind, r;
    int64_t o1, n1, o2, n2, ld, ld2;
    const void *A, *s, *B;
} hm_solve_op;
/* W = R^{-1} for upper triangular blocks (W upper, zeros below the diagonal),
   one CTA per block in shared memory: blocks up to 112 rows in FP64 and 159
   in FP32 (larger ones: HM_ERR_UNSUPPORTED).  Used once per diagonal leaf of
   a hierarchical Cholesky factor, so that solvetransposed applies each leaf
   as a product (HM_SOLVE_INV).  Asynchronous. */
typedef struct {
    int64_t n;
    const void *R; int64_t ldr;
    void *W; int64_t ldw;
} hm_trtri_problem;
int hm_trtri_batched(int dtype, int nprob, const hm_trtri_problem *probs, void *stream);

int hm_solve_transposed(int dtype, int nops, const hm_solve_op *ops, void *B, int64_t ldb, int64_t ncols,
                        void *stream);

/* hierarchicalcholesky(A) (src/cholesky.jl:12-92) of a whole HODLR tree in
   one call, the recursion run natively.  The tree is a node list: node i
   covers n rows; a leaf (left = right = -1) holds its dense diagonal block D
   (n x n, ld ldd; the upper triangle is read); an internal node splits its
   rows n1 + (n - n1) between its children left and right and holds its upper
   off-diagonal block A12 = U diag(s) V^T (U n1 x r, V (n - n1) x r, r >= 0).
   Every block of A22 is updated when its ancestor is reached and the blocks
   are factored in the reference's order; A12 - R12'R12 updates take
   R12'R12 = V H V^T whole (H = diag(s) X^T X diag(s), X = R11^{-T} U) into
   one truncated SVD per block.  The inputs are only read.  On success *ctx
   owns the factor (free with hm_hchol_free): hm_hchol_result gives, per
   node, R12 = U diag(s) V^T (rank r; U n1 x r, V (n - n1) x r) or the leaf's
   upper factor R (n x n) and, for leaves up to 112 rows (FP64; 159 FP32),
   W = R^{-1}.  A leaf that is not positive definite: HM_ERR_NOT_POSDEF with
   fail = {node, pivot} of the first such leaf in the reference's order, no
   context.  Synchronous.  The A22 updates' truncated SVDs run on a second
   stream of the library's and overlap with the leaf factorisations and solves
   on `stream`; the host reads a block's new rank when it next uses it. */
typedef struct {
    int64_t n, n1;
    int32_t left, right;
    const void *D; int64_t ldd;
    const void *U; int64_t ldu;
    const void *s;
    const void *V; int64_t ldv;
    int32_t r;
} hm_hchol_node;
typedef struct {
    int32_t r;
    void *U; int64_t ldu;
    void *s;
    void *V; int64_t ldv;
    void *R; int64_t ldr;
    void *W; int64_t ldw;
} hm_hchol_out;
int hm_hchol_factor(int dtype, int nnodes, const hm_hchol_node *nodes, int32_t root, void **ctx, int32_t *fail,
                    void *stream);
int hm_hchol_result(void *ctx, int32_t node, hm_hchol_out *out);
int hm_hchol_free(void *ctx);

#ifdef __cplusplus
}
#endif

#endif /* HMGPU_H */
