/*
 * fmgpu.h -- C ABI of the GB300 (sm_103a) structured-operator matvec engine.
 *
 * The engine replaces the compute behind fastmat's Matrix.forward /
 * Matrix.backward for Circulant, Toeplitz, Fourier, Hadamard, Kron and the
 * Diag / Partial / Permutation / Product / Sum / Hermitian / Conjugate
 * compositions that chain them.  An operator tree is described to the library
 * as a flat array of fm_node records; the library compiles it into a plan
 * (a short list of fused CUDA launches plus the device constants they read)
 * that is executed on column-major (Fortran-order) data, one column per
 * right-hand side, exactly as fastmat lays out its 2-D arrays.
 *
 * Every entry point returns an int status (FM_OK == 0).  On failure
 * fm_last_error() returns a message for the calling thread.  Nothing in this
 * interface uses C++ or torch types.
 *
 * Reference interfaces replaced (paths relative to the fastmat project root):
 *   fm_plan_create   <- the operator constructors that precompute transform
 *                       state: Fourier.__init__ (fastmat/Fourier.pyx:63-161),
 *                       Circulant.__init__ (fastmat/Circulant.pyx:63-227),
 *                       Toeplitz.__init__ (fastmat/Toeplitz.pyx:79-322),
 *                       Hadamard.__init__ (fastmat/Hadamard.pyx:113-133),
 *                       Kron.__init__ (fastmat/Kron.pyx:79-129)
 *   fm_execute       <- Matrix.forward / Matrix.backward and the _forwardC /
 *                       _backwardC hooks they dispatch to
 *                       (fastmat/Matrix.pyx:1819-1829, 1844-1910,
 *                        1912-1922, 1937-2007)
 *   fm_execute_host  <- the same, called with host (numpy) buffers as
 *                       fastmat's _forwardC(arrX, arrRes, ...) receives them
 *                       (fastmat/Matrix.pyx:1892-1901)
 *   fm_plan_destroy  <- instance deallocation (operators are immutable,
 *                       fastmat/Matrix.pyx:341-358)
 */
#ifndef FMGPU_H
#define FMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FM_OK 0
#define FM_ERR_VALUE 1        /* bad shape / argument   -> ValueError        */
#define FM_ERR_TYPE 2         /* unsupported dtype      -> TypeError         */
#define FM_ERR_UNSUPPORTED 3  /* not implemented case   -> NotImplementedError*/
#define FM_ERR_CUDA 4         /* CUDA runtime failure   -> RuntimeError      */
#define FM_ERR_NOMEM 5        /* device allocation fail -> MemoryError       */
#define FM_ERR_TIMEOUT 6      /* a bounded device wait gave up               */

/* ---- element types: same numbering as fastmat's ftype
 *      (fastmat/core/types.pxd:45-55) ------------------------------------- */
#define FM_I8 0
#define FM_I16 1
#define FM_I32 2
#define FM_I64 3
#define FM_F32 4
#define FM_F64 5
#define FM_C64 6
#define FM_C128 7

/* ---- operator node kinds ------------------------------------------------ */
#define FM_NODE_FOURIER 1      /* n = order                                   */
#define FM_NODE_CIRCULANT 2    /* vec0 = defining column c (len0 = n)         */
#define FM_NODE_TOEPLITZ 3     /* vec0 = column (len0 = rows), vec1 = row
                                  vector (len1 = cols - 1), fastmat order
                                  T[0, j] = vecR[-j]                          */
#define FM_NODE_HADAMARD 4     /* n = order (size 2^n)                        */
#define FM_NODE_DIAG 5         /* vec0 = diagonal                             */
#define FM_NODE_PARTIAL 6      /* one child; vec0 = row indices (int64) or
                                  NULL, vec1 = column indices (int64) or NULL */
#define FM_NODE_PERMUTATION 7  /* vec0 = sigma (int64)                        */
#define FM_NODE_PRODUCT 8      /* children applied right to left, times
                                  (scalar_re + i scalar_im)                   */
#define FM_NODE_SUM 9          /* children summed                             */
#define FM_NODE_KRON 10        /* children = square factors, factor 0 is the
                                  most significant index (np.kron order)      */
#define FM_NODE_HERMITIAN 11   /* one child; forward <-> backward             */
#define FM_NODE_CONJUGATE 12   /* one child; conj o child o conj              */
#define FM_NODE_EYE 13         /* identity of size rows                       */
#define FM_NODE_DENSE 14       /* vec0 = rows x cols matrix, column-major     */
#define FM_NODE_BLOCKS 15      /* n = number of block rows R; children = the
                                  R x C blocks row by row, -1 for a zero
                                  block (every block row and block column
                                  holds at least one block); blocks of a row
                                  share their height, of a column their
                                  width (fastmat's Blocks and BlockDiag)     */
#define FM_NODE_SPARSE 16      /* CSR matrix: n = number of nonzeros, vec0 =
                                  the n values, vec1 = int64 row pointers
                                  (rows + 1) followed by the n column
                                  indices (len1 = rows + 1 + n)             */

typedef struct fm_node {
    int32_t kind;
    int32_t dtype;          /* the operator's fastmat dtype (FM_*)            */
    int64_t rows, cols;     /* operator shape                                 */
    int32_t first_child;    /* index into the children array                  */
    int32_t num_children;
    int64_t n;              /* kind-specific size (order, ...)                */
    const void *vec0;       /* host pointer, kind-specific, copied at create  */
    int64_t len0;
    int32_t type0;          /* FM_* element type of vec0                      */
    int32_t pad0;
    const void *vec1;
    int64_t len1;
    int32_t type1;
    int32_t pad1;
    double scalar_re, scalar_im;
} fm_node;

/* compute types accepted by fm_plan_create besides the FM_* element types:
 * float64 / complex128 data computed in double-float arithmetic (pairs of
 * float32, about 2^-48 relative precision) on the FP32 pipes, which this GPU
 * runs far faster than its FP64 pipe; buffers keep float64 / complex128 */
#define FM_F64_DF 16
#define FM_C128_DF 17
/* float32 data whose Hadamard transforms run their 16-point groups on the
 * tensor cores: each group is a 16 x 16 +-1 matrix product in BF16 with
 * FP32 accumulation, the float32 operand split exactly into three BF16
 * terms (relative error of the order of float32's); everything else in
 * float32.  Buffers are float32. */
#define FM_F32_TC 18

/* plan precisions */
#define FM_PREC_NATIVE 0  /* compute in the operator/input promoted type     */
#define FM_PREC_FP32 1    /* opt-in: float32 / complex64 arithmetic          */

/* directions */
#define FM_FORWARD 0
#define FM_BACKWARD 1

typedef struct fm_plan fm_plan;

/* Compile an operator tree.  `compute_type` is the element type the plan
 * computes and stores intermediates in (FM_F32, FM_F64, FM_C64, FM_C128 or
 * FM_I64 for integer-only trees, or one of the forms below).  A tree that
 * only moves data (Permutation, Partial, Eye, Hermitian, Conjugate, scalars
 * +-1 / +-i, and Product / Sum / Kron / Blocks of such trees) computes in
 * its I/O type even when FM_F64_DF, FM_C128_DF or FM_F32_TC is asked for:
 * its outputs are then input elements bit for bit (or IEEE sums of them, in
 * fastmat's order), as fastmat's gathers produce them
 * (fastmat/Permutation.pyx:120-124, fastmat/Partial.pyx:268-294).  Node
 * vectors are host pointers, copied during the call; the caller may free
 * them afterwards.  Device constants (spectra, chirps, twiddles, index
 * maps) are built on the current device, the plan's device: every call
 * that launches work for the plan must be made with that device current
 * (FM_ERR_VALUE otherwise), except fm_execute_host, which switches to it. */
int fm_plan_create(const fm_node *nodes, int32_t num_nodes,
                   const int32_t *children, int32_t num_children,
                   int32_t root, int32_t compute_type, fm_plan **out_plan);

/* y = A x (FM_FORWARD) or y = A^H x (FM_BACKWARD) on `num_cols` columns.
 * x and y are DEVICE pointers, column-major with leading dimensions ld_x /
 * ld_y (in elements).  x may have any FM_* element type (it is converted in
 * the first launch); y has element type y_type.  x is never written.  x and y
 * must not overlap.  Runs asynchronously on `stream` (a cudaStream_t, NULL =
 * default stream); a plan must not run on two streams at once. */
int fm_execute(fm_plan *plan, int32_t direction,
               const void *x, int32_t x_type, int64_t ld_x,
               void *y, int32_t y_type, int64_t ld_y,
               int64_t num_cols, void *stream);

/* Same as fm_execute, but records a CUDA event around every launch and
 * writes each launch's elapsed milliseconds into ms[0 .. *num_launches-1]
 * (capacity given in *num_launches on entry).  Synchronises the stream.
 * Instrumentation for benchmarks; it has no counterpart in the reference. */
int fm_execute_profiled(fm_plan *plan, int32_t direction,
                        const void *x, int32_t x_type, int64_t ld_x,
                        void *y, int32_t y_type, int64_t ld_y,
                        int64_t num_cols, void *stream, float *ms,
                        int32_t *num_launches);

/* ---- execution without device allocation ------------------------------
 * fm_execute_static runs a plan exactly like fm_execute, but never allocates
 * device memory during the call.  It exists for callers that must not call
 * cudaMalloc/cudaFree while they run: code that works inside a fixed memory
 * budget because another allocator (for example a framework's caching
 * allocator) has already reserved the device memory, and latency-critical
 * loops that cannot afford the device-wide synchronisation those calls
 * imply.  fm_execute instead grows a per-plan scratch buffer with cudaMalloc
 * the first time a plan runs on more columns than before.
 *
 * The scratch that multi-launch plans keep between launches (long
 * four-step transforms, Sum) is taken from one fixed array of
 * FM_STATIC_SCRATCH_BYTES (16 MiB) compiled into the library; every GPU that
 * loads the library reserves it until the process exits.  A call whose plan
 * needs more scratch for `num_cols` columns than the array holds returns
 * FM_ERR_VALUE without launching anything.  Plans that need no scratch use
 * none of it.
 *
 * All calls share the one array per device and it keeps whatever the last
 * call left in it; every launch writes the scratch it reads first, so
 * nothing has to be cleared between calls.  Calls whose work overlaps on the
 * GPU (for example on two streams) race on the array: order them.  The first
 * call on each device looks up the array's device address (host code cannot
 * use the symbol directly); make that first call before any stream capture.
 * The plan itself is built beforehand by fm_plan_create, which does
 * allocate.  This entry point has no counterpart in the reference. */
#define FM_STATIC_SCRATCH_BYTES (16u << 20)
int fm_execute_static(fm_plan *plan, int32_t direction,
                      const void *x, int32_t x_type, int64_t ld_x,
                      void *y, int32_t y_type, int64_t ld_y,
                      int64_t num_cols, void *stream);

/* Same as fm_execute with HOST buffers: copies x to the device, runs the
 * plan and copies the result back into y before returning (synchronous),
 * and reports a device-side failure of the call (as fm_plan_check).  Runs on
 * the plan's device, whatever device is current, and leaves the current
 * device as it was.  Large calls are split into column chunks pipelined over
 * three streams (copy in, compute, copy out), so with page-locked host
 * buffers the copies of one chunk overlap the transform of the next.  The
 * device operand buffers and streams are kept per device, shared by all
 * plans and sized by the largest call so far, until the process exits;
 * calls on one device take turns. */
int fm_execute_host(fm_plan *plan, int32_t direction,
                    const void *x, int32_t x_type, int64_t ld_x,
                    void *y, int32_t y_type, int64_t ld_y,
                    int64_t num_cols);

/* Free the device operand buffers fm_execute_host keeps for the current
 * device (for example after a one-off large call); the next host call
 * allocates them again.  The reference has no counterpart. */
int fm_release_host_staging(void);

/* Tile shape of launch `launch` of a direction: vectors per tile and the
 * depth (2..4) of its copy ring, keeping the launch's tile layout;
 * fm_plan_set_tile returns FM_ERR_VALUE for an infeasible request and leaves
 * the launch unchanged.  layout: 0 vector-major padded, 1 element-major (TMA
 * boxes), 2 vector-major dense.  The reference has no counterpart. */
int fm_plan_set_tile(fm_plan *plan, int32_t direction, int32_t launch,
                     int32_t vectors_per_tile, int32_t nbuf);
/* Same with the tile layout: 0 vector-major padded, 1 element-major (TMA
 * boxes; strided views), 2 vector-major dense (contiguous vectors, one bulk
 * copy per run of vectors). */
int fm_plan_set_tile_layout(fm_plan *plan, int32_t direction, int32_t launch,
                            int32_t vectors_per_tile, int32_t nbuf,
                            int32_t layout);
int fm_plan_get_tile(const fm_plan *plan, int32_t direction, int32_t launch,
                     int32_t *vectors_per_tile, int32_t *nbuf,
                     int32_t *layout);

/* Autotuner: for every launch of `direction`, time each feasible tile
 * shape on temporary buffers shaped like the launch's operands for
 * `num_cols` columns (a sample of at most ~512 MiB per operand) and keep the
 * fastest.  Synchronous; allocates temporaries.  The choices can be read
 * back with fm_plan_get_tile and replayed with fm_plan_set_tile (the Python
 * layer caches them on disk).  The reference has no counterpart (its
 * calibration fits CPU runtime models, fastmat/core/calibration.py). */
int fm_plan_autotune(fm_plan *plan, int32_t direction, int64_t num_cols,
                     void *stream);

/* Report (and clear) a failure that kernels of this plan recorded on the
 * device since the last check: FM_ERR_TIMEOUT if a bounded wait for a tile
 * copy gave up.  Synchronises with the device.  fm_execute_host checks on
 * every call; callers of the asynchronous entry points check after they
 * synchronise.  The reference has no device and no counterpart. */
int fm_plan_check(fm_plan *plan);

/* Number of polls a bounded wait of this plan's kernels (a tile copy's
 * mbarrier) makes before it gives up and the launch records FM_ERR_TIMEOUT
 * for fm_plan_check; default 2^22 (each poll may suspend the thread for up to
 * about a microsecond).  A kernel that gives up still waits, with the
 * default limit, for the copies it has in flight, then returns.  0 makes the
 * first wait give up at once: the failure path can be exercised without a
 * fault.  Takes effect from the next launch.  The reference has no device
 * and no counterpart. */
int fm_plan_set_wait_limit(fm_plan *plan, int64_t polls);

int fm_plan_destroy(fm_plan *plan);

/* Plan introspection for tests and benchmarks. */
typedef struct fm_plan_info {
    int64_t rows, cols;          /* operator shape                           */
    int32_t num_launches_fwd;    /* kernel launches per forward call         */
    int32_t num_launches_bwd;
    int64_t scratch_bytes_per_col; /* device scratch a column needs          */
    int64_t const_bytes;         /* device constants owned by the plan       */
    int32_t compute_type;
    int32_t pad;
} fm_plan_info;
int fm_plan_get_info(const fm_plan *plan, fm_plan_info *info);

/* Human-readable dump of the lowered launches (stage list) into buf. */
int fm_plan_describe(const fm_plan *plan, int32_t direction, char *buf,
                     int64_t buf_len);

/* ---- batches: many operators in one persistent launch -----------------
 * A batch binds a list of plans (one operator each, forward or backward)
 * to their operands: column-major x / y device buffers with num_cols
 * columns each (leading dimensions ld_x / ld_y; types as in fm_execute).
 * fm_batch_execute runs ALL of them in one cooperative persistent launch:
 * the k-th launch of every plan forms level k, the tiles of a level are
 * spread over all CTAs, and the CTAs meet at a grid barrier (a bounded
 * wait) between levels.  Plans must share one compute type, FM_C64 or
 * FM_C128_DF, and must outlive the batch (it reads their constants).  The
 * batch owns the scratch every operator needs for its columns.
 * fm_batch_execute_graph captures that launch into a CUDA graph on its
 * first call (on a stream the batch owns) and replays the graph on `stream`
 * from then on.  The operand pointers are fixed at creation, so a graph
 * replay reads and writes the same buffers.  The reference applies its
 * operators one call at a time; this has no counterpart there. */
typedef struct fm_batch fm_batch;
int fm_batch_create(int32_t num_ops, fm_plan *const *plans,
                    const int32_t *directions, const void *const *x,
                    const int32_t *x_types, const int64_t *ld_x,
                    void *const *y, const int32_t *y_types,
                    const int64_t *ld_y, const int64_t *num_cols,
                    fm_batch **batch);
int fm_batch_execute(fm_batch *batch, void *stream);
int fm_batch_execute_graph(fm_batch *batch, void *stream);
/* Synchronises; FM_ERR_TIMEOUT if a bounded wait of the batch gave up. */
int fm_batch_check(fm_batch *batch);
/* Polls of the batch's grid-barrier waits before a CTA gives up, records
 * FM_ERR_TIMEOUT and returns (default 2^22; 0: at once).  Must be set
 * before the first fm_batch_execute_graph, which captures the launch. */
int fm_batch_set_wait_limit(fm_batch *batch, int64_t polls);
/* Launches of the bound plans it replaces, levels, tiles. */
int fm_batch_get_info(const fm_batch *batch, int64_t *num_launches,
                      int64_t *num_levels, int64_t *num_tiles);
int fm_batch_destroy(fm_batch *batch);

/* ---- gradients of the differentiable path -----------------------------
 * Column reduction behind the parameter gradients of a chain of operators.
 * u, v (and w) are column-major arrays of num_cols columns whose columns are
 * viewed as 3-D blocks (A, n, Cc): row r = (a * n + j) * Cc + c, the view of
 * one Kron mode (A = product of the leading factor sizes, Cc = product of
 * the trailing ones; A = Cc = 1 for a plain vector).  Writes, on `stream`,
 *
 *     out[j] = scale * sum_{a < A, c < Cc, k < num_cols} u[r + k ld_u]
 *                                                        * conj(v[r + k ld_v])
 *
 * for j < n (conj is the identity for real types).  With u the upstream
 * gradient and v the input of a Diag factor this is the gradient of the
 * diagonal; with u, v in the Fourier domain it is the spectrum of the
 * circular cross-correlation giving the gradient of a circulant or Toeplitz
 * defining vector.  If d is not NULL, w[r + k ld_w] = conj(d[j]) * u[...] is
 * written in the same pass: the adjoint of the Diag factor, fastmat's
 * Diag backward (fastmat/Diag.pyx:149-167).  type: FM_F32, FM_F64, FM_C64
 * or FM_C128 for every array.  Deterministic (fixed summation order).
 * Allocates its partial sums stream-ordered (cudaMallocAsync).  The
 * reference has no gradients; this has no counterpart there. */
int fm_reduce_mulconj(int64_t A, int64_t n, int64_t Cc, int64_t num_cols,
                      int32_t type, const void *u, int64_t ld_u,
                      const void *v, int64_t ld_v, void *out, double scale,
                      const void *d, void *w, int64_t ld_w, void *stream);

/* Test hook for the out-of-memory path: after `after` more device
 * allocations of this library succeed, the next one fails as if the device
 * were full (the call then returns FM_ERR_NOMEM and frees what it had
 * allocated); after < 0 disarms it.  One-shot, process-wide.  The reference
 * has no counterpart. */
int fm_debug_fail_allocation(int32_t after);

/* Message of the last failing call on this thread ("" if none). */
const char *fm_last_error(void);

/* ABI version (major * 100 + minor). */
int32_t fm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FMGPU_H */
