/*
 * plsqr_gpu.h — C ABI of the GB300 PLSQR3 operator and LSQR driver.
 *
 * The library replaces, on one GPU, the hot path of PLSQR3:
 *   - the operator  aprod(version, procRank, numProc, mode, m, n, x, y,
 *     UsrWrk, isFinalIteration, iteration)             source/aprod.h:10-13
 *     (mode 1: y <- y + A x, mode 2: x <- x + A^T y, A = [K; D]),
 *   - the driver    lsqr(..., aprod, damp, UsrWrk, u, v, w, x, se, atol,
 *     btol, conlim, itnlim, nout, outputs..., lsqr_iteration) source/lsqr.h:32-62,
 *   - the loaders of the kernel and damping binary/info files and the result
 *     writer (source/plsqr3.c:1008-1626, 1986-2013), single partition.
 *
 * Conventions: every function returns 0 (PLSQR_OK) or a negative PLSQR_ERR_*
 * code and never exits the process (the reference calls exit(-1) / MPI_Abort
 * on the same conditions).  Matrices and vectors are FP64 (the reference with
 * SDVERSION=2) and indices are 0-based int32 with int32 or int64 pointer
 * arrays.  A context owns all of its device memory and one CUDA stream; it is
 * not reentrant (like the reference's function-static scratch), so use one
 * context per host thread.  No type in these signatures depends on CUDA.
 */
#ifndef PLSQR_GPU_H
#define PLSQR_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLSQR_GPU_ABI_VERSION 4

/* ---- error codes ------------------------------------------------------- */
#define PLSQR_OK 0
#define PLSQR_ERR_ARG (-1)      /* invalid argument or size                    */
#define PLSQR_ERR_IO (-2)       /* file cannot be opened, read or written      */
#define PLSQR_ERR_FORMAT (-3)   /* file or matrix content is inconsistent      */
#define PLSQR_ERR_NOMEM (-4)    /* host allocation failed                      */
#define PLSQR_ERR_CUDA (-5)     /* CUDA runtime error (device memory, launch)  */
#define PLSQR_ERR_NODEV (-6)    /* no usable CUDA device                       */
#define PLSQR_ERR_STATE (-7)    /* call out of sequence                        */
#define PLSQR_ERR_TIMEOUT (-8)  /* a bounded device wait gave up               */
#define PLSQR_ERR_INTERNAL (-9) /* internal consistency check failed           */
#define PLSQR_ERR_NUMERIC (-10) /* NaN or Inf in an input, or magnitudes the
                                   FP64 sums of squares of the norms cannot
                                   hold: a largest |value| above 2^500, or a
                                   vector whose nonzeros are all below 2^-500 */

/* source/main.h:26-36 precision switch, as a run-time choice */
#define PLSQR_PREC_FP64 0  /* FP64 values, vectors, reductions              */
#define PLSQR_PREC_MIXED 1 /* FP32 inner sweeps on the value split, FP64 outer */

/* Order of the FP64 sums (PLSQR_PREC_FP64 contexts). */
#define PLSQR_ORDER_FAST 0      /* products and norms summed in parallel order
                                   (default; results within rounding of the
                                   reference's, not its bits)                 */
#define PLSQR_ORDER_REFERENCE 1 /* every product, sum and norm in the order and
                                   rounding of the reference's CPU code
                                   (CPUSpMV.c, mycblas.c, lsqr.c built for FP64
                                   without FMA contraction): a solve returns the
                                   reference's bits, at a fraction of the speed */

/* Compressed sparse matrix, by column (ptr over columns, idx = row) or by
 * row (ptr over rows, idx = column); SpMatCSC / SpMatCSR of
 * source/main.h:123-130, 158-165.  Exactly one of ptr32 / ptr64 is set, so
 * the reference's own int* col_ptr can be passed without a copy. */
typedef struct {
  int32_t num_row;
  int32_t num_col;
  int64_t nnz;
  const int32_t *ptr32;
  const int64_t *ptr64;
  const int32_t *idx;
  const double *val;
} plsqr_sparse;

/* The reference command line (source/plsqr3.c:105-186): file names are
 * relative to dir; -row_ptn / -col_ptn have no meaning on one partition. */
typedef struct {
  const char *dir;
  const char *ker_f;        /* -ker_f  kernel records, sorted by column     */
  const char *ker_i;        /* -ker_i  ASCII "col nnz start", 1-based       */
  const char *damp_f;       /* -damp_f damping records, sorted by row       */
  const char *damp_i;       /* -damp_i int32 nnz per damping row            */
  const char *damp_f_bycol; /* -damp_f_bycol damping records, by column     */
  const char *damp_i_bycol; /* -damp_i_bycol int32 nnz per column           */
  const char *b_k;          /* -b_k    ASCII measurement vector             */
  int32_t row_k, row_d, col;
  /* -col_perm: NULL, or an ASCII file of `col` 1-based column numbers; the
   * kernel matrix is then loaded with its column i taken from file column
   * perm[i], as the reference's COL_PERM build does (read_col_perm and
   * mpiio_load_kernelColBin2ReorderedCSC, source/plsqr3.c:261-283, 1348-1361,
   * 1652-1713); the damping files and b_k are read as given and x comes out
   * in the permuted column order (the float64 result file of
   * source/lsqr.c:95-99 is written so).                                      */
  const char *col_perm;
} plsqr_files;

typedef struct {
  int32_t device;    /* CUDA device ordinal (default 0)                       */
  int32_t precision; /* PLSQR_PREC_*                                          */
  int32_t use_graph; /* capture each LSQR iteration as a CUDA graph (def. 1)  */
  int32_t verbose;   /* print the per-iteration alpha/beta lines like lsqr.c  */
  /* Optional model grid (nx, ny, nz) with column = (iz*ny + iy)*nx + ix, the
   * cell map of damping_binary.py; when given (and nx*ny*nz = n) the A^T y
   * product visits the columns in 3-D Morton order so that cells sharing
   * rays are gathered together.  Zeros: natural column order. */
  int32_t grid[3];
  int32_t order; /* PLSQR_ORDER_* (FP64 contexts; mixed precision needs FAST) */
  /* Nonzero: once the unit layouts hold both FP64 products, release the
   * by-row and by-column copies of K they were built from (device memory
   * about 1.7x the 16 bytes per nonzero instead of 3.7x).  FP64 contexts in
   * the fast order only (PLSQR_ERR_ARG otherwise).  plsqr_lsqr and
   * plsqr_aprod are unchanged, bit for bit; the batched solver, which reads
   * those copies, returns PLSQR_ERR_STATE on such a context. */
  int32_t lean;
} plsqr_opts;

typedef struct {
  int32_t m_k, m_d, n;
  int64_t nnz_k, nnz_d;
  int64_t device_bytes;       /* device memory held by the context        */
  int32_t sm_count;
  double hbm_bytes_aprod1;    /* algorithmic bytes of one mode-1 aprod    */
  double hbm_bytes_aprod2;    /* algorithmic bytes of one mode-2 aprod    */
  double hbm_bytes_iteration; /* algorithmic bytes of one LSQR iteration  */
} plsqr_info;

/* Arguments of lsqr() (source/lsqr.h:32-62); call_lsqr uses damp = 0,
 * atol = btol = 1e-10, conlim = 100, itnlim = 1000 (source/lsqr.c:47-51). */
typedef struct {
  double damp, atol, btol, conlim;
  int32_t itnlim;
  int32_t lsqr_iteration; /* iterations run; istop does not stop the loop,
                             as in source/lsqr.c:829-834                      */
  int32_t want_se;        /* compute the standard-error estimate se[]        */
  int32_t stop_on_istop;  /* 0 = reference behaviour                         */
  const char *result_txt; /* NULL, or path of the Paige-Saunders log written
                             like result.txt (source/lsqr.c:246-268, 780-905) */
  /* PLSQR_PREC_MIXED contexts only: `sweeps` outer refinement steps, each
   * an FP32 LSQR of `inner` iterations on r = b - A x (FP64); the history
   * then holds sweeps * inner + 1 records and lsqr_iteration is unused.
   * damp > 0 requires sweeps = 1 (PLSQR_ERR_ARG otherwise).                 */
  int32_t sweeps, inner;
  /* PLSQR_PREC_MIXED contexts only: starting solution x0 [n] (warm start) or
   * NULL (x0 = 0, as in source/lsqr.c:311-312).  The first sweep corrects
   * from r = b - A x0; where ||r|| is not below ||b|| the solve restarts
   * from 0 (cold-start fallback) and plsqr_result.warm is 0.  Needs damp = 0
   * (damping would regularise the correction, not the solution).           */
  const double *x0;
} plsqr_lsqr_args;

/* Scalars of one iteration (index 0 = start-up, source/lsqr.c:343-445). */
typedef struct {
  double alpha, beta, rnorm, arnorm, test1, test2, anorm, acond, xnorm, x0;
  double err; /* ||x - x_ref|| / ||x_ref|| when a reference x is set, else -1 */
  int32_t istop, pad;
} plsqr_iter;

/* Outputs of lsqr() (source/lsqr.c:908-914; arnorm_out is test2 there). */
typedef struct {
  int32_t istop, itn;
  double anorm, acond, rnorm, arnorm_out, xnorm;
  double arnorm, bnorm, dxmax;
  int32_t maxdx;
  int32_t warm;         /* 1 when the solve started from the caller's x0     */
  double seconds;       /* device time of the iteration loop (CUDA events), the
                           region of the reference's "Parallel LSQR time"
                           (source/lsqr.c:476-842)                            */
  double seconds_total; /* device time from the start-up's first kernel to the
                           end of the loop (mixed precision: the whole solve)  */
} plsqr_result;

typedef struct plsqr_ctx plsqr_ctx;

/* ---- library ----------------------------------------------------------- */
const char *plsqr_strerror(int code);
int plsqr_abi_version(void);
/* Bounds checks.  *checked = 1 in the bounds-checked build of the library
 * (compiled with -DPLSQR_CHECK: the unit-layout kernels check every slot,
 * gather index, line and lane they touch, record a failed check and skip the
 * access), 0 in the normal build; *flags = the checks that failed on the
 * current device since the last reset (bits: 1 slot, 2 gather index, 4 line,
 * 8 lane, 16 fill; always 0 in the normal build).  No counterpart in the
 * reference. */
int plsqr_check_flags(int32_t *checked, uint32_t *flags, int32_t reset);
void plsqr_default_opts(plsqr_opts *opts);
void plsqr_default_lsqr_args(plsqr_lsqr_args *args);
/* Number of CUDA devices; 0 and PLSQR_OK when the driver has none. */
int plsqr_device_count(int32_t *count);

/* ---- context: replaces PLSQR3_main's loading + initPPDataV3_TRI +
 *      InitPPDataV3_TRI_GPU (source/plsqr3.c:218-575, tridiagonal.c:13-95,
 *      lsqr.c:455) ------------------------------------------------------- */
/* From the matrices in the reference's in-memory layout: K by column
 * (matCSC_k), D by row (matCSR_d) and D by column (matCSC_d_bycol).  The
 * kernel matrix is also transposed to rows on the device. */
int plsqr_ctx_create(const plsqr_sparse *k_csc, const plsqr_sparse *d_csr,
                     const plsqr_sparse *d_csc, const plsqr_opts *opts,
                     plsqr_ctx **out);
/* From the reference's files; b_k is loaded too (plsqr3.c:580-589). */
int plsqr_ctx_create_files(const plsqr_files *files, const plsqr_opts *opts,
                           plsqr_ctx **out);
/* FinalPPDataV3_TRI_GPU (source/lsqr.c:873). NULL is accepted. */
void plsqr_ctx_destroy(plsqr_ctx *ctx);
int plsqr_ctx_info(const plsqr_ctx *ctx, plsqr_info *info);
/* Last CUDA error text seen by the context (empty if none). */
const char *plsqr_ctx_last_error(const plsqr_ctx *ctx);

/* ---- vectors of PPDataV3_TRI: u = [vec_y_k; vec_y_d], v = vec_x -------- */
int plsqr_set_u(plsqr_ctx *ctx, const double *y_k, const double *y_d);
int plsqr_get_u(plsqr_ctx *ctx, double *y_k, double *y_d);
int plsqr_set_v(plsqr_ctx *ctx, const double *v);
int plsqr_get_v(plsqr_ctx *ctx, double *v);
/* b_k loaded by plsqr_ctx_create_files (or NULL-safe copy out). */
int plsqr_get_b(plsqr_ctx *ctx, double *b_k);

/* ---- operator ---------------------------------------------------------- */
/* aprod on the device-resident vectors: mode 1 y += A x, mode 2 x += A^T y
 * (source/aprod.c:24-84, aprod_impl.c:22-524).  iteration and is_final have
 * the reference's meaning and do not change the result. */
int plsqr_aprod(plsqr_ctx *ctx, int mode, int iteration, int is_final);
/* The same with host vectors, the drop-in for the reference call: the input
 * vectors are copied to the device, the updated one is copied back
 * (mode 1 reads x, updates y_k/y_d; mode 2 reads y_k/y_d, updates x). */
int plsqr_aprod_host(plsqr_ctx *ctx, int mode, double *y_k, double *y_d,
                     double *x, int iteration, int is_final);

/* ---- driver ------------------------------------------------------------ */
/* lsqr() on the device (source/lsqr.c:195-917).  b_k (host, m_k values; NULL
 * = the b_k the context loaded) is the right-hand side, the damping part of
 * b is zero.  x, w, se (host, n values each) may be NULL; hist may be NULL or
 * hold lsqr_iteration + 1 records. */
int plsqr_lsqr(plsqr_ctx *ctx, const plsqr_lsqr_args *args, const double *b_k,
               double *x, double *w, double *se, plsqr_iter *hist,
               plsqr_result *res);
/* A reference solution (host, n values) against which every iteration
 * records ||x - x_ref|| / ||x_ref|| in plsqr_iter.err; NULL clears it. */
int plsqr_set_reference_x(plsqr_ctx *ctx, const double *x_ref);
/* The last solution x (host, n values). */
int plsqr_get_x(plsqr_ctx *ctx, double *x);
/* mpiio_write_result (source/plsqr3.c:1986-2013): raw FP64 x[n]. */
int plsqr_write_result(plsqr_ctx *ctx, const char *path);

/* ---- measurement (no counterpart in the reference) ---------------------- */
/* Average device time of one launch of the mode-1 or mode-2 product kernel
 * (y += A x or x += A^T y on the context's vectors, which it overwrites),
 * from CUDA events around `reps` back-to-back launches on the context's
 * stream. */
int plsqr_bench_aprod(plsqr_ctx *ctx, int mode, int reps, double *ms_per_launch);
/* The same for one LSQR iteration replayed from its CUDA graph; needs a
 * preceding plsqr_lsqr on the context (state and history are overwritten). */
int plsqr_bench_iteration(plsqr_ctx *ctx, int reps, double *ms_per_iteration);

/* ---- timing report: the reference's GPTL timers (source/lsqr.c:473-842,
 *      aprod_impl.c:69-497; gptl.c writes them to timing.<rank>) ----------- */
/* on = 1: the following FP64 solves on the context run their iterations
 * without the CUDA graph and record CUDA events around five regions of every
 * iteration, named after the reference's timers: spmv, norm1, spmvT,
 * update_x, krylov_p1 (each region's "covers" text in the report lists the
 * reference timers whose work it holds); the host side of every region is
 * an NVTX range of the same name.  Without timing, the solve is one NVTX
 * range "LSQR_MAIN_ITERATION" around graph launches.  on = 0 restores the
 * graph replay. */
int plsqr_set_timing(plsqr_ctx *ctx, int on);
/* JSON report of the last timed solve: LSQR_MAIN_ITERATION seconds, the
 * start-up, per region the total, mean, min and max, and every iteration's
 * time per region.  PLSQR_ERR_STATE when no timed solve has run. */
int plsqr_write_timing(const plsqr_ctx *ctx, const char *path);

/* ---- product without device allocation ----------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory: code whose device memory belongs to another allocator or a fixed
 * budget (a framework's caching allocator, an MPI rank that sized its
 * buffers before the solve), and callers that cannot block on the driver's
 * allocator (cudaMalloc and cudaFree may synchronise the device).
 * y <- y + A x for an n_rows-row CSR matrix (row_ptr int64[n_rows+1],
 * col_idx/val 16-byte aligned, indices in range of x) and *nrm2 = ||y||_2
 * after the update; every pointer is device memory, the work is ordered on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) and nothing is
 * synchronised.  It allocates no memory: its per-block partial sums live in a
 * 128 KB static device array of the library (held by every GPU that loads the
 * library until exit), so n_rows is limited to PLSQR_NOALLOC_MAX_ROWS
 * (PLSQR_ERR_ARG beyond it).  The first call on a device looks up that array
 * and should come before any stream capture (a first call on a capturing
 * stream returns PLSQR_ERR_STATE and does nothing); calls share the array,
 * so calls that overlap on the GPU race.  The looked-up address is kept for
 * the process: calls after a cudaDeviceReset are not supported. */
#define PLSQR_NOALLOC_MAX_ROWS 1048576
int plsqr_aprod1_nrm2_noalloc(int32_t n_rows, const int64_t *row_ptr,
                              const int32_t *col_idx, const double *val,
                              const double *x, double *y, double *nrm2,
                              void *stream);

/* ---- several right-hand sides on one operator ---------------------------
 * No counterpart in the reference, whose lsqr() solves one right-hand side
 * per run (source/lsqr.c:195-917).  These entries advance k <= 32 LSQR solves
 * in lock step on the context's matrix, one k-wide product per matrix read:
 * right-hand side j solves min || [K; lambda_j D] x_j - [b_j; 0] || (the
 * damping rows weighted by lambda_j).  The form is the refinement solver of
 * PLSQR_PREC_MIXED: `sweeps` FP64 residuals b - A x over the FP64 kernel
 * values, each followed by `inner` LSQR iterations whose kernel products use
 * the FP32 high half of the value split while vectors, norms and the scalar
 * recurrences stay FP64. */
#define PLSQR_BATCH_MAX 32
typedef struct {
  int32_t k;             /* right-hand sides, 1 .. PLSQR_BATCH_MAX            */
  int32_t sweeps, inner; /* refinement sweeps, LSQR iterations per sweep      */
  int32_t variant_rows;  /* product variant of A x (plsqr_batch_variant), or
                            -1 = pick by timing (cached per operator shape)  */
  int32_t variant_cols;  /* the same for A^T y                                */
  int32_t retire_every;  /* 0: every right-hand side runs sweeps*inner
                            iterations.  R > 0: every R inner iterations the
                            finished right-hand sides retire: with
                            retire_err > 0 (needs x_ref) those with err <=
                            retire_err, in any sweep; else those whose
                            stopping test has fired (istop != 0) in the last
                            sweep (conlim = 100, the reference's constant,
                            fires once cond(A) passes 100: set conlim to
                            suit).  A retiree's x and result are kept as they
                            stand (result itn = the iteration it retired at;
                            history records up to it), and the others go on
                            packed into the narrowest block width that holds
                            them.  The solve ends when none is left.        */
  double damp, atol, btol, conlim; /* lsqr() arguments of every solve; damp > 0
                                      requires sweeps = 1                    */
  const double *b_k;     /* [k][m_k]: right-hand side j at b_k + j*m_k        */
  const double *lambda;  /* [k] damping-row weights; NULL = all 1             */
  const double *x_ref;   /* [k][n] solutions to measure the error against
                            (history field err), or NULL                      */
  const double *x0;      /* [k][n] starting solutions (warm start), or NULL =
                            0: the first sweep corrects from b - A x0.  A
                            right-hand side whose starting residual is not
                            below ||b|| starts from 0 instead (cold start);
                            info.warm says which kept x0.  Needs damp = 0.   */
  double retire_err;     /* see retire_every; 0 = retire on istop         */
} plsqr_batch_args;
void plsqr_default_batch_args(plsqr_batch_args *a);

/* Product variants: kVW-wide gathers (4 = float4, 2 = float2), kLPR lanes per
 * line, kU nonzeros in flight per lane; kLPR = 0 is the slab form (the
 * gathered block staged through shared memory a slab at a time, kw/4 lanes
 * per line); kLPR = -1 the units form (passes of 4 or 8 columns: the
 * block's rows staged per slab in shared memory, the matrix in the FP32 unit
 * layout with 16-bit slab-local indices, a lane per line).  Returns
 * PLSQR_ERR_ARG past the last. */
int plsqr_batch_variant(int32_t index, int32_t *vw, int32_t *lanes_per_line,
                        int32_t *unroll);

typedef struct {
  int32_t k, kp;                    /* right-hand sides, padded block width   */
  int32_t variant_rows, variant_cols; /* variants in use                      */
  int32_t tuned;                    /* 1: timed by the last call, 0: cached   */
  int32_t warm;                     /* bit j: right-hand side j kept its x0   */
  double ms_rows, ms_cols;          /* their times per product when timed     */
} plsqr_batch_info;

/* Solve; x: [k][n] (or NULL), hist: [k][sweeps*inner + 1] (or NULL; entry 0
 * is the start of the first sweep), res: [k] (or NULL). */
int plsqr_batch_lsqr(plsqr_ctx *ctx, const plsqr_batch_args *a, double *x,
                     plsqr_iter *hist, plsqr_result *res, plsqr_batch_info *info);
/* Time one k-wide product (mode 1: A x, mode 2: A^T y) of a variant (-1 =
 * the tuned one), averaged over reps launches, after one untimed launch. */
int plsqr_batch_bench_aprod(plsqr_ctx *ctx, int32_t k, int mode, int32_t variant,
                            int reps, double *ms_per_launch);

/* ---- independent problems in one persistent launch ----------------------
 * No counterpart in the reference, which solves one problem per run.  Each
 * problem is a complete lsqr() of lsqr_iteration iterations in FP64 (the
 * reference's arithmetic, source/lsqr.c:195-917), on its own operator
 * [K; D] and right-hand side.  One cooperative kernel launch runs all of them:
 * a host planner gives every problem a group of thread blocks (in proportion
 * to its work, several small problems queued on one group when blocks run
 * out), and each group works through its queue, its blocks meeting at
 * barriers in device memory.  Every barrier wait is bounded (wait_ns): past
 * the limit the launch ends and the solve returns PLSQR_ERR_TIMEOUT. */
typedef struct {
  plsqr_sparse k_csc, d_csr, d_csc; /* as for plsqr_ctx_create              */
  const double *b_k;                /* [k_csc.num_row]                      */
  int32_t lsqr_iteration;           /* iterations run (as plsqr_lsqr_args)  */
  int32_t itnlim;
  double damp, atol, btol, conlim;
} plsqr_problem;
void plsqr_default_problem(plsqr_problem *p); /* call_lsqr's constants */

typedef struct plsqr_multi plsqr_multi;
typedef struct {
  int32_t count;         /* problems                                        */
  int32_t blocks;        /* thread blocks of the persistent launch          */
  int32_t groups;        /* block groups (each runs a queue of problems)    */
  int32_t blocks_per_sm; /* resident blocks per SM of the launch            */
  int64_t device_bytes;  /* device memory held                              */
  int64_t wait_ns;       /* limit of one barrier wait                       */
  double seconds;        /* device time of the last solve                   */
} plsqr_multi_info;

/* Uploads the problems (copied; the caller's arrays may be freed after). */
int plsqr_multi_create(const plsqr_problem *probs, int32_t count,
                       const plsqr_opts *opts, plsqr_multi **out);
void plsqr_multi_destroy(plsqr_multi *mp);
const char *plsqr_multi_last_error(const plsqr_multi *mp);
int plsqr_multi_info_get(const plsqr_multi *mp, plsqr_multi_info *info);
/* The plan: group[p] of every problem and the blocks of every group
 * (arrays of count entries; group_blocks entries past info.groups are 0). */
int plsqr_multi_plan(const plsqr_multi *mp, int32_t *group, int32_t *group_blocks);
/* exact = 1: the products round every multiply and add apart, in the
 * reference's order, so each row and column sum is the reference's to the
 * bit (twice the FP64 instructions); 0 (default): fused multiply-adds in the
 * same order. */
int plsqr_multi_set_exact(plsqr_multi *mp, int32_t exact);
/* sweeps > 0: FP32 inner / FP64 outer.  Every problem runs `sweeps`
 * refinement sweeps; each is an LSQR of lsqr_iteration iterations for the
 * correction dx on the FP64 residual r = b - A x, with the kernel products
 * in FP32 values (rounded to nearest) times hi + lo FP32 pairs of the FP64
 * vectors (error-free FP32 products and sums), vectors, damping products,
 * norms and recurrence in FP64; x += dx after each sweep.  hist and res then
 * hold the last sweep's LSQR.  0 (default): one FP64 LSQR.  Not with
 * exact products (PLSQR_ERR_ARG). */
int plsqr_multi_set_mixed(plsqr_multi *mp, int32_t sweeps);
/* Set the barrier wait limit (nanoseconds, >= 1000); default one second. */
int plsqr_multi_set_wait(plsqr_multi *mp, int64_t wait_ns);
/* Solve all problems.  x: the solutions one after another (sum of n_p
 * values) or NULL; hist: lsqr_iteration_p + 1 records per problem, one after
 * another, or NULL; res: [count] or NULL. */
int plsqr_multi_solve(plsqr_multi *mp, double *x, plsqr_iter *hist, plsqr_result *res);
/* The planner alone, on the host: problems with the given modelled bytes per
 * iteration and iteration counts on `blocks` blocks of bw_block bytes/s
 * each.  group[count]; group_blocks needs max(count, blocks) entries;
 * *n_groups = groups made. */
int plsqr_multi_plan_host(const double *bytes, const int32_t *iters, int32_t count,
                          int32_t blocks, double bw_block, int32_t *group,
                          int32_t *group_blocks, int32_t *n_groups);
/* Runs one bounded wait on a flag that nothing sets, on the device, with the
 * given limit: returns PLSQR_ERR_TIMEOUT and leaves the context usable. */
int plsqr_multi_check_wait(plsqr_multi *mp, int64_t wait_ns);

/* ---- learned warm start ---------------------------------------------------
 * No counterpart in the reference.  A 3-D U-Net (3 levels, 16/32/64
 * channels, BF16 weights with FP32 masters, FP32 accumulation) on the model
 * grid maps the column-norm-scaled back-projection A^T b to a starting
 * solution x0, which plsqr_batch_args.x0 hands to the solver (with the cold
 * start as fallback).  Volumes are nx*ny*nz floats in column order
 * ((z*ny + y)*nx + x); nx, ny, nz multiples of 4. */
typedef struct plsqr_unet plsqr_unet;
int plsqr_unet_create(int32_t nx, int32_t ny, int32_t nz, uint64_t seed, int32_t device,
                      plsqr_unet **out);
void plsqr_unet_destroy(plsqr_unet *net);
const char *plsqr_unet_last_error(const plsqr_unet *net);
/* x0 = net(in) (host arrays). */
int plsqr_unet_predict(plsqr_unet *net, const float *in, float *out);
/* One Adam step on the squared error against target (host arrays); *loss is
 * the mean squared error in units of the input's root mean square. */
int plsqr_unet_train_step(plsqr_unet *net, const float *in, const float *target, float lr,
                          float *loss);
/* The same two calls on device arrays (nx*ny*nz floats on the network's
 * device), ordered after the work already queued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream); the caller's stream
 * waits for the result.  Both return once the step has run. */
int plsqr_unet_predict_device(plsqr_unet *net, const float *in, float *out, void *stream);
int plsqr_unet_train_step_device(plsqr_unet *net, const float *in, const float *target, float lr,
                                 float *loss, void *stream);
/* All weights (set = 0: read into buf; 1: load from buf).  buf = NULL:
 * *count = the number of floats. */
int plsqr_unet_weights(plsqr_unet *net, float *buf, int64_t *count, int32_t set);
/* One 3x3x3 convolution + ReLU layer, forward and backward, on host arrays
 * (x [n][cin], w [cout][27*cin] with tap-major k, dy [n][cout]); the
 * network's kernels checked in isolation. */
int plsqr_nn_conv3d_check(int32_t nx, int32_t ny, int32_t nz, int32_t cin, int32_t cout,
                          const float *x, const float *w, const float *b, const float *dy,
                          float *y, float *dx, float *dw, float *db);

/* Weight the context's damping rows: D becomes lambda * D (both copies, from
 * the values the context was created with).  For one-right-hand-side solves
 * of the weighted problems above. */
int plsqr_set_damping_weight(plsqr_ctx *ctx, double lambda);

/* ---- files, host side (no GPU needed) ----------------------------------- */
/* read_kernel_col_info (plsqr3.c:1379-1409): nnz[n], start[n] (0-based,
 * -1 where the file has 0) and the total. */
int plsqr_io_read_kernel_info(const char *path, int32_t n, int32_t *nnz,
                              int64_t *start, int64_t *total);
/* mpiio_load_kernelColBin2CSC_once (plsqr3.c:1515-1626): K by column. */
int plsqr_io_read_kernel(const char *bin_path, const char *info_path,
                         int32_t m_k, int32_t n, int64_t *col_ptr,
                         int32_t *row_idx, double *val);
/* mpiio_load_damp_info (plsqr3.c:1008-1025) and the column info read at
 * plsqr3.c:503-508: int32 counts, returns their sum in *total. */
int plsqr_io_read_int32_counts(const char *path, int64_t count, int32_t *out,
                               int64_t *total);
/* mpiio_load_damp_once (plsqr3.c:1027-1194), CSR (by_col = 0) or CSC. */
int plsqr_io_read_damping(const char *bin_path, int by_col, int32_t m_d,
                          int32_t n, int64_t nnz, int64_t *ptr, int32_t *idx,
                          double *val);
/* b_k, ASCII %le one per line (plsqr3.c:580-589). */
int plsqr_io_read_rhs(const char *path, int32_t m_k, double *b_k);
/* read_col_perm (plsqr3.c:1348-1361): n 1-based column numbers, returned
 * 0-based; PLSQR_ERR_FORMAT when fewer than n or one out of 1..n. */
int plsqr_io_read_col_perm(const char *path, int32_t n, int32_t *perm);
/* Column i of the result = column perm[i] of the by-column matrix (ptr, idx,
 * val over n columns), each column's entries in stored order
 * (plsqr3.c:1695-1713); tptr holds n + 1 values, tidx / tval the nonzeros of
 * the selected columns. */
int plsqr_permute_columns(int32_t n, const int64_t *ptr, const int32_t *idx, const double *val,
                          const int32_t *perm, int64_t *tptr, int32_t *tidx, double *tval);
/* Writers of the same formats (the PLSQR3_tools outputs:
 * Ker2PLSQR3.c:499-608, damping_binary.py:75-616). */
int plsqr_io_write_kernel(const char *bin_path, const char *info_path,
                          int32_t m_k, int32_t n, const int64_t *col_ptr,
                          const int32_t *row_idx, const double *val);
int plsqr_io_write_damping(const char *row_bin, const char *row_info,
                           const char *col_bin, const char *col_info,
                           int32_t m_d, int32_t n, const int64_t *row_ptr,
                           const int32_t *col_idx, const double *val,
                           const int64_t *col_ptr, const int32_t *row_idx,
                           const double *cval);
int plsqr_io_write_rhs(const char *path, int32_t m_k, const double *b_k);
int plsqr_io_write_x(const char *path, int32_t n, const double *x);

/* ---- synthetic problems and helpers, host side ------------------------- */
typedef struct {
  int32_t nx, ny, nz;       /* grid; column = iz*ny*nx + iy*nx + ix          */
  int32_t n_rays;           /* kernel rows                                   */
  double tube_radius;       /* cells within this distance of the ray         */
  int32_t face_axis;        /* rays join the two faces normal to this axis;
                               -1 = a random axis per ray                    */
  int32_t n_blobs;          /* Gaussian blobs in x_true                      */
  double value_scale;       /* kernel value = |N(0,1)| * value_scale         */
  double blob_sigma;        /* blob width in cells                           */
  double checker_amp;       /* checkerboard amplitude (0 = none)             */
  int32_t checker_period;   /* checkerboard period in cells                  */
  int32_t pad;
  double noise_frac;        /* noise sigma / rms(K x_true)                   */
  double damp_identity;     /* identity damping weight                       */
  double damp_lap;          /* second-difference damping weight (xx, yy, zz) */
  double damp_cross;        /* cross-difference weight (xy, xz, yz rows of
                               damping_binary.py:291-511); 0 leaves those rows
                               out                                           */
  int32_t n_params;         /* parameter fields of the model (damping_binary.py
                               np): the damping matrix repeats per field, with
                               columns offset by nx*ny*nz and rows by the rows
                               of one field; 0 or 1 = one field               */
  int32_t pad2;
  uint64_t seed;
} plsqr_synth_params;

void plsqr_synth_default_params(plsqr_synth_params *p);
int plsqr_synth_kernel_counts(const plsqr_synth_params *p, int64_t *row_ptr);
int plsqr_synth_kernel_fill(const plsqr_synth_params *p, const int64_t *row_ptr,
                            int32_t *col_idx, double *val);
int plsqr_synth_damping_size(const plsqr_synth_params *p, int64_t *m_d,
                             int64_t *nnz_d);
int plsqr_synth_damping_fill(const plsqr_synth_params *p, int64_t *row_ptr,
                             int32_t *col_idx, double *val);
int plsqr_synth_xtrue(const plsqr_synth_params *p, double *x);
int plsqr_synth_rhs(const plsqr_synth_params *p, const int64_t *row_ptr,
                    const int32_t *col_idx, const double *val,
                    const double *xtrue, double *b);
/* b = kx + noise_frac * rms(kx) * N(0,1) with the normals of `noise_seed`
 * (plsqr_synth_rhs adds those of p->seed to K x_true): the same measurements
 * with another noise realisation. */
int plsqr_synth_noisy(const plsqr_synth_params *p, uint64_t noise_seed, int64_t m,
                      const double *kx, double *b);
/* CSR <-> CSC transpose; output lines keep ascending input-line order. */
int plsqr_transpose(int64_t n_lines, int64_t n_out, const int64_t *ptr,
                    const int32_t *idx, const double *val, int64_t *tptr,
                    int32_t *tidx, double *tval);

#ifdef __cplusplus
}
#endif
#endif /* PLSQR_GPU_H */
