/*
 * aprod_gpu.c — drop-in replacement for the reference's source/aprod.c
 * (aprod(), source/aprod.h:10-13) that runs the operator on one GPU through
 * libplsqr_gpu, for a maintainer who keeps the reference's lsqr.c and its
 * driver (plsqr3.c) on a single rank.
 *
 * Build it with the reference's own headers in place of aprod.c, FP64
 * (SDVERSION 2, so that MY_FLOAT_TYPE is double), and link -lplsqr_gpu.  The
 * first call builds a GPU context from the matrices in PPDataV3_TRI (K by
 * column, D by row and by column, main.h:246-251, 414); every call then copies
 * the input vector to the device and the updated one back, as the reference's
 * own GPU wrappers did around each product (aprod_impl.c:116-119, 154, 190).
 * lsqr.c passes isFinalIteration = 1 to both calls of its last iteration
 * (:491-507, :564); the context is released by the second of them, the
 * mode-2 call, or at exit where that call does not come (beta = 0 in the
 * last iteration skips it, lsqr.c:530).  Errors end the run through
 * MPI_Abort, as the reference's aprod does on its own failures.
 */
#include <stdio.h>
#include <stdlib.h>

#include "main.h"
#include "aprod.h"
#include "plsqr_gpu.h"

/* the library computes in FP64: the reference must be built with SDVERSION 2 */
typedef char aprod_gpu_needs_fp64[sizeof(MY_FLOAT_TYPE) == sizeof(double) ? 1 : -1];

static plsqr_ctx *g_ctx;

static void release_ctx(void) {
  plsqr_ctx_destroy(g_ctx);
  g_ctx = NULL;
}

static int make_ctx(PPDataV3_TRI *p) {
  const SpMatCSC *k = p->matCSC_k;
  const SpMatCSR *d = p->matCSR_d;
  const SpMatCSC *dc = p->matCSC_d_bycol;
  plsqr_sparse ks = {k->numRow, k->numCol, k->numNonzero, k->col_ptr, NULL, k->row_idx, k->val};
  plsqr_sparse ds = {d->numRow, d->numCol, d->numNonzero, d->row_ptr, NULL, d->col_idx, d->val};
  plsqr_sparse dcs = {dc->numRow, dc->numCol, dc->numNonzero, dc->col_ptr, NULL, dc->row_idx,
                      dc->val};
  static int at_exit;
  plsqr_opts o;
  plsqr_default_opts(&o);
  o.lean = 1; /* the operator alone: the unit layouts of K are all it reads */
  const int rc = plsqr_ctx_create(&ks, &ds, &dcs, &o, &g_ctx);
  /* registered after the CUDA runtime has started, so that it runs first */
  if (rc == PLSQR_OK && !at_exit) at_exit = atexit(release_ctx) == 0;
  return rc;
}

void aprod(int version, int procRank, int numProc, int mode, int m, int n, MY_FLOAT_TYPE x[],
           MY_FLOAT_TYPE y[], void *UsrWork, int isFinalIteration, int iteration) {
  PPDataV3_TRI *p = (PPDataV3_TRI *)UsrWork;
  int rc;
  (void)version, (void)procRank, (void)m, (void)n, (void)x, (void)y;
  if (numProc != 1) {
    fprintf(stderr, "aprod on GPU: one rank holds the whole operator (got %d ranks)\n", numProc);
    MPI_Abort(MPI_COMM_WORLD, 1);
  }
  rc = g_ctx ? PLSQR_OK : make_ctx(p);
  if (rc == PLSQR_OK)
    rc = plsqr_aprod_host(g_ctx, mode, p->vec_y_k, p->vec_y_d, p->vec_x, iteration,
                          isFinalIteration);
  if (rc != PLSQR_OK) {
    fprintf(stderr, "aprod on GPU: %s\n", plsqr_strerror(rc));
    MPI_Abort(MPI_COMM_WORLD, 1);
  }
  if (isFinalIteration && mode == 2) release_ctx();
}
