/*
 * plsqr3_gpu: the PLSQR3 program on one GB300.
 *
 * Same command line as the reference (source/plsqr3.c:105-186, README:150-170):
 *   plsqr3_gpu -dir D -ker_f F -ker_i F -damp_f F -damp_i F -damp_f_bycol F
 *              -damp_i_bycol F -b_k F -row_k M -row_d M -col N -itn K
 * and the same outputs as call_lsqr (source/lsqr.c:34-184): result.txt in the
 * working directory and the float64 solution
 * p_resultx_itn=<K>_NProc=1_float64_mpiio.bin.  -row_ptn and -col_ptn
 * describe a multi-rank partition and are accepted and ignored; -col_perm
 * FILE loads the kernel with its columns permuted, as the reference's
 * COL_PERM build does (the solution then comes out in the permuted order).
 * Additional options: -precision fp64|mixed, -sweeps S, -inner I, -device G,
 * -quiet, -x0 FILE: a starting solution for the mixed solver, col raw
 * float64 values (the format of the solution file above), kept where it
 * lowers the residual, -order fast|reference: the FP64 sums in parallel order
 * (default) or in the reference's order (its bits), and -timing FILE: the
 * iteration timed per region (the reference's GPTL timer names, NVTX
 * ranges) and written to FILE as JSON.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "plsqr_gpu.h"

int main(int argc, char **argv) {
  /* defaults of source/plsqr3.c:105-119 */
  const char *dir = "../data_plsqr3";
  const char *ker_i = "kernel_col.mm2.info", *ker_f = "kernel_col.mm2.bin";
  const char *damp_i = "plsqr3_reorder_small_all.damp.info.bin";
  const char *damp_f = "plsqr3_reorder_small_all.damp.bin";
  const char *damp_i_c = "plsqr3_reorder_small_all.damp.bycol.info.bin";
  const char *damp_f_c = "plsqr3_reorder_small_all.damp.bycol.bin";
  const char *b_k = "vecotrB_ker";
  const char *x0_path = NULL, *timing_path = NULL, *col_perm = NULL;
  int order = PLSQR_ORDER_FAST;
  int row_k = 10, row_d = 1825, col = 520, itn = 40;
  int precision = PLSQR_PREC_FP64, sweeps = 4, inner = 50, device = 0, verbose = 1;
  for (int i = 1; i < argc; i++) {
    const char *a = argv[i];
    const char *v = i + 1 < argc ? argv[i + 1] : NULL;
#define STR(flag, var)                 \
  if (!strcmp(a, flag) && v) {         \
    var = v;                           \
    i++;                               \
    continue;                          \
  }
#define INT(flag, var)                 \
  if (!strcmp(a, flag) && v) {         \
    var = atoi(v);                     \
    i++;                               \
    continue;                          \
  }
    STR("-dir", dir);
    STR("-ker_i", ker_i);
    STR("-ker_f", ker_f);
    STR("-damp_i", damp_i);
    STR("-damp_f", damp_f);
    STR("-damp_i_bycol", damp_i_c);
    STR("-damp_f_bycol", damp_f_c);
    STR("-b_k", b_k);
    STR("-x0", x0_path);
    STR("-timing", timing_path);
    INT("-row_k", row_k);
    INT("-row_d", row_d);
    INT("-col", col);
    INT("-itn", itn);
    INT("-sweeps", sweeps);
    INT("-inner", inner);
    INT("-device", device);
    STR("-col_perm", col_perm);
    if ((!strcmp(a, "-row_ptn") || !strcmp(a, "-col_ptn")) && v) {
      fprintf(stderr, "%s ignored: one GPU holds the whole problem\n", a);
      i++;
      continue;
    }
    if (!strcmp(a, "-precision") && v) {
      precision = !strcmp(v, "mixed") ? PLSQR_PREC_MIXED : PLSQR_PREC_FP64;
      i++;
      continue;
    }
    if (!strcmp(a, "-order") && v) {
      order = !strcmp(v, "reference") ? PLSQR_ORDER_REFERENCE : PLSQR_ORDER_FAST;
      i++;
      continue;
    }
    if (!strcmp(a, "-quiet")) {
      verbose = 0;
      continue;
    }
    fprintf(stderr, "%d: cannot recognize %s\n", 0, a); /* plsqr3.c:184 */
  }
  plsqr_files f;
  memset(&f, 0, sizeof(f));
  f.dir = dir;
  f.ker_f = ker_f;
  f.ker_i = ker_i;
  f.damp_f = damp_f;
  f.damp_i = damp_i;
  f.damp_f_bycol = damp_f_c;
  f.damp_i_bycol = damp_i_c;
  f.b_k = b_k;
  f.row_k = row_k;
  f.row_d = row_d;
  f.col = col;
  f.col_perm = col_perm;
  plsqr_opts o;
  plsqr_default_opts(&o);
  o.device = device;
  o.precision = precision;
  o.verbose = verbose && precision == PLSQR_PREC_FP64;
  o.order = order;
  /* one FP64 solve in the fast order needs only the unit layouts of K */
  o.lean = precision == PLSQR_PREC_FP64 && order == PLSQR_ORDER_FAST;
  plsqr_ctx *ctx = NULL;
  int rc = plsqr_ctx_create_files(&f, &o, &ctx);
  if (rc) {
    fprintf(stderr, "plsqr3_gpu: loading failed: %s\n", plsqr_strerror(rc));
    return 1;
  }
  plsqr_lsqr_args a;
  plsqr_default_lsqr_args(&a); /* call_lsqr constants, source/lsqr.c:47-51 */
  a.lsqr_iteration = itn;
  a.result_txt = "result.txt";
  a.sweeps = sweeps;
  a.inner = inner;
  double *x0 = NULL;
  if (x0_path) {
    FILE *fx = fopen(x0_path, "rb");
    x0 = (double *)malloc(sizeof(double) * (size_t)(col > 0 ? col : 1));
    const size_t got = fx && x0 ? fread(x0, sizeof(double), (size_t)col, fx) : 0;
    if (fx) fclose(fx);
    if (got != (size_t)col) {
      fprintf(stderr, "plsqr3_gpu: cannot read %d float64 values from %s\n", col, x0_path);
      free(x0);
      plsqr_ctx_destroy(ctx);
      return 1;
    }
    a.x0 = x0;
  }
  if (timing_path) plsqr_set_timing(ctx, 1);
  printf("\nStarting plsqr algorithm...procRank=%d\n", 0);
  plsqr_result r;
  rc = plsqr_lsqr(ctx, &a, NULL, NULL, NULL, NULL, NULL, &r);
  if (rc == PLSQR_OK && timing_path) {
    const int trc = plsqr_write_timing(ctx, timing_path);
    if (trc) fprintf(stderr, "plsqr3_gpu: timing report %s: %s\n", timing_path, plsqr_strerror(trc));
  }
  free(x0);
  if (rc == PLSQR_OK && x0_path) printf("x0 %s\n", r.warm ? "kept" : "not kept (cold start)");
  if (rc) {
    fprintf(stderr, "plsqr3_gpu: lsqr failed: %s (%s)\n", plsqr_strerror(rc),
            plsqr_ctx_last_error(ctx));
    plsqr_ctx_destroy(ctx);
    return 1;
  }
  char fname[256];
  snprintf(fname, sizeof(fname), "p_resultx_itn=%d_NProc=%d_float%d_mpiio.bin", itn, 1, 64);
  rc = plsqr_write_result(ctx, fname);
  plsqr_ctx_destroy(ctx);
  if (rc) {
    fprintf(stderr, "plsqr3_gpu: writing %s failed: %s\n", fname, plsqr_strerror(rc));
    return 1;
  }
  return 0;
}
