/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C FP64 restatement of the reference PLSQR3 CPU path for one rank:
 * the LSQR driver (source/lsqr.c:195-917), the operator aprod in its
 * tridiagonal form (source/aprod_impl.c:22-524), the CPU SpMV kernels
 * (source/CPUSpMV.c) and the BLAS-1 norm and scale helpers
 * (source/mycblas.c, source/cblas.h).  Every operation is done in the order
 * the reference does it, so that, compiled with the same flags, it returns the
 * same bits as the reference built with SDVERSION=2.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
 * library, and only as the reference that results are compared with or as
 * the timed CPU baseline.
 */
#ifndef PLSQR_ORACLE_H
#define PLSQR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Compressed sparse matrix, either by column (ptr over columns, idx = row)
 * or by row (ptr over rows, idx = column); mirrors SpMatCSC / SpMatCSR
 * (source/main.h:123-130, 158-165) with a 64-bit pointer array. */
typedef struct {
  int num_row;
  int num_col;
  int64_t nnz;
  const int64_t *ptr;
  const int32_t *idx;
  const double *val;
} oracle_sparse;

/* Single-rank PPDataV3_TRI (source/main.h:397-494): the kernel matrix by
 * column, the damping matrix by row and by column, and the three vectors the
 * operator updates in place. */
typedef struct {
  oracle_sparse k_csc;   /* m_k x n, by column */
  oracle_sparse d_csr;   /* m_d x n, by row */
  oracle_sparse d_csc;   /* m_d x n, by column */
  double *y_k;           /* [m_k] kernel part of u */
  double *y_d;           /* [m_d] damping part of u */
  double *x;             /* [n]   v */
} oracle_problem;

/* Per-iteration record of the scalars lsqr() computes (index 0 = start-up). */
typedef struct {
  double alpha, beta, rnorm, arnorm, test1, test2, anorm, acond, xnorm, x0;
  int istop;
} oracle_iter;

typedef struct {
  int istop, itn;
  double anorm, acond, rnorm, arnorm_out /* = test2, source/lsqr.c:913 */, xnorm;
  double arnorm; /* alpha*|tau| of the last iteration */
  double bnorm, dxmax;
  int maxdx;
  /* wall time of the iteration loop, the region of the reference's
   * "Parallel LSQR time" (source/lsqr.c:476-478, 836-842) */
  double loop_seconds;
} oracle_result;

/* source/CPUSpMV.c:162-183  Ax[row_idx[e]] += val[e]*x[col], columns ascending */
void oracle_spmv_csc(const oracle_sparse *a, const double *x, double *ax);
/* source/CPUSpMV.c:50-89    Ax[r] = Ax[r] + sum_e val[e]*x[col_idx[e]-start] */
void oracle_spmv_csr(const oracle_sparse *a, const double *x, int start, double *ax);
/* source/CPUSpMV.c:203-296  tAy[c] = tAy[c] + sum_e val[e]*y[row_idx[e]-start] */
void oracle_spmvT_csc(const oracle_sparse *a, const double *y, int start, double *tay);
/* source/mycblas.c:182-222  scaled sum of squares 2-norm */
double oracle_dnrm2(int64_t n, const double *v);
/* source/cblas.h:219-229 */
double oracle_d2norm(double a, double b);

/* source/aprod.c:24-84 with aprod_impl.c:22-267 (mode 1: y += A x) and
 * aprod_impl.c:276-524 (mode 2: x += A^T y), single rank. */
int oracle_aprod(int mode, oracle_problem *p);

/* source/lsqr.c:195-917 with damp, atol, btol, conlim, itnlim as the caller
 * passes them (call_lsqr uses 0, 1e-10, 1e-10, 100, 1000: lsqr.c:47-51).
 * On entry p->y_k holds b_k, p->y_d zero; v (p->x), w, x are overwritten.
 * hist may be NULL, else it has lsqr_iteration+1 entries.  result_txt may be
 * NULL, else the Paige-Saunders log the reference writes to result.txt is
 * written there.  Returns 0, or -1 if result_txt cannot be opened. */
int oracle_lsqr(oracle_problem *p, double damp, double atol, double btol,
                double conlim, int itnlim, int lsqr_iteration, double *w,
                double *x, double *se, oracle_iter *hist, oracle_result *res,
                const char *result_txt);

/* The operator as lsqr() receives it (source/aprod.h:10-13 for one rank:
 * the version, rank and size arguments dropped, the vectors in p):
 * mode 1 updates p->y_k / p->y_d with A p->x, mode 2 updates p->x with
 * A^T [p->y_k; p->y_d]; m, n, isFinalIteration and iteration as lsqr.c
 * passes them (:366, :491-507, :564).  Returns 0, or non-zero to stop the
 * solve with an error. */
typedef int (*oracle_aprod_fn)(int mode, int m, int n, oracle_problem *p, void *usr,
                               int is_final, int iteration);

/* oracle_lsqr with the operator supplied by the caller (usr is passed
 * through): the reference's loop driving another implementation of aprod. */
int oracle_lsqr_op(oracle_problem *p, oracle_aprod_fn op, void *usr, double damp,
                   double atol, double btol, double conlim, int itnlim,
                   int lsqr_iteration, double *w, double *x, double *se,
                   oracle_iter *hist, oracle_result *res, const char *result_txt);

/* Number of OpenMP threads the oracle runs with (0 = OpenMP default). */
void oracle_set_threads(int nthreads);
int oracle_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
