/*
 * ORACLE — test infrastructure, not product code (see plsqr_oracle.h).
 *
 * FP64 restatement of the reference PLSQR3 CPU path on one rank.  On one rank
 * every MPI step of the reference is a copy (Allreduce of t_k,
 * aprod_impl.c:121; Allreduce of a squared partial norm, mycblas.c:176) and
 * the extended vectors equal the local ones (tridiagonal.c:80-85), so they are
 * written here as the copies they are.  Loop orders and expression shapes
 * follow the reference line by line; build with -ffp-contract=off.
 */
#include "plsqr_oracle.h"

#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* group_size_omp = 10 * threads (source/plsqr3.c:44-58) */
static int group_size(void) {
#ifdef _OPENMP
  return 10 * omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* source/CPUSpMV.c:162-183 (serial column scatter) */
void oracle_spmv_csc(const oracle_sparse *a, const double *x, double *ax) {
  for (int c = 0; c < a->num_col; ++c) {
    const double xc = x[c];
    for (int64_t e = a->ptr[c]; e < a->ptr[c + 1]; ++e)
      ax[a->idx[e]] += a->val[e] * xc;
  }
}

/* source/CPUSpMV.c:50-89 (row gather, OpenMP dynamic schedule) */
void oracle_spmv_csr(const oracle_sparse *a, const double *x, int start, double *ax) {
  const int m = a->num_row;
  const int chunk = (m + group_size() - 1) / group_size();
#pragma omp parallel for schedule(dynamic, chunk > 0 ? chunk : 1)
  for (int r = 0; r < m; ++r) {
    double t = ax[r];
    for (int64_t e = a->ptr[r]; e < a->ptr[r + 1]; ++e)
      t += a->val[e] * x[a->idx[e] - start];
    ax[r] = t;
  }
}

/* source/CPUSpMV.c:203-245 and 255-296 (column gather, OpenMP) */
void oracle_spmvT_csc(const oracle_sparse *a, const double *y, int start, double *tay) {
  const int n = a->num_col;
  const int chunk = (n + group_size() - 1) / group_size();
#pragma omp parallel for schedule(dynamic, chunk > 0 ? chunk : 1)
  for (int c = 0; c < n; ++c) {
    double t = tay[c];
    for (int64_t e = a->ptr[c]; e < a->ptr[c + 1]; ++e)
      t += a->val[e] * y[a->idx[e] - start];
    tay[c] = t;
  }
}

/* source/mycblas.c:182-222 */
double oracle_dnrm2(int64_t n, const double *v) {
  double scale = 0.0, ssq = 1.0;
  if (n <= 0) return 0;
  if (n == 1) return fabs(v[0]);
  for (int64_t i = 0; i < n; ++i) {
    const double xi = v[i];
    if (xi != 0.0) {
      const double ax = fabs(xi);
      if (scale < ax) {
        ssq = 1.0 + ssq * (scale / ax) * (scale / ax);
        scale = ax;
      } else {
        ssq += (ax / scale) * (ax / scale);
      }
    }
  }
  return scale * sqrt(ssq);
}

/* source/mycblas.c:158-180 on one rank: the Allreduce of the square is a copy */
static double dnrm2_parallel(int64_t n, const double *v) {
  const double part = oracle_dnrm2(n, v);
  const double square = part * part;
  return sqrt(square);
}

/* source/mycblas.c:99-133 */
static double dnrm2_forVecY(const oracle_problem *p) {
  const double pk = oracle_dnrm2(p->k_csc.num_row, p->y_k);
  const double pd = dnrm2_parallel(p->d_csr.num_row, p->y_d);
  return sqrt(pk * pk + pd * pd);
}

/* source/mycblas.c:286-309 */
static void dscal(int64_t n, double alpha, double *v) {
  const int64_t chunk = (n + group_size() - 1) / group_size();
#pragma omp parallel for schedule(dynamic, chunk > 0 ? chunk : 1)
  for (int64_t i = 0; i < n; ++i) v[i] *= alpha;
}

/* source/mycblas.c:240-273 */
static void dscal_plsqr3(oracle_problem *p, double alpha) {
  dscal(p->k_csc.num_row, alpha, p->y_k);
  dscal(p->d_csr.num_row, alpha, p->y_d);
}

/* source/cblas.h:219-229 */
double oracle_d2norm(double a, double b) {
  const double scale = fabs(a) + fabs(b);
  if (scale == 0.0) return 0.0;
  return scale * sqrt((a / scale) * (a / scale) + (b / scale) * (b / scale));
}

/* source/aprod_impl.c:22-267, single rank */
static int aprod_mode_1(oracle_problem *p) {
  const int mk = p->k_csc.num_row, md = p->d_csr.num_row, n = p->k_csc.num_col;
  double *t_k = calloc(mk > 0 ? mk : 1, sizeof(double));
  double *t_d = calloc(md > 0 ? md : 1, sizeof(double));
  double *ext_x = malloc((n > 0 ? n : 1) * sizeof(double));
  if (!t_k || !t_d || !ext_x) {
    free(t_k); free(t_d); free(ext_x);
    return -1;
  }
  oracle_spmv_csc(&p->k_csc, p->x, t_k);            /* :86 */
  /* :121 Allreduce on one rank: t_k_allreduce == t_k */
  {
    const int chunk = (mk + 32 * 5 - 1) / (32 * 5); /* :136 */
#pragma omp parallel for schedule(dynamic, chunk > 0 ? chunk : 1)
    for (int i = 0; i < mk; ++i) p->y_k[i] += t_k[i]; /* :138-140 */
  }
  memcpy(ext_x, p->x, (size_t)n * sizeof(double));   /* :157-159 */
  oracle_spmv_csr(&p->d_csr, ext_x, 0, t_d);          /* :221 */
  for (int i = 0; i < md; ++i) p->y_d[i] += t_d[i];   /* :222-224 */
  free(t_k); free(t_d); free(ext_x);
  return 0;
}

/* source/aprod_impl.c:276-524, single rank */
static int aprod_mode_2(oracle_problem *p) {
  const int md = p->d_csr.num_row, n = p->k_csc.num_col;
  double *s_k = calloc(n > 0 ? n : 1, sizeof(double));
  double *s_d = calloc(n > 0 ? n : 1, sizeof(double));
  double *ext_y = malloc((md > 0 ? md : 1) * sizeof(double));
  if (!s_k || !s_d || !ext_y) {
    free(s_k); free(s_d); free(ext_y);
    return -1;
  }
  oracle_spmvT_csc(&p->k_csc, p->y_k, 0, s_k);        /* :344/354 */
  memcpy(ext_y, p->y_d, (size_t)md * sizeof(double)); /* :398-402 */
  oracle_spmvT_csc(&p->d_csc, ext_y, 0, s_d);          /* :462/484 */
  for (int i = 0; i < n; ++i) p->x[i] += (s_k[i] + s_d[i]); /* :465-467 */
  free(s_k); free(s_d); free(ext_y);
  return 0;
}

int oracle_aprod(int mode, oracle_problem *p) {
  if (mode == 1) return aprod_mode_1(p);
  if (mode == 2) return aprod_mode_2(p);
  return -2;
}

/* The Paige-Saunders log strings of source/lsqr.c:246-268; the log format
 * is an output contract, so the text is kept identical. */
static const char fmt_1000[] = " %s        Least-squares solution of  Ax = b\n"
                               " The matrix  A  has %7d rows  and %7d columns\n"
                               " damp   = %-22.2e    wantse = %10i\n"
                               " atol   = %-22.2e    conlim = %10.2e\n"
                               " btol   = %-22.2e    itnlim = %10d\n\n";
static const char fmt_1200[] = "    Itn       x(1)           Function"
                               "     Compatible    LS      Norm A   Cond A\n";
static const char fmt_1300[] = "    Itn       x(1)           Function"
                               "     Compatible    LS      Norm Abar   Cond Abar\n";
static const char fmt_1500[] = " %6d %16.9e %16.9e %9.2e %9.2e %8.1e %8.1e\n";
static const char fmt_1550[] = " %6d %16.9e %16.9e %9.2e %9.2e\n";
static const char fmt_1600[] = "\n";
static const char fmt_2000[] = "\n"
                               " %s       istop  = %-10d      itn    = %-10d\n"
                               " %s       anorm  = %11.5e     acond  = %11.5e\n"
                               " %s       vnorm  = %11.5e     xnorm  = %11.5e\n"
                               " %s       rnorm  = %11.5e     arnorm = %11.5e\n";
static const char fmt_2100[] = " %s       max dx = %7.1e occured at itn %-9d\n"
                               " %s              = %7.1e*xnorm\n";
static const char fmt_3000[] = " %s       %s\n";
static const char *const msg[6] = {
    "The exact solution is  x = 0",
    "A solution to Ax = b was found, given atol, btol",
    "A least-squares solution was found, given atol",
    "A damped least-squares solution was found, given atol",
    "Cond(Abar) seems to be too large, given conlim",
    "The iteration limit was reached"};

/* The built-in operator in the callback's form. */
static int builtin_aprod(int mode, int m, int n, oracle_problem *p, void *usr, int is_final,
                         int iteration) {
  (void)m, (void)n, (void)usr, (void)is_final, (void)iteration;
  return oracle_aprod(mode, p);
}

int oracle_lsqr(oracle_problem *p, double damp, double atol, double btol,
                double conlim, int itnlim, int lsqr_iteration, double *w,
                double *x, double *se, oracle_iter *hist, oracle_result *res,
                const char *result_txt) {
  return oracle_lsqr_op(p, builtin_aprod, NULL, damp, atol, btol, conlim, itnlim,
                        lsqr_iteration, w, x, se, hist, res, result_txt);
}

/* source/lsqr.c:195-917, one rank; the operator is called where and as the
 * reference calls its aprod argument (lsqr.c:366, 491-507, 564) */
int oracle_lsqr_op(oracle_problem *p, oracle_aprod_fn op, void *usr, double damp,
                   double atol, double btol, double conlim, int itnlim,
                   int lsqr_iteration, double *w, double *x, double *se,
                   oracle_iter *hist, oracle_result *res, const char *result_txt) {
  const int n = p->k_csc.num_col;
  const int num_row = p->k_csc.num_row + p->d_csr.num_row;
  const bool damped = damp > 0.0;
  const bool wantse = se != NULL;
  const char enter[] = "Enter LSQR.  ", exit_[] = "Exit  LSQR.  ";
  FILE *nout = NULL;
  if (result_txt) {
    nout = fopen(result_txt, "w");
    if (!nout) return -1;
  }

  int istop = 0, itn = 0, nstop = 0, maxdx = 0, nconv;
  double anorm = 0, acond = 0, rnorm = 0, arnorm = 0, xnorm = 0;
  double alpha, arnorm0, beta, bnorm = 0, cs, cs1, cs2, ctol, delta, dknorm,
      dnorm, dxk, dxmax, gamma, gambar, phi, phibar, psi, res2, rho, rhobar,
      rhbar1, rhs, rtol, sn, sn1, sn2, t, tau, temp, test1 = 0, test2 = 0,
      test3, theta, t1, t2, t3, xnorm1, z, zbar;
  (void)arnorm0;
  double loop_seconds = 0.0; /* stays 0 when the start-up ends the solve (:400-401) */

  if (nout) fprintf(nout, fmt_1000, enter, num_row, n, damp, (int)wantse, atol,
                    conlim, btol, itnlim);
  ctol = 0.0;
  if (conlim > 0.0) ctol = 1.0 / conlim;
  dnorm = 0; dxmax = 0; res2 = 0; psi = 0; xnorm1 = 0; cs2 = -1.0; sn2 = 0; z = 0;

  /* :311-314 */
  for (int i = 0; i < n; ++i) p->x[i] = 0.0;
  for (int i = 0; i < n; ++i) x[i] = 0.0;
  if (wantse) for (int i = 0; i < n; ++i) se[i] = 0.0;

  alpha = 0.0;
  beta = dnrm2_forVecY(p); /* :343 */
  if (beta > 0.0) {
    dscal_plsqr3(p, 1.0 / beta); /* :361 */
    if (op(2, num_row, n, p, usr, 0, 0)) goto fail; /* :366 */
    alpha = dnrm2_parallel(n, p->x); /* :375 */
  }
  if (alpha > 0.0) { /* :392-395 */
    dscal(n, 1.0 / alpha, p->x);
    memcpy(w, p->x, (size_t)n * sizeof(double));
  }
  arnorm = arnorm0 = alpha * beta;
  if (hist) {
    memset(&hist[0], 0, sizeof(hist[0]));
    hist[0].alpha = alpha;
    hist[0].beta = beta;
    hist[0].rnorm = beta;
    hist[0].arnorm = arnorm;
    hist[0].x0 = n > 0 ? x[0] : 0.0;
  }
  if (arnorm == 0.0) goto goto_800; /* :400-401 */

  rhobar = alpha;
  phibar = beta;
  bnorm = beta;
  rnorm = beta;
  if (nout) {
    fprintf(nout, damped ? fmt_1300 : fmt_1200);
    test1 = 1.0;
    test2 = alpha / beta;
    fprintf(nout, fmt_1550, itn, x[0], rnorm, test1, test2);
    fprintf(nout, fmt_1600);
  }

  struct timespec t_loop0, t_loop1; /* :476-478 */
  clock_gettime(CLOCK_MONOTONIC, &t_loop0);
  if (lsqr_iteration > 0)
    while (1) { /* :480-837 */
      itn = itn + 1;
      const int last = itn == lsqr_iteration; /* :491-494 */
      dscal_plsqr3(p, -alpha); /* :502 */
      if (op(1, num_row, n, p, usr, last, itn)) goto fail; /* :507 */
      beta = dnrm2_forVecY(p);   /* :516 */
      temp = oracle_d2norm(alpha, beta);
      temp = oracle_d2norm(temp, damp);
      anorm = oracle_d2norm(anorm, temp);
      if (beta > 0.0) {
        dscal_plsqr3(p, 1.0 / beta); /* :538 */
        dscal(n, -beta, p->x);       /* :558 */
        if (op(2, num_row, n, p, usr, last, itn)) goto fail; /* :564 */
        alpha = dnrm2_parallel(n, p->x);   /* :577 */
        if (alpha > 0.0) dscal(n, 1.0 / alpha, p->x); /* :595 */
      }
      /* :609-629 */
      rhbar1 = rhobar;
      if (damped) {
        rhbar1 = oracle_d2norm(rhobar, damp);
        cs1 = rhobar / rhbar1;
        sn1 = damp / rhbar1;
        psi = sn1 * phibar;
        phibar = cs1 * phibar;
      }
      rho = oracle_d2norm(rhbar1, beta);
      cs = rhbar1 / rho;
      sn = beta / rho;
      theta = sn * alpha;
      rhobar = -cs * alpha;
      phi = cs * phibar;
      phibar = sn * phibar;
      tau = sn * phi;
      /* :634-692 */
      t1 = phi / rho;
      t2 = -theta / rho;
      t3 = 1.0 / rho;
      dknorm = 0.0;
      if (wantse) {
        for (int i = 0; i < n; ++i) {
          t = w[i];
          x[i] = t1 * t + x[i];
          w[i] = t2 * t + p->x[i];
          t = (t3 * t) * (t3 * t);
          se[i] = t + se[i];
          dknorm = t + dknorm;
        }
      } else {
        for (int i = 0; i < n; ++i) {
          t = w[i];
          x[i] = t1 * t + x[i];
          w[i] = t2 * t + p->x[i];
          dknorm = (t3 * t) * (t3 * t) + dknorm;
        }
      }
      /* :703-775 */
      dknorm = sqrt(dknorm);
      dnorm = oracle_d2norm(dnorm, dknorm);
      dxk = fabs(phi * dknorm);
      if (dxmax < dxk) {
        dxmax = dxk;
        maxdx = itn;
      }
      delta = sn2 * rho;
      gambar = -cs2 * rho;
      rhs = phi - delta * z;
      zbar = rhs / gambar;
      xnorm = oracle_d2norm(xnorm1, zbar);
      gamma = oracle_d2norm(gambar, theta);
      cs2 = gambar / gamma;
      sn2 = theta / gamma;
      z = rhs / gamma;
      xnorm1 = oracle_d2norm(xnorm1, z);

      acond = anorm * dnorm;
      res2 = oracle_d2norm(res2, psi);
      rnorm = oracle_d2norm(res2, phibar);
      arnorm = alpha * fabs(tau);

      test1 = rnorm / bnorm;
      test2 = 0.0;
      if (rnorm > 0.0) test2 = arnorm / (anorm * rnorm);
      test3 = 1.0 / acond;
      t1 = test1 / (1.0 + anorm * xnorm / bnorm);
      rtol = btol + atol * anorm * xnorm / bnorm;
      t3 = 1.0 + test3;
      t2 = 1.0 + test2;
      t1 = 1.0 + t1;
      if (itn >= itnlim) istop = 5;
      if (t3 <= 1.0) istop = 4;
      if (t2 <= 1.0) istop = 2;
      if (t1 <= 1.0) istop = 1;
      if (test3 <= ctol) istop = 4;
      if (test2 <= atol) istop = 2;
      if (test1 <= rtol) istop = 1;

      if (hist) {
        oracle_iter *h = &hist[itn];
        h->alpha = alpha; h->beta = beta; h->rnorm = rnorm; h->arnorm = arnorm;
        h->test1 = test1; h->test2 = test2; h->anorm = anorm; h->acond = acond;
        h->xnorm = xnorm; h->x0 = n > 0 ? x[0] : 0.0; h->istop = istop;
      }

      /* :780-811 */
      if (nout) {
        bool print = n <= 40 || itn <= 10 || itn >= itnlim - 10 || itn % 10 == 0 ||
                     test3 <= 2.0 * ctol || test2 <= 10.0 * atol ||
                     test1 <= 10.0 * rtol || istop != 0;
        if (print) fprintf(nout, fmt_1500, itn, x[0], rnorm, test1, test2, anorm, acond);
      }
      /* :820-827 */
      if (istop == 0) {
        nstop = 0;
      } else {
        nconv = 1;
        nstop = nstop + 1;
        if (nstop < nconv && itn < itnlim) istop = 0;
      }
      if (itn == lsqr_iteration) break; /* :833 */
    }
  clock_gettime(CLOCK_MONOTONIC, &t_loop1); /* :836-842 */
  loop_seconds =
      (double)(t_loop1.tv_sec - t_loop0.tv_sec) + 1e-9 * (double)(t_loop1.tv_nsec - t_loop0.tv_nsec);

  /* :878-891 */
  if (wantse) {
    t = 1.0;
    if (num_row > n) t = num_row - n;
    if (damped) t = num_row;
    t = rnorm / sqrt(t);
    for (int i = 0; i < n; ++i) se[i] = t * sqrt(se[i]);
  }

goto_800:
  if (damped && istop == 2) istop = 3;
  if (nout) {
    fprintf(nout, fmt_2000, exit_, istop, itn, exit_, anorm, acond, exit_, bnorm,
            xnorm, exit_, rnorm, arnorm);
    fprintf(nout, fmt_2100, exit_, dxmax, maxdx, exit_, dxmax / (xnorm + 1.0e-20));
    fprintf(nout, fmt_3000, exit_, msg[istop]);
    fclose(nout);
  }
  if (res) {
    res->istop = istop; res->itn = itn; res->anorm = anorm; res->acond = acond;
    res->rnorm = rnorm; res->arnorm_out = test2; res->xnorm = xnorm;
    res->arnorm = arnorm; res->bnorm = bnorm; res->dxmax = dxmax; res->maxdx = maxdx;
    res->loop_seconds = loop_seconds;
  }
  return 0;

fail:
  if (nout) fclose(nout);
  return -3;
}
