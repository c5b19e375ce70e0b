// The solver's text outputs: the Paige-Saunders log that the reference writes
// to result.txt (source/lsqr.c:246-268 formats, 271-276 header, 430-445 start
// line, 780-811 per-iteration lines, 895-905 exit block) and the per-iteration
// alpha/beta lines it prints on stdout (lsqr.c:352, 383, 489, 521, 579, 841).
// The log format is an output contract, so the format strings are the
// reference's.  The lines are produced from the per-iteration history that the
// device records, after the solve.
#include <stdio.h>
#include <string.h>

#include "plsqr_internal.h"

namespace {

const char fmt_1000[] = " %s        Least-squares solution of  Ax = b\n"
                        " The matrix  A  has %7d rows  and %7d columns\n"
                        " damp   = %-22.2e    wantse = %10i\n"
                        " atol   = %-22.2e    conlim = %10.2e\n"
                        " btol   = %-22.2e    itnlim = %10d\n\n";
const char fmt_1200[] = "    Itn       x(1)           Function"
                        "     Compatible    LS      Norm A   Cond A\n";
const char fmt_1300[] = "    Itn       x(1)           Function"
                        "     Compatible    LS      Norm Abar   Cond Abar\n";
const char fmt_1500[] = " %6d %16.9e %16.9e %9.2e %9.2e %8.1e %8.1e\n";
const char fmt_1550[] = " %6d %16.9e %16.9e %9.2e %9.2e\n";
const char fmt_1600[] = "\n";
const char fmt_2000[] = "\n"
                        " %s       istop  = %-10d      itn    = %-10d\n"
                        " %s       anorm  = %11.5e     acond  = %11.5e\n"
                        " %s       vnorm  = %11.5e     xnorm  = %11.5e\n"
                        " %s       rnorm  = %11.5e     arnorm = %11.5e\n";
const char fmt_2100[] = " %s       max dx = %7.1e occured at itn %-9d\n"
                        " %s              = %7.1e*xnorm\n";
const char fmt_3000[] = " %s       %s\n";
const char *const msg[6] = {"The exact solution is  x = 0",
                            "A solution to Ax = b was found, given atol, btol",
                            "A least-squares solution was found, given atol",
                            "A damped least-squares solution was found, given atol",
                            "Cond(Abar) seems to be too large, given conlim",
                            "The iteration limit was reached"};

}  // namespace

// itn < 0: the start-up found arnorm == 0 and the loop never ran
// (source/lsqr.c:400-401): only the header and the exit block are written.
int write_result_txt(const char *path, int num_row, int n, const plsqr_lsqr_args *a,
                     const plsqr_iter *hist, int itn, const plsqr_result *r) {
  FILE *f = fopen(path, "w");
  if (!f) return PLSQR_ERR_IO;
  const char enter[] = "Enter LSQR.  ", exit_[] = "Exit  LSQR.  ";
  const bool damped = a->damp > 0.0;
  const double ctol = a->conlim > 0.0 ? 1.0 / a->conlim : 0.0;
  fprintf(f, fmt_1000, enter, num_row, n, a->damp, (int)(a->want_se != 0), a->atol, a->conlim,
          a->btol, a->itnlim);
  if (itn >= 0) {
    fprintf(f, damped ? fmt_1300 : fmt_1200);
    const double beta = hist[0].beta, alpha = hist[0].alpha;
    fprintf(f, fmt_1550, 0, 0.0, beta, 1.0, alpha / beta);
    fprintf(f, fmt_1600);
    const double bnorm = beta;
    for (int k = 1; k <= itn; ++k) {
      const plsqr_iter &h = hist[k];
      const double test3 = 1.0 / h.acond;
      const double rtol = a->btol + a->atol * h.anorm * h.xnorm / bnorm;
      const bool print = n <= 40 || k <= 10 || k >= a->itnlim - 10 || k % 10 == 0 ||
                         test3 <= 2.0 * ctol || h.test2 <= 10.0 * a->atol ||
                         h.test1 <= 10.0 * rtol || h.istop != 0;
      if (print) fprintf(f, fmt_1500, k, h.x0, h.rnorm, h.test1, h.test2, h.anorm, h.acond);
    }
  }
  fprintf(f, fmt_2000, exit_, r->istop, r->itn, exit_, r->anorm, r->acond, exit_, r->bnorm,
          r->xnorm, exit_, r->rnorm, r->arnorm);
  fprintf(f, fmt_2100, exit_, r->dxmax, r->maxdx, exit_, r->dxmax / (r->xnorm + 1.0e-20));
  const int is = (r->istop >= 0 && r->istop < 6) ? r->istop : 0;
  fprintf(f, fmt_3000, exit_, msg[is]);
  return fclose(f) == 0 ? PLSQR_OK : PLSQR_ERR_IO;
}

void print_iterations(const plsqr_iter *hist, int itn, double seconds) {
  printf("------------------------iteration=%d----------------------------------\n", 0);
  printf("%d: beta=%e from vector y\n", 0, hist[0].beta);
  if (hist[0].beta > 0.0) printf("%d: alpha=%e from vector x\n", 0, hist[0].alpha);
  for (int k = 1; k <= itn; ++k) {
    printf("------------------------iteration=%d----------------------------------\n", k);
    printf("%d: beta=%e from vector y\n", 0, hist[k].beta);
    if (hist[k].beta > 0.0) printf("%d: alpha=%e from vector x\n", 0, hist[k].alpha);
  }
  printf("Parallel LSQR time=%lf s\n", seconds);
  fflush(stdout);
}
