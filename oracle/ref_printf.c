/* Companion of ref_printf.h (reference build only). */
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

int oracle_ref_printf(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int n = vprintf(fmt, ap);
  va_end(ap);
  const char *tag = strstr(fmt, "beta=%e") ? "beta" : strstr(fmt, "alpha=%e") ? "alpha" : NULL;
  if (tag) {
    /* both lines are printed as ("%d: <tag>=%e ...", int rank, double value) */
    va_start(ap, fmt);
    (void)va_arg(ap, int);
    double v = va_arg(ap, double);
    va_end(ap);
    printf("ORACLE_%s %.17e\n", tag, v);
  }
  return n;
}
