/*
 * Test infrastructure for the reference build only: force-included into the
 * reference lsqr.c so that the per-iteration "alpha=%e" / "beta=%e" lines it
 * prints are also emitted at full precision (%.17e), which makes the oracle's
 * alpha_k / beta_k comparable bit for bit.  Every other printf passes through.
 */
#ifndef ORACLE_REF_PRINTF_H
#define ORACLE_REF_PRINTF_H
#include <stdio.h>
int oracle_ref_printf(const char *fmt, ...);
#define printf oracle_ref_printf
#endif
