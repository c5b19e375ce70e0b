// Plain data types shared by device and host code (no device code here).
#pragma once

#include <stdint.h>

namespace plsqr {

// Maximum number of per-block partial sums a reduction kernel may write.
constexpr int kMaxParts = 16384;

struct DevState {
  // lsqr() arguments (source/lsqr.h:32-62)
  double damp, atol, btol, ctol;
  int32_t itnlim, want_se, has_ref, n_iter;
  // running scalars (source/lsqr.c:221-235)
  double alpha, beta, rhobar, phibar, bnorm, anorm, acond, dnorm, dxmax;
  double res2, psi, xnorm, xnorm1, cs2, sn2, z, rnorm, arnorm;
  double test1, test2, test3;
  double ref_norm2;  // ||x_ref||^2 when a reference solution is set
  int32_t itn, istop, nstop, maxdx;
  // values of the current iteration, written by the x/w update kernel and
  // folded into the running scalars by the tail kernel
  double s_alpha, s_rhobar, s_phibar, s_phi, s_rho, s_theta, s_tau, s_psi;
  int32_t s_beta_pos, done;
  int32_t hist_base;  // history index of this solve's iteration 0
  int32_t slot;       // batched solver: the right-hand side's history row
  double err;         // ||x - x_ref|| / ||x_ref|| after the last iteration (-1: no x_ref)
};

// One compressed-sparse operand as the kernels see it, with values of type T
// (FP64, or the FP32 high half of the value split).
template <typename T>
struct CsrT {
  const int64_t *ptr;
  const int32_t *idx;
  const T *val;
  int32_t n_lines;
};
using Csr = CsrT<double>;

}  // namespace plsqr
