// Device-resident LSQR state and the scalar arithmetic of source/lsqr.c.
//
// All scalar steps are written with explicit round-to-nearest intrinsics
// (__dmul_rn, __dadd_rn, ...) so that nvcc cannot contract a*b+c into an FMA:
// given the same alpha_k and beta_k, the device recurrence produces the same
// bits as the reference's C code built without FMA contraction.
#pragma once

#include <stdint.h>

#include "dev_types.h"
#include "plsqr_gpu.h"

namespace plsqr {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// source/cblas.h:219-229
__device__ __forceinline__ double d2norm(double a, double b) {
  const double scale = dadd(fabs(a), fabs(b));
  if (scale == 0.0) return 0.0;
  const double as = ddiv(a, scale), bs = ddiv(b, scale);
  return dmul(scale, __dsqrt_rn(dadd(dmul(as, as), dmul(bs, bs))));
}

// Rotation of source/lsqr.c:609-636 computed from the state before the
// iteration and the new alpha, beta.  Pure function of its inputs, so every
// block of a grid computes the same values.
struct Step {
  double rhobar, phibar, psi, phi, rho, theta, tau, t1, t2, t3;
};

__device__ __forceinline__ Step lsqr_step(const DevState &s, double alpha, double beta) {
  Step o;
  double rhbar1 = s.rhobar, phibar = s.phibar, psi = s.psi;
  if (s.damp > 0.0) {
    rhbar1 = d2norm(s.rhobar, s.damp);
    const double cs1 = ddiv(s.rhobar, rhbar1), sn1 = ddiv(s.damp, rhbar1);
    psi = dmul(sn1, phibar);
    phibar = dmul(cs1, phibar);
  }
  const double rho = d2norm(rhbar1, beta);
  const double cs = ddiv(rhbar1, rho), sn = ddiv(beta, rho);
  o.theta = dmul(sn, alpha);
  o.rhobar = dmul(-cs, alpha);
  o.phi = dmul(cs, phibar);
  o.phibar = dmul(sn, phibar);
  o.tau = dmul(sn, o.phi);
  o.psi = psi;
  o.rho = rho;
  o.t1 = ddiv(o.phi, rho);
  o.t2 = ddiv(-o.theta, rho);
  o.t3 = ddiv(1.0, rho);
  return o;
}

// source/lsqr.c:703-775 plus the history record; runs on one thread.
__device__ __forceinline__ void lsqr_tail(DevState &s, double dknorm2, double err2,
                                          double x0, plsqr_iter *hist) {
  const int itn = s.itn + 1;
  s.alpha = s.s_alpha;
  s.rhobar = s.s_rhobar;
  s.phibar = s.s_phibar;
  s.psi = s.s_psi;
  const double phi = s.s_phi, rho = s.s_rho, theta = s.s_theta, tau = s.s_tau;
  const double dknorm = __dsqrt_rn(dknorm2);
  s.dnorm = d2norm(s.dnorm, dknorm);
  const double dxk = fabs(dmul(phi, dknorm));
  if (s.dxmax < dxk) {
    s.dxmax = dxk;
    s.maxdx = itn;
  }
  const double delta = dmul(s.sn2, rho);
  const double gambar = dmul(-s.cs2, rho);
  const double rhs = dsub(phi, dmul(delta, s.z));
  const double zbar = ddiv(rhs, gambar);
  s.xnorm = d2norm(s.xnorm1, zbar);
  const double gamma = d2norm(gambar, theta);
  s.cs2 = ddiv(gambar, gamma);
  s.sn2 = ddiv(theta, gamma);
  s.z = ddiv(rhs, gamma);
  s.xnorm1 = d2norm(s.xnorm1, s.z);

  s.acond = dmul(s.anorm, s.dnorm);
  s.res2 = d2norm(s.res2, s.psi);
  s.rnorm = d2norm(s.res2, s.phibar);
  s.arnorm = dmul(s.alpha, fabs(tau));

  s.test1 = ddiv(s.rnorm, s.bnorm);
  s.test2 = 0.0;
  if (s.rnorm > 0.0) s.test2 = ddiv(s.arnorm, dmul(s.anorm, s.rnorm));
  s.test3 = ddiv(1.0, s.acond);
  double t1 = ddiv(s.test1, dadd(1.0, ddiv(dmul(s.anorm, s.xnorm), s.bnorm)));
  const double rtol = dadd(s.btol, ddiv(dmul(dmul(s.atol, s.anorm), s.xnorm), s.bnorm));
  const double t3 = dadd(1.0, s.test3), t2 = dadd(1.0, s.test2);
  t1 = dadd(1.0, t1);
  int istop = s.istop;
  if (itn >= s.itnlim) istop = 5;
  if (t3 <= 1.0) istop = 4;
  if (t2 <= 1.0) istop = 2;
  if (t1 <= 1.0) istop = 1;
  if (s.test3 <= s.ctol) istop = 4;
  if (s.test2 <= s.atol) istop = 2;
  if (s.test1 <= rtol) istop = 1;
  s.istop = istop;
  s.err = s.has_ref ? __dsqrt_rn(ddiv(err2, s.ref_norm2)) : -1.0;
  if (hist) {
    plsqr_iter &h = hist[s.hist_base + itn];
    h.alpha = s.alpha;
    h.beta = s.beta;
    h.rnorm = s.rnorm;
    h.arnorm = s.arnorm;
    h.test1 = s.test1;
    h.test2 = s.test2;
    h.anorm = s.anorm;
    h.acond = s.acond;
    h.xnorm = s.xnorm;
    h.x0 = x0;
    h.err = s.err;
    h.istop = istop;
    h.pad = 0;
  }
  // source/lsqr.c:820-827 (nconv = 1)
  if (istop == 0) {
    s.nstop = 0;
  } else {
    s.nstop = s.nstop + 1;
    if (s.nstop < 1 && itn < s.itnlim) s.istop = 0;
  }
  s.itn = itn;
}

}  // namespace plsqr
