// Kernels of the mixed-precision solver: FP32 inner LSQR sweeps on the high
// half of the FP32 hi+lo value split, FP64 outer residual over hi+lo.
//
// Inner sweep: the kernel matrix is read as {int32 index, FP32 hi} (8 bytes
// per nonzero instead of 12), u, v, w, dx are FP32, every norm is accumulated
// in FP64 and the scalar recurrence is the FP64 one of lsqr_state.cuh.  The
// damping matrix (1% of the nonzeros) stays FP64 in memory and is rounded to
// FP32 when read.  Outer step: r = b - A x in FP64 with value = hi + lo.
#pragma once

#include "kernels_fp64.cuh"

namespace plsqr {

// The kernel matrix by row with both halves of the value split.
struct CsrF {
  const int64_t *ptr;
  const int32_t *idx;
  const float *hi;
  const float *lo;
  int32_t n_lines;
};

// Sum of (hi[e] + lo[e]) * x[idx[e]] in FP64 by one warp.
__device__ __forceinline__ double warp_dot_hilo(const int32_t *__restrict__ idx,
                                                const float *__restrict__ hi,
                                                const float *__restrict__ lo,
                                                const double *__restrict__ x, int64_t beg,
                                                int64_t end, int lane) {
  double acc0 = 0.0, acc1 = 0.0;
  int64_t a4 = (beg + 3) & ~int64_t(3);
  if (a4 > end) a4 = end;
  if (beg + lane < a4)
    acc0 = ((double)hi[beg + lane] + (double)lo[beg + lane]) * x[idx[beg + lane]];
  const int64_t e4 = a4 + ((end - a4) & ~int64_t(3));
  const int4 *__restrict__ idx4 = reinterpret_cast<const int4 *>(idx);
  const float4 *__restrict__ hi4 = reinterpret_cast<const float4 *>(hi);
  const float4 *__restrict__ lo4 = reinterpret_cast<const float4 *>(lo);
  for (int64_t g = (a4 >> 2) + lane; g < (e4 >> 2); g += 32) {
    const int4 c = __ldg(idx4 + g);
    const float4 h = __ldg(hi4 + g), l = __ldg(lo4 + g);
    acc0 = fma((double)h.x + (double)l.x, __ldg(x + c.x), acc0);
    acc1 = fma((double)h.y + (double)l.y, __ldg(x + c.y), acc1);
    acc0 = fma((double)h.z + (double)l.z, __ldg(x + c.z), acc0);
    acc1 = fma((double)h.w + (double)l.w, __ldg(x + c.w), acc1);
  }
  if (e4 + lane < end)
    acc1 = fma((double)hi[e4 + lane] + (double)lo[e4 + lane], x[idx[e4 + lane]], acc1);
  double s = acc0 + acc1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// Value split: hi = fl32(v), lo = fl32(v - hi).
static __global__ void k_split_hilo(const double *__restrict__ v, int64_t nnz, float *__restrict__ hi,
                             float *__restrict__ lo) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double x = v[e];
    const float h = __double2float_rn(x);
    hi[e] = h;
    if (lo) lo[e] = __double2float_rn(x - (double)h);
  }
}

// Outer residual r = [b_k; 0] - A x in FP64 (kernel values hi + lo, damping
// values FP64), into u; per-block partial sums of squares as k_aprod1.
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_residual(CsrF K, Csr D, const int32_t *__restrict__ kpart, const double *__restrict__ x,
               const double *__restrict__ b, double *__restrict__ u, int gk,
               double *__restrict__ parts) {
  __shared__ double smem[kThreads / 32];
  double sq = 0.0;
  if ((int)blockIdx.x < gk) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    const int r1 = kpart[w + 1];
    for (int r = kpart[w]; r < r1; ++r) {
      const double t = warp_dot_hilo(K.idx, K.hi, K.lo, x, K.ptr[r], K.ptr[r + 1], lane);
      if (lane == 0) {
        const double y = b[r] - t;
        u[r] = y;
        sq = fma(y, y, sq);
      }
    }
  } else {
    const int gd = gridDim.x - gk;
    double *ud = u + K.n_lines;
    for (int r = (blockIdx.x - gk) * kThreads + threadIdx.x; r < D.n_lines; r += gd * kThreads) {
      double t = 0.0;
      for (int64_t e = D.ptr[r]; e < D.ptr[r + 1]; ++e) t = fma(D.val[e], x[D.idx[e]], t);
      const double y = -t;
      ud[r] = y;
      sq = fma(y, y, sq);
    }
  }
  const double bs = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0) parts[blockIdx.x] = bs;
}

// uf = fl32(u) (u already scaled by 1/beta in FP64)
static __global__ void k_to_f32(const double *__restrict__ u, int64_t m, float *__restrict__ uf) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    uf[i] = __double2float_rn(u[i]);
}

// Inner N2: alpha, v *= 1/alpha, FP64 rotation, FP32 dx/w update; error of
// x_outer + dx against the reference solution.  start = 1: w = v, dx = 0.
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_update_dx_f32(float *__restrict__ v, float *__restrict__ w, float *__restrict__ dx,
                    const double *__restrict__ x_outer, const double *__restrict__ xref, int n,
                    const double *__restrict__ parts, int gp, DevState *__restrict__ st,
                    double *__restrict__ parts_dk, double *__restrict__ parts_err, int start) {
  __shared__ double smem[kThreads / 32];
  __shared__ double s_alpha, s_ra;
  __shared__ Step s_step;
  const int beta_pos = st->s_beta_pos;
  const double vv = beta_pos ? sum_parts<kThreads>(parts, gp, smem) : 0.0;
  if (threadIdx.x == 0) {
    double alpha = st->alpha;
    if (beta_pos) alpha = __dsqrt_rn(vv);
    if (start && !beta_pos) alpha = 0.0;
    s_alpha = alpha;
    s_ra = (beta_pos && alpha > 0.0) ? ddiv(1.0, alpha) : 0.0;
    if (!start) s_step = lsqr_step(*st, alpha, st->beta);
  }
  __syncthreads();
  const float ra = (float)s_ra;
  if (start) {
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
      float vi = v[i];
      if (ra != 0.f) vi *= ra;
      v[i] = vi;
      w[i] = ra != 0.f ? vi : 0.f;
      dx[i] = 0.f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      const double alpha = s_alpha, beta = st->beta;
      st->alpha = alpha;
      st->arnorm = dmul(alpha, beta);
      st->rhobar = alpha;
      st->phibar = beta;
      st->bnorm = beta;
      st->rnorm = beta;
      st->done = st->arnorm == 0.0;
    }
    return;
  }
  const Step sp = s_step;
  const float t1 = (float)sp.t1, t2 = (float)sp.t2, t3 = (float)sp.t3;
  double dk = 0.0, e2 = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    float vi = v[i];
    if (ra != 0.f) {
      vi *= ra;
      v[i] = vi;
    }
    const float t = w[i];
    const float d = fmaf(t1, t, dx[i]);
    dx[i] = d;
    w[i] = fmaf(t2, t, vi);
    const float tt = (t3 * t) * (t3 * t);
    dk += (double)tt;
    if (xref) {
      const double e = (x_outer[i] + (double)d) - xref[i];
      e2 = fma(e, e, e2);
    }
  }
  const double bdk = block_sum<kThreads>(dk, smem);
  const double be2 = xref ? block_sum<kThreads>(e2, smem) : 0.0;
  if (threadIdx.x == 0) {
    parts_dk[blockIdx.x] = bdk;
    if (parts_err) parts_err[blockIdx.x] = be2;
    if (blockIdx.x == 0) {
      st->s_alpha = s_alpha;
      st->s_rhobar = sp.rhobar;
      st->s_phibar = sp.phibar;
      st->s_psi = sp.psi;
      st->s_phi = sp.phi;
      st->s_rho = sp.rho;
      st->s_theta = sp.theta;
      st->s_tau = sp.tau;
    }
  }
}

// x += dx (end of an outer sweep)
static __global__ void k_add_dx(double *__restrict__ x, const float *__restrict__ dx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += (double)dx[i];
}

}  // namespace plsqr
