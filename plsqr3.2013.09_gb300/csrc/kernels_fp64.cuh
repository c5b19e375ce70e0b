// FP64 kernels of one LSQR iteration on the GB300 (sm_103a).
//
// The operator A = [K; D] is held four ways so that both products are
// gathers (no atomics, deterministic):
//   K by row    (k_rp, k_ci, k_v)   A x, kernel part   (transposed on device)
//   D by row    (d_rp, d_ci, d_v)   A x, damping part
//   K by column (kc_p, kc_ri, kc_v) A^T y, kernel part
//   D by column (dc_p, dc_ri, dc_v) A^T y, damping part
// u = [y_k; y_d] is one array of m = m_k + m_d values.
//
// Kernel rows and columns hold thousands of nonzeros: one warp streams a
// row with 16-byte loads (4 indices, 2x2 values per lane and step) and
// reduces with shuffles.  Damping rows hold at most 3 nonzeros and damping
// columns at most 10: one thread sums them sequentially in stored order, as
// the reference does (CPUSpMV.c:63-72, 267-277).
//
// Reductions (norms, dknorm, error) write one partial per block; the next
// kernel sums the partials in a fixed order, so results do not depend on
// scheduling, and no kernel waits on another block.
#pragma once

#include "lsqr_state.cuh"

namespace plsqr {

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }

// Four consecutive values, 16-byte aligned, in 16-byte loads.
__device__ __forceinline__ void load4(const double *v, int64_t g, double (&o)[4]) {
  const double2 a = __ldg(reinterpret_cast<const double2 *>(v) + 2 * g);
  const double2 b = __ldg(reinterpret_cast<const double2 *>(v) + 2 * g + 1);
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}
__device__ __forceinline__ void load4(const float *v, int64_t g, float (&o)[4]) {
  const float4 a = __ldg(reinterpret_cast<const float4 *>(v) + g);
  o[0] = a.x;
  o[1] = a.y;
  o[2] = a.z;
  o[3] = a.w;
}

// This lane's share of sum val[e] * x[idx[e]] over [beg, end) when one warp
// streams the range: per lane and step one 16-byte load of 4 indices and the
// 4 values (16 or 32 bytes), kUnroll steps in flight.  Reduce across the warp
// with warp_sum.
template <typename T, int kUnroll>
__device__ __forceinline__ T lane_dot(const int32_t *__restrict__ idx, const T *__restrict__ val,
                                      const T *__restrict__ x, int64_t beg, int64_t end,
                                      int lane) {
  T acc0 = 0, acc1 = 0;
  // head: up to 3 elements until beg is a multiple of 4
  int64_t a4 = (beg + 3) & ~int64_t(3);
  if (a4 > end) a4 = end;
  if (beg + lane < a4) acc0 = val[beg + lane] * x[idx[beg + lane]];
  const int64_t e4 = a4 + ((end - a4) & ~int64_t(3));
  const int4 *__restrict__ idx4 = reinterpret_cast<const int4 *>(idx);
  int64_t g = (a4 >> 2) + lane;
  const int64_t gend = e4 >> 2;
  for (; g + 32 * (kUnroll - 1) < gend; g += 32 * kUnroll) {
    int4 c[kUnroll];
    T v[kUnroll][4];
#pragma unroll
    for (int q = 0; q < kUnroll; ++q) {
      c[q] = __ldg(idx4 + g + 32 * q);
      load4(val, g + 32 * q, v[q]);
    }
#pragma unroll
    for (int q = 0; q < kUnroll; ++q) {
      acc0 = fmaT(v[q][0], __ldg(x + c[q].x), acc0);
      acc1 = fmaT(v[q][1], __ldg(x + c[q].y), acc1);
      acc0 = fmaT(v[q][2], __ldg(x + c[q].z), acc0);
      acc1 = fmaT(v[q][3], __ldg(x + c[q].w), acc1);
    }
  }
  for (; g < gend; g += 32) {
    const int4 c0 = __ldg(idx4 + g);
    T v0[4];
    load4(val, g, v0);
    acc0 = fmaT(v0[0], __ldg(x + c0.x), acc0);
    acc1 = fmaT(v0[1], __ldg(x + c0.y), acc1);
    acc0 = fmaT(v0[2], __ldg(x + c0.z), acc0);
    acc1 = fmaT(v0[3], __ldg(x + c0.w), acc1);
  }
  // tail: up to 3 elements
  if (e4 + lane < end) acc1 = fmaT(val[e4 + lane], x[idx[e4 + lane]], acc1);
  return acc0 + acc1;
}

template <int kUnroll>
__device__ __forceinline__ double lane_dot_f64(const int32_t *__restrict__ idx,
                                               const double *__restrict__ val,
                                               const double *__restrict__ x, int64_t beg,
                                               int64_t end, int lane) {
  return lane_dot<double, kUnroll>(idx, val, x, beg, end, lane);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T s) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// Sum of val[e] * x[idx[e]] over [beg, end) by one warp; valid in every lane.
__device__ __forceinline__ double warp_dot_f64(const int32_t *__restrict__ idx,
                                               const double *__restrict__ val,
                                               const double *__restrict__ x, int64_t beg,
                                               int64_t end, int lane) {
  return warp_sum(lane_dot_f64<2>(idx, val, x, beg, end, lane));
}

// Sequential sum in stored order, mul and add rounded separately.
__device__ __forceinline__ double seq_dot_f64(const int32_t *__restrict__ idx,
                                              const double *__restrict__ val,
                                              const double *__restrict__ x, int64_t beg,
                                              int64_t end) {
  double t = 0.0;
  for (int64_t e = beg; e < end; ++e) t = dadd(t, dmul(val[e], x[idx[e]]));
  return t;
}

template <int kThreads>
__device__ __forceinline__ double block_sum(double v, double *smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < kThreads / 32 ? smem[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// Sum of parts[0..n) in a fixed order; valid in thread 0.  Every block that
// calls it on the same data gets the same bits.
template <int kThreads>
__device__ __forceinline__ double sum_parts(const double *parts, int n, double *smem) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) v += parts[i];
  return block_sum<kThreads>(v, smem);
}

// Scale applied to the old vector in the fused products:
enum ScaleMode : int {
  kScaleOne = 0,       // plain aprod: y += A x
  kScaleNegAlpha = 1,  // LSQR mode 1: u = -alpha u + A v
  kScaleNegBeta = 2,   // LSQR mode 2: v = -beta v + A^T u (skipped if beta == 0)
  kScaleZero = 3,      // LSQR start-up: v = 0 + A^T u
};

// Updated vector element y = s*old + t, rounded like the reference's dscal
// followed by the += of the product (FP64), or one FP32 fma.
__device__ __forceinline__ double scaled_add(double s, double old, double t) {
  return dadd(dmul(s, old), t);
}
__device__ __forceinline__ float scaled_add(double s, float old, float t) {
  return fmaf((float)s, old, t);
}

// Damping row r times x, in stored order; FP64: mul and add rounded apart as
// in CPUSpMV.c:67-70, FP32: the FP64 values rounded to FP32.
__device__ __forceinline__ double damp_row(const Csr &D, const double *__restrict__ x, int r) {
  return seq_dot_f64(D.idx, D.val, x, D.ptr[r], D.ptr[r + 1]);
}
__device__ __forceinline__ float damp_row(const Csr &D, const float *__restrict__ x, int r) {
  float t = 0.f;
  for (int64_t e = D.ptr[r]; e < D.ptr[r + 1]; ++e) t = fmaf((float)D.val[e], x[D.idx[e]], t);
  return t;
}

// ---------------------------------------------------------------------------
// M1: u_k[r] = s*u_k[r] + (K v)[r], u_d[r] = s*u_d[r] + (D v)[r], with the
// sums of squares of the new u (in FP64): one partial per warp of the kernel
// blocks, parts[0 .. gk*kThreads/32), then one per damping block.  Warp w of
// the kernel blocks owns rows [kpart[w], kpart[w+1]), a contiguous range
// holding about the same number of nonzeros as every other warp's; writing a
// partial per warp lets a warp that finishes early leave without waiting at
// a block barrier.  T = double: the FP64 solver; T = float: the inner sweeps
// of the mixed solver (values: the FP32 high half).
template <typename T, int kThreads, int kUnroll>
__global__ void __launch_bounds__(kThreads)
    k_aprod1(CsrT<T> K, Csr D, const int32_t *__restrict__ kpart, const T *__restrict__ v,
             T *__restrict__ u, int gk, int mode, const DevState *__restrict__ st,
             double *__restrict__ parts) {
  __shared__ double smem[kThreads / 32];
  double s = 1.0;
  if (mode == kScaleNegAlpha) s = -st->alpha;
  double sq = 0.0;
  if ((int)blockIdx.x < gk) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    const int r1 = kpart[w + 1];
    for (int r = kpart[w]; r < r1; ++r) {
      const T t = warp_sum(lane_dot<T, kUnroll>(K.idx, K.val, v, K.ptr[r], K.ptr[r + 1], lane));
      if (lane == 0) {
        const T y = scaled_add(s, u[r], t);  // dscal, then y_k += t_k
        u[r] = y;
        sq = fma((double)y, (double)y, sq);
      }
    }
    if (lane == 0 && parts) parts[w] = sq;
    return;
  }
  const int gd = gridDim.x - gk;
  T *ud = u + K.n_lines;
  for (int r = (blockIdx.x - gk) * kThreads + threadIdx.x; r < D.n_lines; r += gd * kThreads) {
    const T y = scaled_add(s, ud[r], damp_row(D, v, r));
    ud[r] = y;
    sq = fma((double)y, (double)y, sq);
  }
  const double b = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0 && parts) parts[gk * (kThreads / 32) + (blockIdx.x - gk)] = b;
}

// ---------------------------------------------------------------------------
// N1: beta = sqrt(sum_k + sum_d); u *= 1/beta.  LSQR start-up (start = 1)
// also takes this path with beta = ||b||.
__device__ __forceinline__ double scale_elem(double x, double r) { return dmul(x, r); }
__device__ __forceinline__ float scale_elem(float x, double r) { return x * (float)r; }

// mirror (optional): FP32 copy of the scaled u, gathered by FP32 products;
// mirror_lo (optional): the rest, u - mirror rounded to FP32.
template <typename T, int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_norm_u(T *__restrict__ u, int64_t m, const double *__restrict__ parts, int gk, int gd,
             DevState *__restrict__ st, int start, float *__restrict__ mirror = nullptr,
             float *__restrict__ mirror_lo = nullptr) {
  __shared__ double smem[kThreads / 32];
  __shared__ double s_rb;
  const double sk = sum_parts<kThreads>(parts, gk, smem);
  const double sd = sum_parts<kThreads>(parts + gk, gd, smem);
  if (threadIdx.x == 0) {
    const double beta = __dsqrt_rn(dadd(sk, sd));
    s_rb = beta > 0.0 ? ddiv(1.0, beta) : 0.0;
    if (blockIdx.x == 0) {
      st->beta = beta;
      st->s_beta_pos = beta > 0.0;
      if (!start) {  // source/lsqr.c:526-528
        double temp = d2norm(st->alpha, beta);
        temp = d2norm(temp, st->damp);
        st->anorm = d2norm(st->anorm, temp);
      }
    }
  }
  __syncthreads();
  const double rb = s_rb;
  if (rb == 0.0) return;  // beta == 0: u is left as is
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * kThreads) {
    const T y = scale_elem(u[i], rb);
    u[i] = y;
    if (mirror) {
      const float h = (float)y;
      mirror[i] = h;
      if (mirror_lo) mirror_lo[i] = (float)((double)y - (double)h);
    }
  }
}

// ---------------------------------------------------------------------------
// M2: v[c] = s*v[c] + (K^T u_k + D^T u_d)[c]; per-block partial sum of
// squares of the new v.  The columns are visited in the order corder (the
// natural order, or 3-D Morton order of the cells); block b owns the visit
// positions [cpart[b], cpart[b+1]) (balanced by nonzeros) and its warps take
// them in turn, so that neighbouring cells, which share most of their rays,
// are gathered at the same time on the same SM and reuse u_k from L1.  A column's kernel entries
// are streamed by the whole warp and its damping entries (a few per column)
// are spread over the lanes, so every FP64 instruction runs on a full warp.
// In LSQR mode the kernel is skipped when beta == 0 (source/lsqr.c:530).
template <typename T, int kThreads, int kUnroll>
__global__ void __launch_bounds__(kThreads)
    k_aprod2(CsrT<T> KC, Csr DC, const int32_t *__restrict__ cpart,
             const int32_t *__restrict__ corder, const T *__restrict__ u, int m_k,
             T *__restrict__ v, int mode, const DevState *__restrict__ st,
             double *__restrict__ parts) {
  __shared__ double smem[kThreads / 32];
  double s = 1.0;
  if (mode == kScaleNegBeta) {
    if (!st->s_beta_pos) return;
    s = -st->beta;
  } else if (mode == kScaleZero) {
    if (!st->s_beta_pos) return;
    s = 0.0;
  }
  const T *ud = u + m_k;
  const int lane = threadIdx.x & 31;
  const int c1 = cpart[blockIdx.x + 1];
  double sq = 0.0;
  for (int k = cpart[blockIdx.x] + (threadIdx.x >> 5); k < c1; k += kThreads / 32) {
    const int c = corder[k];
    T acc = lane_dot<T, kUnroll>(KC.idx, KC.val, u, KC.ptr[c], KC.ptr[c + 1], lane);
    for (int64_t e = DC.ptr[c] + lane; e < DC.ptr[c + 1]; e += 32)
      acc = fmaT((T)DC.val[e], ud[DC.idx[e]], acc);
    const T t = warp_sum(acc);
    if (lane == 0) {
      const T y = scaled_add(s, v[c], t);  // x += (s_k + s_d)
      v[c] = y;
      sq = fma((double)y, (double)y, sq);
    }
  }
  const double b = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0 && parts) parts[blockIdx.x] = b;
}

// ---------------------------------------------------------------------------
// N2: alpha = ||v||, v *= 1/alpha, then the rotation and the x/w update
// (source/lsqr.c:577-692).  Writes per-block partials of dknorm^2 to
// parts_dk and of ||x - x_ref||^2 to parts_err.  start = 1: the LSQR start-up
// (source/lsqr.c:375-445): w = v, x = 0, no rotation.
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_update_x(double *__restrict__ v, double *__restrict__ w, double *__restrict__ x,
               double *__restrict__ se, const double *__restrict__ xref, int n,
               const double *__restrict__ parts, int gp, DevState *__restrict__ st,
               double *__restrict__ parts_dk, double *__restrict__ parts_err,
               plsqr_iter *__restrict__ hist, int start, float *__restrict__ v_mirror = nullptr,
               const double *__restrict__ x_base = nullptr, float *__restrict__ v_mirror_lo = nullptr) {
  __shared__ double smem[kThreads / 32];
  __shared__ double s_alpha, s_ra;
  __shared__ Step s_step;
  const int beta_pos = st->s_beta_pos;
  const double vv = beta_pos ? sum_parts<kThreads>(parts, gp, smem) : 0.0;
  if (threadIdx.x == 0) {
    double alpha = st->alpha;  // unchanged when beta == 0
    if (beta_pos) alpha = __dsqrt_rn(vv);
    if (start && !beta_pos) alpha = 0.0;
    s_alpha = alpha;
    s_ra = (beta_pos && alpha > 0.0) ? ddiv(1.0, alpha) : 0.0;
    if (!start) s_step = lsqr_step(*st, alpha, st->beta);
  }
  __syncthreads();
  const double ra = s_ra;
  if (start) {
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
      double vi = v[i];
      if (ra != 0.0) vi = dmul(vi, ra);
      v[i] = vi;
      if (v_mirror) {
        const float h = (float)vi;
        v_mirror[i] = h;
        if (v_mirror_lo) v_mirror_lo[i] = (float)(vi - (double)h);
      }
      w[i] = ra != 0.0 ? vi : 0.0;  // w = v only when alpha > 0 (lsqr.c:392-395)
      x[i] = 0.0;
      if (se) se[i] = 0.0;
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
      if (hist) {
        plsqr_iter &h = hist[0];
        h.alpha = alpha;
        h.beta = beta;
        h.rnorm = beta;
        h.arnorm = st->arnorm;
        h.test1 = 1.0;
        h.test2 = beta > 0.0 ? ddiv(alpha, beta) : 0.0;
        h.anorm = 0.0;
        h.acond = 0.0;
        h.xnorm = 0.0;
        h.x0 = 0.0;
        h.err = st->has_ref ? 1.0 : -1.0;
        h.istop = 0;
        h.pad = 0;
      }
    }
    return;
  }
  const Step sp = s_step;
  double dk = 0.0, e2 = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double vi = v[i];
    if (ra != 0.0) {
      vi = dmul(vi, ra);
      v[i] = vi;
    }
    if (v_mirror) {
      const float h = (float)vi;
      v_mirror[i] = h;
      if (v_mirror_lo) v_mirror_lo[i] = (float)(vi - (double)h);
    }
    const double t = w[i];
    const double xi = dadd(dmul(sp.t1, t), x[i]);
    x[i] = xi;
    w[i] = dadd(dmul(sp.t2, t), vi);
    const double tt = dmul(dmul(sp.t3, t), dmul(sp.t3, t));
    if (se) se[i] = dadd(tt, se[i]);
    dk += tt;
    if (xref) {
      const double d = (x_base ? x_base[i] + xi : xi) - xref[i];
      e2 = fma(d, d, e2);
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

// ---------------------------------------------------------------------------
// T: the rest of the iteration's scalars and the history record (one block).
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_tail(DevState *__restrict__ st, const double *__restrict__ parts_dk,
           const double *__restrict__ parts_err, int gp, const double *__restrict__ x,
           plsqr_iter *__restrict__ hist) {
  __shared__ double smem[kThreads / 32];
  const double dk = sum_parts<kThreads>(parts_dk, gp, smem);
  const double e2 = parts_err ? sum_parts<kThreads>(parts_err, gp, smem) : 0.0;
  if (threadIdx.x == 0) lsqr_tail(*st, dk, e2, x[0], hist);
}

// ---------------------------------------------------------------------------
// Sum of squares of u = [y_k; y_d] (kernel part in blocks [0, gk), damping
// part in [gk, grid)), for the start-up beta = ||b||.
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_sumsq_u(const double *__restrict__ u, int m_k, int64_t m_d, int gk,
              double *__restrict__ parts) {
  __shared__ double smem[kThreads / 32];
  double sq = 0.0;
  if ((int)blockIdx.x < gk) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < m_k;
         i += (int64_t)gk * kThreads)
      sq = fma(u[i], u[i], sq);
  } else {
    const int gd = gridDim.x - gk;
    for (int64_t i = (blockIdx.x - gk) * (int64_t)kThreads + threadIdx.x; i < m_d;
         i += (int64_t)gd * kThreads)
      sq = fma(u[m_k + i], u[m_k + i], sq);
  }
  const double b = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0) parts[blockIdx.x] = b;
}

// ||x_ref||^2 into st->ref_norm2 (one block).
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_ref_norm(const double *__restrict__ xref, int n, DevState *__restrict__ st) {
  __shared__ double smem[kThreads / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) s = fma(xref[i], xref[i], s);
  const double b = block_sum<kThreads>(s, smem);
  if (threadIdx.x == 0) st->ref_norm2 = b;
}

// se[i] = t * sqrt(se[i]) (source/lsqr.c:878-891)
static __global__ void k_finish_se(double *__restrict__ se, int n, const DevState *__restrict__ st,
                            int num_row) {
  const double rnorm = st->rnorm;
  double t = 1.0;
  if (num_row > n) t = (double)(num_row - n);
  if (st->damp > 0.0) t = (double)num_row;
  t = ddiv(rnorm, __dsqrt_rn(t));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    se[i] = dmul(t, __dsqrt_rn(se[i]));
}

}  // namespace plsqr
