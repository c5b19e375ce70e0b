// Kernels of the batched solver: k right-hand sides (k <= 32) advanced in
// lock step, one LSQR per right-hand side, sharing every read of the matrix.
//
// Right-hand side j solves min || [K; lambda_j D] x_j - [b_j; 0] ||.  Vectors
// are blocks with the right-hand sides contiguous, padded to kp = 4, 8, 16 or
// 32 columns: U[r*kp + j] (m = m_k + m_d rows), V, W, X, DX [c*kp + j], all
// FP64, plus the FP32 mirrors Uf (kernel rows only) and Vf that the kernel
// products gather.  Padding columns hold zeros and never become active.
//
// Kernel products ("team" form).  A team of kLPR lanes owns one line (a
// kernel row for A x, a kernel column for A^T y).  Inside the team, R = kp/kVW
// lanes cover one row of the gathered block with kVW-wide loads (float4 or
// float2), so one gather reads the 4*kp contiguous bytes of that row; the
// team's S = kLPR/R subgroups take the line's nonzeros in turn, kU at a time.
// Each lane sums its FP32 products in short runs joined by an error-free
// two-sum; the subgroups' sums are added in FP64 with shuffles and combined
// into the FP64 block.  Values are the FP32 high half of the value split;
// damping terms, norms and the LSQR recurrences are FP64.
//
// Reductions.  Every product or update kernel writes one partial per
// (block, right-hand side) and the block that finishes last (arrival counter)
// adds the partials in block order and advances the scalar state: the result
// does not depend on which block is last.  No block waits for another.
#pragma once

#include <climits>

#include "kernels_fp64.cuh"

namespace plsqr {

constexpr int kBatchMax = 32;
constexpr int kBatchThreads = 256;
// resident blocks per SM of the team products (their launch bounds): five
// measured faster than four (more gathers in flight) despite a few spilled
// registers
constexpr int kTeamBlocksPerSm = 5;

// Per-right-hand-side coefficients handed from one kernel to the next.
struct BatchCoef {
  double rb[kBatchMax];  // 1/beta_j (0: u_j is left as is)
  double ra[kBatchMax];  // 1/alpha_j (0: v_j is left as is)
  double t1[kBatchMax], t2[kBatchMax], t3[kBatchMax];  // x/w update of source/lsqr.c:685-690
  double sc[kBatchMax];  // scale of the running block in the next product
  int32_t act[kBatchMax];  // 1: the next product updates right-hand side j
  unsigned int count;      // arrival counter of the last-block reductions
  unsigned int pad;
};

// True in the block that arrives last; its partial sums and every other
// block's are then visible.  Callers that wrote partials have fenced them.
__device__ __forceinline__ bool batch_last_block(unsigned int *count) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(count, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// Sum of column j of parts[n][kp], in row order, read past L1.
__device__ __forceinline__ double batch_col_sum(const double *parts, int n, int kp, int j) {
  double s = 0.0;
  for (int q = 0; q < n; ++q) s += __ldcg(parts + (int64_t)q * kp + j);
  return s;
}

// Block reduction of one value per thread, where thread t holds right-hand
// side t % kp; threads j < kp return the sums (fixed order), others 0.
__device__ __forceinline__ double batch_block_sum(double v, int kp, double *red) {
  red[threadIdx.x] = v;
  __syncthreads();
  double s = 0.0;
  if ((int)threadIdx.x < kp)
    for (int t = threadIdx.x; t < (int)blockDim.x; t += kp) s += red[t];
  __syncthreads();
  return s;
}

template <int kVW>
struct VecF;
template <>
struct VecF<4> {
  __device__ static __forceinline__ void load(const float *p, float *o) {
    const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = q.x, o[1] = q.y, o[2] = q.z, o[3] = q.w;
  }
};
template <>
struct VecF<2> {
  __device__ static __forceinline__ void load(const float *p, float *o) {
    const float2 q = __ldg(reinterpret_cast<const float2 *>(p));
    o[0] = q.x, o[1] = q.y;
  }
};

// hi + lo += x with an error-free transformation of the FP32 add (Knuth's
// two-sum): hi keeps the rounded sum and lo collects every add's rounding
// error, so a long run of partial sums keeps FP32 rounding per partial and
// costs no FP64 instruction (the GB300's FP64 pipe is 1/64 of its FP32 rate).
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += err;
}

// One team's dot products of line l with every column of the gathered block
// xf[*, kp]: on return the lanes of subgroup 0 (tl < R) hold the sums for
// right-hand sides tl*kVW .. tl*kVW + kVW - 1.  `mask` names the team's lanes.
// The FP32 products are summed in runs of at most kRun steps per lane whose
// sums are added with two_sum_add: a line of thousands of nonzeros stays at
// FP32 rounding per run instead of a rounding error that grows with its
// length.
template <int kVW, int kLPR, int kU>
__device__ __forceinline__ void team_dot(const int32_t *__restrict__ idx,
                                         const float *__restrict__ val,
                                         const float *__restrict__ xf, int kp, int64_t beg,
                                         int64_t end, int tl, unsigned mask, double *out) {
  constexpr int kRun = 16;
  const int R = kp / kVW, S = kLPR / R;
  const int sub = tl / R, q = tl - sub * R;
  const float *xq = xf + q * kVW;
  float hi[kVW], lo[kVW];
#pragma unroll
  for (int v = 0; v < kVW; ++v) hi[v] = lo[v] = 0.f;
  int64_t e = beg + sub;
  while (e < end) {
    float acc[kVW];
#pragma unroll
    for (int v = 0; v < kVW; ++v) acc[v] = 0.f;
    int steps = 0;
    // kU entries per step: their indices and values first, then kU gathers in
    // flight at once, then the multiply-adds
    for (; steps < kRun && e + (kU - 1) * S < end; ++steps, e += kU * S) {
      int32_t c[kU];
      float a[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        c[u] = __ldg(idx + e + u * S);
        a[u] = __ldg(val + e + u * S);
      }
      float g[kU][kVW];
#pragma unroll
      for (int u = 0; u < kU; ++u) VecF<kVW>::load(xq + (int64_t)c[u] * kp, g[u]);
#pragma unroll
      for (int u = 0; u < kU; ++u)
#pragma unroll
        for (int v = 0; v < kVW; ++v) acc[v] = fmaf(a[u], g[u][v], acc[v]);
    }
    if (steps < kRun) {  // the line's last few entries, one at a time
      for (; e < end; e += S) {
        float g[kVW];
        VecF<kVW>::load(xq + (int64_t)__ldg(idx + e) * kp, g);
        const float a = __ldg(val + e);
#pragma unroll
        for (int v = 0; v < kVW; ++v) acc[v] = fmaf(a, g[v], acc[v]);
      }
    }
#pragma unroll
    for (int v = 0; v < kVW; ++v) two_sum_add(hi[v], lo[v], acc[v]);
  }
#pragma unroll
  for (int v = 0; v < kVW; ++v) {
    double r = (double)hi[v] + (double)lo[v];
    for (int off = R; off < kLPR; off <<= 1) r += __shfl_xor_sync(mask, r, off);
    out[v] = r;
  }
}

// Lane mask of the team of kLPR lanes that holds `lane`.
template <int kLPR>
__device__ __forceinline__ unsigned team_mask(int lane) {
  return kLPR == 32 ? 0xffffffffu : (((1u << kLPR) - 1u) << (lane / kLPR * kLPR));
}

// Per-block sums of squares kept by teams: sqs[team][j], teams of the block in
// order, then threads j < kp add them up (fixed order).
template <int kLPR>
__device__ __forceinline__ double team_block_sum(double (*sqs)[kBatchMax], int kp) {
  __syncthreads();
  double s = 0.0;
  if ((int)threadIdx.x < kp)
    for (int t = 0; t < kBatchThreads / kLPR; ++t) s += sqs[t][threadIdx.x];
  return s;
}

// The end of a batched A x (last block): beta_j, 1/beta_j, anorm in LSQR mode
// (source/lsqr.c:526-528).
__device__ __forceinline__ void rows_finish(const double *parts, int n_parts, int kw, int k,
                                            int mode, DevState *st, BatchCoef *cf) {
  if ((int)threadIdx.x < k) {
    const int j = threadIdx.x;
    DevState &S = st[j];
    const double beta = __dsqrt_rn(batch_col_sum(parts, n_parts, kw, j));
    S.beta = beta;
    S.s_beta_pos = beta > 0.0;
    cf->rb[j] = beta > 0.0 ? ddiv(1.0, beta) : 0.0;
    if (mode == kScaleNegAlpha) {
      double temp = d2norm(S.alpha, beta);
      temp = d2norm(temp, S.damp);
      S.anorm = d2norm(S.anorm, temp);
    }
  } else if ((int)threadIdx.x < kBatchMax) {
    cf->rb[threadIdx.x] = 0.0;
  }
  if (threadIdx.x == 0) cf->count = 0;
}

// Batched A x:  U_k = s_j U_k + K v_j,  U_d = s_j U_d + lambda_j D v_j
// (s_j = -alpha_j in an LSQR iteration, 1 for the plain product).  Blocks
// [0, gk) run the kernel rows in teams, warp w owning rows [wpart[w],
// wpart[w+1]) (balanced by nonzeros); blocks [gk, grid) run the damping rows,
// 32/kp rows per warp with one lane per right-hand side, in FP64.  The last
// block forms beta_j = ||u_j|| and, in LSQR mode, anorm (source/lsqr.c:526-528).
template <int kVW, int kLPR, int kU>
__global__ void __launch_bounds__(kBatchThreads, kTeamBlocksPerSm)
    k_bprod_rows(CsrT<float> K, Csr D, const int32_t *__restrict__ wpart, int gk, int kp, int k,
                 const float *__restrict__ vf, const double *__restrict__ v64,
                 double *__restrict__ u, const double *__restrict__ lambda, int mode,
                 DevState *__restrict__ st, BatchCoef *__restrict__ cf,
                 double *__restrict__ parts) {
  __shared__ double sqs[kBatchThreads / kLPR][kBatchMax];
  __shared__ double red[kBatchThreads];
  __shared__ double s_sc[kBatchMax], s_lam[kBatchMax];
  if (threadIdx.x < kBatchMax) {
    const int j = threadIdx.x;
    s_sc[j] = (j < k && mode == kScaleNegAlpha) ? -st[j].alpha : 1.0;
    s_lam[j] = (j < k && lambda) ? lambda[j] : 1.0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double bsum;
  if ((int)blockIdx.x < gk) {
    constexpr int kTeams = 32 / kLPR;
    const int R = kp / kVW;
    const int team = lane / kLPR, tl = lane % kLPR, q = tl % R;
    const unsigned mask = team_mask<kLPR>(lane);
    const int w = blockIdx.x * (kBatchThreads / 32) + wib;
    const int r1 = wpart[w + 1];
    double sq[kVW];
#pragma unroll
    for (int v = 0; v < kVW; ++v) sq[v] = 0.0;
    for (int r = wpart[w] + team; r < r1; r += kTeams) {
      double t[kVW];
      team_dot<kVW, kLPR, kU>(K.idx, K.val, vf, kp, K.ptr[r], K.ptr[r + 1], tl, mask, t);
      if (tl < R) {
#pragma unroll
        for (int v = 0; v < kVW; ++v) {
          const int j = q * kVW + v;
          if (j < k) {
            double *p = u + (int64_t)r * kp + j;
            const double y = dadd(dmul(s_sc[j], *p), t[v]);
            *p = y;
            sq[v] = fma(y, y, sq[v]);
          }
        }
      }
    }
    const int ti = wib * kTeams + team;
    if (tl < R) {
#pragma unroll
      for (int v = 0; v < kVW; ++v) sqs[ti][q * kVW + v] = sq[v];
    }
    bsum = team_block_sum<kLPR>(sqs, kp);
  } else {
    const int spw = 32 / kp;  // damping rows per warp
    const int slot = lane / kp, j = lane % kp;
    const int gd = gridDim.x - gk;
    const double *__restrict__ v64j = v64 + j;
    double *ud = u + (int64_t)K.n_lines * kp;
    double sq = 0.0;
    for (int r = ((blockIdx.x - gk) * (kBatchThreads / 32) + wib) * spw + slot; r < D.n_lines;
         r += gd * (kBatchThreads / 32) * spw) {
      double t = 0.0;
      for (int64_t e = D.ptr[r]; e < D.ptr[r + 1]; ++e)
        t = fma(D.val[e], v64j[(int64_t)D.idx[e] * kp], t);
      if (j < k) {
        double *p = ud + (int64_t)r * kp + j;
        const double y = dadd(dmul(s_sc[j], *p), dmul(s_lam[j], t));
        *p = y;
        sq = fma(y, y, sq);
      }
    }
    bsum = batch_block_sum(sq, kp, red);
  }
  if ((int)threadIdx.x < kp) parts[(int64_t)blockIdx.x * kp + threadIdx.x] = bsum;
  if (!batch_last_block(&cf->count)) return;
  rows_finish(parts, gridDim.x, kp, k, mode, st, cf);
}


// The end of a batched A^T y (last block): alpha_j and the rotation of the
// iteration (source/lsqr.c:551-636), or the start-up values
// (source/lsqr.c:387-409) when mode is kScaleZero.
__device__ __forceinline__ void cols_finish(const double *parts, int n_parts, int kp, int k,
                                            int mode, DevState *st, BatchCoef *cf) {
  if ((int)threadIdx.x < kBatchMax) {
    const int j = threadIdx.x;
    double ra = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
    if (j < k && mode == kScaleZero) {
      DevState &S = st[j];
      const int bp = S.s_beta_pos;
      const double alpha = bp ? __dsqrt_rn(batch_col_sum(parts, n_parts, kp, j)) : 0.0;
      ra = (bp && alpha > 0.0) ? ddiv(1.0, alpha) : 0.0;
      S.alpha = alpha;
      S.arnorm = dmul(alpha, S.beta);
      S.rhobar = alpha;
      S.phibar = S.beta;
      S.bnorm = S.beta;
      S.rnorm = S.beta;
      S.done = S.arnorm == 0.0;
    } else if (j < k && mode == kScaleNegBeta && !st[j].done) {
      DevState &S = st[j];
      const int bp = S.s_beta_pos;
      const double alpha = bp ? __dsqrt_rn(batch_col_sum(parts, n_parts, kp, j)) : S.alpha;
      ra = (bp && alpha > 0.0) ? ddiv(1.0, alpha) : 0.0;
      const Step sp = lsqr_step(S, alpha, S.beta);
      S.s_alpha = alpha;
      S.s_rhobar = sp.rhobar;
      S.s_phibar = sp.phibar;
      S.s_psi = sp.psi;
      S.s_phi = sp.phi;
      S.s_rho = sp.rho;
      S.s_theta = sp.theta;
      S.s_tau = sp.tau;
      t1 = sp.t1;
      t2 = sp.t2;
      t3 = sp.t3;
    }
    cf->ra[j] = ra;
    cf->t1[j] = t1;
    cf->t2[j] = t2;
    cf->t3[j] = t3;
  }
  if (threadIdx.x == 0) cf->count = 0;
}

// Batched A^T y:  V_j = s_j V_j + K^T u_j + lambda_j D^T u_j  with s_j =
// -beta_j in an LSQR iteration (right-hand sides with beta_j = 0 keep v_j,
// source/lsqr.c:530), 0 at the start of a solve, 1 for the plain product.
// Warp w owns columns [wpart[w], wpart[w+1]) and its teams take them in turn;
// a column's damping entries (a few) are added in FP64 by the lanes that hold
// its sums.  The last block forms alpha_j and the rotation of the iteration
// (source/lsqr.c:551-636), or the start-up values (source/lsqr.c:387-409).
template <int kVW, int kLPR, int kU>
__global__ void __launch_bounds__(kBatchThreads, kTeamBlocksPerSm)
    k_bprod_cols(CsrT<float> KC, Csr DC, const int32_t *__restrict__ wpart, int kp, int k,
                 const float *__restrict__ uf, const double *__restrict__ u64, int m_k,
                 double *__restrict__ v, const double *__restrict__ lambda, int mode,
                 DevState *__restrict__ st, BatchCoef *__restrict__ cf,
                 double *__restrict__ parts) {
  __shared__ double sqs[kBatchThreads / kLPR][kBatchMax];
  __shared__ double s_sc[kBatchMax], s_lam[kBatchMax];
  __shared__ int s_act[kBatchMax];
  if (threadIdx.x < kBatchMax) {
    const int j = threadIdx.x;
    double s = 1.0;
    int act = j < k;
    if (act && (mode == kScaleNegBeta || mode == kScaleZero)) {
      act = st[j].s_beta_pos && !(mode == kScaleNegBeta && st[j].done);
      s = mode == kScaleZero ? 0.0 : -st[j].beta;
    }
    s_sc[j] = s;
    s_act[j] = act;
    s_lam[j] = (j < k && lambda) ? lambda[j] : 1.0;
  }
  __syncthreads();
  constexpr int kTeams = 32 / kLPR;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int R = kp / kVW;
  const int team = lane / kLPR, tl = lane % kLPR, q = tl % R;
  const unsigned mask = team_mask<kLPR>(lane);
  const int w = blockIdx.x * (kBatchThreads / 32) + wib;
  const int c1 = wpart[w + 1];
  const double *ud = u64 + (int64_t)m_k * kp + q * kVW;
  double sq[kVW];
#pragma unroll
  for (int t = 0; t < kVW; ++t) sq[t] = 0.0;
  for (int c = wpart[w] + team; c < c1; c += kTeams) {
    double t[kVW];
    team_dot<kVW, kLPR, kU>(KC.idx, KC.val, uf, kp, KC.ptr[c], KC.ptr[c + 1], tl, mask, t);
    if (tl < R) {
      double d[kVW];
#pragma unroll
      for (int x = 0; x < kVW; ++x) d[x] = 0.0;
      for (int64_t e = DC.ptr[c]; e < DC.ptr[c + 1]; ++e) {
        const double a = DC.val[e];
        const double *g = ud + (int64_t)DC.idx[e] * kp;
#pragma unroll
        for (int x = 0; x < kVW; ++x) d[x] = fma(a, g[x], d[x]);
      }
#pragma unroll
      for (int x = 0; x < kVW; ++x) {
        const int j = q * kVW + x;
        if (s_act[j]) {
          double *p = v + (int64_t)c * kp + j;
          const double y = dadd(dmul(s_sc[j], *p), dadd(t[x], dmul(s_lam[j], d[x])));
          *p = y;
          sq[x] = fma(y, y, sq[x]);
        }
      }
    }
  }
  if (tl < R) {
#pragma unroll
    for (int x = 0; x < kVW; ++x) sqs[wib * kTeams + team][q * kVW + x] = sq[x];
  }
  const double bsum = team_block_sum<kLPR>(sqs, kp);
  if ((int)threadIdx.x < kp) parts[(int64_t)blockIdx.x * kp + threadIdx.x] = bsum;
  if (!batch_last_block(&cf->count)) return;
  cols_finish(parts, gridDim.x, kp, k, mode, st, cf);
}

// u *= 1/beta_j per right-hand side (u_j left as is where beta_j = 0), and
// the FP32 mirror of the kernel rows.
static __global__ void __launch_bounds__(kBatchThreads)
    k_bscale_u(double *__restrict__ u, float *__restrict__ uf, int64_t m_k, int64_t m, int kp,
               const BatchCoef *__restrict__ cf) {
  __shared__ double rb[kBatchMax];
  if (threadIdx.x < kBatchMax) rb[threadIdx.x] = cf->rb[threadIdx.x];
  __syncthreads();
  const int64_t total = m * kp, tk = m_k * kp;
  for (int64_t i = blockIdx.x * (int64_t)kBatchThreads + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * kBatchThreads) {
    const double r = rb[i & (kp - 1)];
    double y = u[i];
    if (r != 0.0) {
      y = dmul(y, r);
      u[i] = y;
    }
    if (i < tk) uf[i] = (float)y;
  }
}


// History record of a right-hand side that has stopped (A^T r = 0 at the
// start of its solve): the state as it is, one more iteration counted.
__device__ __forceinline__ void batch_hist_idle(DevState &S, double err2, plsqr_iter *hist) {
  const int itn = S.itn + 1;
  S.err = S.has_ref ? __dsqrt_rn(ddiv(err2, S.ref_norm2)) : -1.0;
  if (hist) {
    plsqr_iter &h = hist[S.hist_base + itn];
    h.alpha = S.alpha;
    h.beta = S.beta;
    h.rnorm = S.rnorm;
    h.arnorm = S.arnorm;
    h.test1 = S.test1;
    h.test2 = S.test2;
    h.anorm = S.anorm;
    h.acond = S.acond;
    h.xnorm = S.xnorm;
    h.x0 = 0.0;
    h.err = S.err;
    h.istop = S.istop;
    h.pad = 0;
  }
  S.itn = itn;
}

// Batched N2: v_j *= 1/alpha_j (and its FP32 mirror), then the update
// dx_j += t1_j w_j, w_j = t2_j w_j + v_j with dknorm partials
// (source/lsqr.c:685-690); with a reference block, the squared error of
// x_base + dx.  start = 1: w = v (where alpha_j > 0), dx = 0.  The last block
// finishes each right-hand side's iteration (source/lsqr.c:703-775) and
// writes its history record at hist[slot_j*hist_stride + hist_base + itn].
static __global__ void __launch_bounds__(kBatchThreads)
    k_bupdate(double *__restrict__ v, float *__restrict__ vf, double *__restrict__ w,
              double *__restrict__ dx, const double *__restrict__ x_base,
              const double *__restrict__ xref, int n, int kp, int k,
              BatchCoef *__restrict__ cf, DevState *__restrict__ st,
              double *__restrict__ parts_dk, double *__restrict__ parts_err, int start,
              plsqr_iter *__restrict__ hist, int hist_stride) {
  __shared__ double red[kBatchThreads];
  // each thread keeps one right-hand side: the block and the grid stride are
  // multiples of kp
  const int j = threadIdx.x & (kp - 1);
  const double ra = cf->ra[j], t1 = cf->t1[j], t2 = cf->t2[j], t3 = cf->t3[j];
  const int64_t total = (int64_t)n * kp;
  double dk = 0.0, e2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kBatchThreads + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * kBatchThreads) {
    double vi = v[i];
    if (ra != 0.0) {
      vi = dmul(vi, ra);
      v[i] = vi;
    }
    vf[i] = (float)vi;
    if (start) {
      w[i] = ra != 0.0 ? vi : 0.0;
      dx[i] = 0.0;
      continue;
    }
    const double t = w[i];
    const double xi = dadd(dmul(t1, t), dx[i]);
    dx[i] = xi;
    w[i] = dadd(dmul(t2, t), vi);
    dk += dmul(dmul(t3, t), dmul(t3, t));
    if (xref) {
      const double d = (x_base[i] + xi) - xref[i];
      e2 = fma(d, d, e2);
    }
  }
  if (start) return;
  const double bdk = batch_block_sum(dk, kp, red);
  const double be2 = batch_block_sum(e2, kp, red);
  if ((int)threadIdx.x < kp) {
    parts_dk[(int64_t)blockIdx.x * kp + threadIdx.x] = bdk;
    parts_err[(int64_t)blockIdx.x * kp + threadIdx.x] = be2;
  }
  if (!batch_last_block(&cf->count)) return;
  if ((int)threadIdx.x < k) {
    const int jj = threadIdx.x;
    DevState &S = st[jj];
    const double d2 = batch_col_sum(parts_dk, gridDim.x, kp, jj);
    const double er = xref ? batch_col_sum(parts_err, gridDim.x, kp, jj) : 0.0;
    plsqr_iter *h = hist ? hist + (int64_t)S.slot * hist_stride : nullptr;
    if (S.done)
      batch_hist_idle(S, er, h);
    else
      lsqr_tail(S, d2, er, x_base[jj], h);
  }
  if (threadIdx.x == 0) cf->count = 0;
}

// ||xref_j||^2 into st[j].ref_norm2.
static __global__ void __launch_bounds__(kBatchThreads)
    k_bref_norm(const double *__restrict__ xref, int n, int kp, int k, DevState *__restrict__ st,
                BatchCoef *__restrict__ cf, double *__restrict__ parts) {
  __shared__ double red[kBatchThreads];
  const int64_t total = (int64_t)n * kp;
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kBatchThreads + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * kBatchThreads)
    s = fma(xref[i], xref[i], s);
  const double b = batch_block_sum(s, kp, red);
  if ((int)threadIdx.x < kp) parts[(int64_t)blockIdx.x * kp + threadIdx.x] = b;
  if (!batch_last_block(&cf->count)) return;
  if ((int)threadIdx.x < k) st[threadIdx.x].ref_norm2 = batch_col_sum(parts, gridDim.x, kp, threadIdx.x);
  if (threadIdx.x == 0) cf->count = 0;
}

// Outer residual of a refinement sweep, in FP64 with the FP64 kernel values:
// U_k = B - K X_j, U_d = -lambda_j D X_j; 32/kp rows per warp, one lane per
// right-hand side, rows handed out in warp order (kernel rows, then damping
// rows).  The last block forms beta_j = ||r_j|| (start-up of the correction
// solve, source/lsqr.c:362-386).
static __global__ void __launch_bounds__(kBatchThreads)
    k_bresidual(Csr K, Csr D, int kp, int k, const double *__restrict__ x,
                const double *__restrict__ b, double *__restrict__ u,
                const double *__restrict__ lambda, DevState *__restrict__ st,
                BatchCoef *__restrict__ cf, double *__restrict__ parts) {
  __shared__ double red[kBatchThreads];
  const int lane = threadIdx.x & 31;
  const int spw = 32 / kp, slot = lane / kp, j = lane % kp;
  const double lam = (j < k && lambda) ? lambda[j] : 1.0;
  const int64_t m = (int64_t)K.n_lines + D.n_lines;
  const int64_t nw = (int64_t)gridDim.x * (kBatchThreads / 32) * spw;
  double sq = 0.0;
  for (int64_t r = ((int64_t)blockIdx.x * (kBatchThreads / 32) + (threadIdx.x >> 5)) * spw + slot;
       r < m; r += nw) {
    double t = 0.0, y;
    if (r < K.n_lines) {
      for (int64_t e = K.ptr[r]; e < K.ptr[r + 1]; ++e)
        t = fma(K.val[e], x[(int64_t)K.idx[e] * kp + j], t);
      y = b[r * kp + j] - t;
    } else {
      const int64_t rd = r - K.n_lines;
      for (int64_t e = D.ptr[rd]; e < D.ptr[rd + 1]; ++e)
        t = fma(D.val[e], x[(int64_t)D.idx[e] * kp + j], t);
      y = -(lam * t);
    }
    if (j >= k) y = 0.0;
    u[r * kp + j] = y;
    sq = fma(y, y, sq);
  }
  const double bs = batch_block_sum(sq, kp, red);
  if ((int)threadIdx.x < kp) parts[(int64_t)blockIdx.x * kp + threadIdx.x] = bs;
  if (!batch_last_block(&cf->count)) return;
  if ((int)threadIdx.x < kBatchMax) {
    const int jj = threadIdx.x;
    double rb = 0.0;
    if (jj < k) {
      const double beta = __dsqrt_rn(batch_col_sum(parts, gridDim.x, kp, jj));
      st[jj].beta = beta;
      st[jj].s_beta_pos = beta > 0.0;
      rb = beta > 0.0 ? ddiv(1.0, beta) : 0.0;
    }
    cf->rb[jj] = rb;
  }
  if (threadIdx.x == 0) cf->count = 0;
}

// dst[i*kp + j] = src[j*ld + i] for j < k, 0 for the padding columns
// (right-hand-side-major host layout to the interleaved device block) and back.
static __global__ void k_bgather(const double *__restrict__ src, int64_t ld, int64_t rows, int kp, int k,
                          double *__restrict__ dst) {
  const int64_t total = rows * kp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / kp;
    const int j = (int)(i - r * kp);
    dst[i] = j < k ? src[(int64_t)j * ld + r] : 0.0;
  }
}
// Block column j < k goes to host column to.c[j] (the right-hand side's
// index in the caller's arrays).
struct ColMap {
  int32_t c[kBatchMax];
};
static __global__ void k_bscatter(const double *__restrict__ src, int64_t rows, int kp, int k,
                                  ColMap to, double *__restrict__ dst, int64_t ld) {
  const int64_t total = rows * kp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / kp;
    const int j = (int)(i - r * kp);
    if (j < k) dst[(int64_t)to.c[j] * ld + r] = src[i];
  }
}

// dst[r] = x[r*kp + j] + dx[r*kp + j]: the solution of a right-hand side
// retired in the middle of a sweep (the sweep's correction added as X += DX
// adds it at the sweep's end).
static __global__ void k_bput(const double *__restrict__ x, const double *__restrict__ dx,
                              int64_t rows, int kp, int j, double *__restrict__ dst) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows;
       r += (int64_t)gridDim.x * blockDim.x)
    dst[r] = x[r * kp + j] + dx[r * kp + j];
}

// Repacking of a block after retirements: dst[r*kq + j] = src[r*kp + from.c[j]]
// for the k right-hand sides kept (j < k), 0 in the padding columns.
template <typename V>
static __global__ void k_bcompact(const V *__restrict__ src, V *__restrict__ dst, int64_t rows,
                                  int kp, int kq, int k, ColMap from) {
  const int64_t total = rows * kq;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / kq;
    const int j = (int)(i - r * kq);
    dst[i] = j < k ? src[r * kp + from.c[j]] : V(0);
  }
}

// x += dx over the whole block.
static __global__ void k_badd(double *__restrict__ x, const double *__restrict__ dx, int64_t total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += dx[i];
}


// ---- slab form ------------------------------------------------------------------
// The gathered block is cut into slabs of kSlabBytes / 2 (768 rows of 32
// columns); a block of kSlabThreads threads streams the slabs through two
// shared-memory buffers (cp.async: slab s+1 is in flight while slab s is
// read) and its teams (kw/4 lanes, a float4 of the block's row each) add the
// nonzeros of their lines that fall in the slab, keeping one cursor per line:
// entries are sorted by index, so a line's entries in slab s follow those in
// slab s-1.  Every team owns kSlabLines lines; a line's FP32 sum over one
// slab is added to its running sum with two_sum_add.  L2 delivers each slab once per
// block instead of 4*kw bytes per nonzero.
constexpr int kSlabThreads = 1024;
constexpr int kSlabBytes = 196608;  // both buffers
constexpr int kSlabLines = 2;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int kTeam>
__device__ __forceinline__ void slab_load(const float *__restrict__ xf, int base, int cnt,
                                          float4 *buf) {
  constexpr int kw = 4 * kTeam;
  const float4 *src = reinterpret_cast<const float4 *>(xf + (int64_t)base * kw);
  for (int i = threadIdx.x; i < cnt * kTeam; i += kSlabThreads) cp_async16(buf + i, src + i);
  cp_async_commit();
}

template <int kTeam>
__device__ __forceinline__ void slab_accumulate(const int64_t *__restrict__ ptr,
                                                const int32_t *__restrict__ idx,
                                                const float *__restrict__ val,
                                                const float *__restrict__ xf, int n_idx,
                                                const int *lines, float4 *sm,
                                                float (*hi)[4], float (*lo)[4]) {
  constexpr int kw = 4 * kTeam;
  constexpr int S = kSlabBytes / 2 / (4 * kw);  // indices per slab
  const int tl = threadIdx.x % kTeam;
  int64_t cur[kSlabLines], end[kSlabLines];
#pragma unroll
  for (int t = 0; t < kSlabLines; ++t) {
    cur[t] = end[t] = 0;
    if (lines[t] >= 0) {
      cur[t] = ptr[lines[t]];
      end[t] = ptr[lines[t] + 1];
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) hi[t][v] = lo[t][v] = 0.f;
  }
  const int n_slabs = (n_idx + S - 1) / S;
  if (n_slabs > 0) slab_load<kTeam>(xf, 0, min(S, n_idx), sm);
  for (int s = 0; s < n_slabs; ++s) {
    const int base = s * S;
    const int cnt = min(S, n_idx - base);
    float4 *buf = sm + (s & 1) * (S * kTeam);
    if (s + 1 < n_slabs) {
      slab_load<kTeam>(xf, base + S, min(S, n_idx - base - S), sm + ((s + 1) & 1) * (S * kTeam));
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // slab s is in shared memory
    const int lim = base + cnt;
#pragma unroll
    for (int t = 0; t < kSlabLines; ++t) {
      int64_t e = cur[t];
      const int64_t e1 = end[t];
      if (e >= e1 || __ldg(idx + e) >= lim) continue;  // nothing of this line here
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      // four entries in flight; stop at the first one past the slab
      while (e < e1) {
        int c[4];
        float a[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const bool in = e + q < e1;
          c[q] = in ? __ldg(idx + e + q) : INT_MAX;
          a[q] = in ? __ldg(val + e + q) : 0.f;
        }
        int used = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (c[q] >= lim) break;
          const float4 g = buf[(c[q] - base) * kTeam + tl];
          acc[0] = fmaf(a[q], g.x, acc[0]);
          acc[1] = fmaf(a[q], g.y, acc[1]);
          acc[2] = fmaf(a[q], g.z, acc[2]);
          acc[3] = fmaf(a[q], g.w, acc[3]);
          ++used;
        }
        e += used;
        if (used < 4) break;
      }
      cur[t] = e;
#pragma unroll
      for (int v = 0; v < 4; ++v) two_sum_add(hi[t][v], lo[t][v], acc[v]);
    }
    __syncthreads();  // slab s is no longer read: its buffer takes slab s+2
  }
}

// Team sums of squares sq[4] (right-hand sides tl*4 .. tl*4+3) to one partial
// per right-hand side of the block, in team order; `red` holds
// kSlabThreads/kTeam * kw doubles.  Threads j < kw return the sums.
template <int kTeam>
__device__ __forceinline__ double slab_block_sum(const double *sq, double *red) {
  constexpr int kw = 4 * kTeam, kTeams = kSlabThreads / kTeam;
  const int team = threadIdx.x / kTeam, tl = threadIdx.x % kTeam;
  __syncthreads();  // red may alias the slab buffer
#pragma unroll
  for (int v = 0; v < 4; ++v) red[team * kw + tl * 4 + v] = sq[v];
  __syncthreads();
  double s = 0.0;
  if ((int)threadIdx.x < kw)
    for (int q = 0; q < kTeams; ++q) s += red[q * kw + threadIdx.x];
  return s;
}


// Slab A x, kernel rows: U_k[r] = s_j U_k[r] + (K V)[r] for the rows of the
// block's team slots (slots[(block*teams + team)*kSlabLines + t], -1 = none);
// partial sums of squares to parts[block*kw + j].  The damping rows and the
// final reduction follow in k_bdamp_rows.
template <int kTeam>
__global__ void __launch_bounds__(kSlabThreads, 1)
    k_bslab_rows(CsrT<float> K, const int32_t *__restrict__ slots, int n, int k,
                 const float *__restrict__ vf, double *__restrict__ u, int mode,
                 const DevState *__restrict__ st, double *__restrict__ parts) {
  extern __shared__ float4 sm[];
  __shared__ double s_sc[kBatchMax];
  constexpr int kw = 4 * kTeam, kTeams = kSlabThreads / kTeam;
  if (threadIdx.x < kBatchMax) {
    const int j = threadIdx.x;
    s_sc[j] = (j < k && mode == kScaleNegAlpha) ? -st[j].alpha : 1.0;
  }
  const int team = threadIdx.x / kTeam, tl = threadIdx.x % kTeam;
  int lines[kSlabLines];
  const int32_t *sl = slots + ((int64_t)blockIdx.x * kTeams + team) * kSlabLines;
#pragma unroll
  for (int t = 0; t < kSlabLines; ++t) lines[t] = sl[t];
  float hi[kSlabLines][4], lo[kSlabLines][4];
  slab_accumulate<kTeam>(K.ptr, K.idx, K.val, vf, n, lines, sm, hi, lo);
  double sq[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int t = 0; t < kSlabLines; ++t) {
    if (lines[t] < 0) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = tl * 4 + v;
      if (j < k) {
        double *p = u + (int64_t)lines[t] * kw + j;
        const double y = dadd(dmul(s_sc[j], *p), (double)hi[t][v] + (double)lo[t][v]);
        *p = y;
        sq[v] = fma(y, y, sq[v]);
      }
    }
  }
  const double b = slab_block_sum<kTeam>(sq, reinterpret_cast<double *>(sm));
  if ((int)threadIdx.x < kw) parts[(int64_t)blockIdx.x * kw + threadIdx.x] = b;
}

// The damping rows of a batched A x (U_d = s_j U_d + lambda_j D V), 32/kw rows
// per warp with one lane per right-hand side, partials after the `first`
// kernel-row partials; the last block reduces all of them (rows_finish).
static __global__ void __launch_bounds__(kBatchThreads)
    k_bdamp_rows(Csr D, int m_k, int kw, int k, const double *__restrict__ v64,
                 double *__restrict__ u, const double *__restrict__ lambda, int mode,
                 DevState *__restrict__ st, BatchCoef *__restrict__ cf,
                 double *__restrict__ parts, int first) {
  __shared__ double red[kBatchThreads];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int spw = 32 / kw, slot = lane / kw, j = lane % kw;
  const double s = (j < k && mode == kScaleNegAlpha) ? -st[j].alpha : 1.0;
  const double lam = (j < k && lambda) ? lambda[j] : 1.0;
  double *ud = u + (int64_t)m_k * kw;
  double sq = 0.0;
  for (int r = (blockIdx.x * (kBatchThreads / 32) + wib) * spw + slot; r < D.n_lines;
       r += gridDim.x * (kBatchThreads / 32) * spw) {
    double t = 0.0;
    for (int64_t e = D.ptr[r]; e < D.ptr[r + 1]; ++e)
      t = fma(D.val[e], v64[(int64_t)D.idx[e] * kw + j], t);
    if (j < k) {
      double *p = ud + (int64_t)r * kw + j;
      const double y = dadd(dmul(s, *p), dmul(lam, t));
      *p = y;
      sq = fma(y, y, sq);
    }
  }
  const double b = batch_block_sum(sq, kw, red);
  if ((int)threadIdx.x < kw) parts[(int64_t)(first + blockIdx.x) * kw + threadIdx.x] = b;
  if (!batch_last_block(&cf->count)) return;
  rows_finish(parts, first + gridDim.x, kw, k, mode, st, cf);
}

// Slab A^T y: V[c] = s_j V[c] + (K^T U_k)[c] + lambda_j (D^T U_d)[c] for the
// columns of the block's team slots; the damping column is added in FP64 by
// the team's lanes.  The last block finishes the product (cols_finish).
template <int kTeam>
__global__ void __launch_bounds__(kSlabThreads, 1)
    k_bslab_cols(CsrT<float> KC, Csr DC, const int32_t *__restrict__ slots, int m_k, int k,
                 const float *__restrict__ uf, const double *__restrict__ u64,
                 double *__restrict__ v, const double *__restrict__ lambda, int mode,
                 DevState *__restrict__ st, BatchCoef *__restrict__ cf,
                 double *__restrict__ parts) {
  extern __shared__ float4 sm[];
  __shared__ double s_sc[kBatchMax], s_lam[kBatchMax];
  __shared__ int s_act[kBatchMax];
  constexpr int kw = 4 * kTeam, kTeams = kSlabThreads / kTeam;
  if (threadIdx.x < kBatchMax) {
    const int j = threadIdx.x;
    double sc = 1.0;
    int act = j < k;
    if (act && (mode == kScaleNegBeta || mode == kScaleZero)) {
      act = st[j].s_beta_pos && !(mode == kScaleNegBeta && st[j].done);
      sc = mode == kScaleZero ? 0.0 : -st[j].beta;
    }
    s_sc[j] = sc;
    s_act[j] = act;
    s_lam[j] = (j < k && lambda) ? lambda[j] : 1.0;
  }
  const int team = threadIdx.x / kTeam, tl = threadIdx.x % kTeam;
  int lines[kSlabLines];
  const int32_t *sl = slots + ((int64_t)blockIdx.x * kTeams + team) * kSlabLines;
#pragma unroll
  for (int t = 0; t < kSlabLines; ++t) lines[t] = sl[t];
  float hi[kSlabLines][4], lo[kSlabLines][4];
  slab_accumulate<kTeam>(KC.ptr, KC.idx, KC.val, uf, m_k, lines, sm, hi, lo);
  const double *ud = u64 + (int64_t)m_k * kw + tl * 4;
  double sq[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int t = 0; t < kSlabLines; ++t) {
    const int c = lines[t];
    if (c < 0) continue;
    double d[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t e = DC.ptr[c]; e < DC.ptr[c + 1]; ++e) {
      const double a = DC.val[e];
      const double *g = ud + (int64_t)DC.idx[e] * kw;
#pragma unroll
      for (int x = 0; x < 4; ++x) d[x] = fma(a, g[x], d[x]);
    }
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const int j = tl * 4 + x;
      if (s_act[j]) {
        double *p = v + (int64_t)c * kw + j;
        const double y = dadd(dmul(s_sc[j], *p),
                              dadd((double)hi[t][x] + (double)lo[t][x], dmul(s_lam[j], d[x])));
        *p = y;
        sq[x] = fma(y, y, sq[x]);
      }
    }
  }
  const double b = slab_block_sum<kTeam>(sq, reinterpret_cast<double *>(sm));
  if ((int)threadIdx.x < kw) parts[(int64_t)blockIdx.x * kw + threadIdx.x] = b;
  if (!batch_last_block(&cf->count)) return;
  cols_finish(parts, gridDim.x, kw, k, mode, st, cf);
}
}  // namespace plsqr
