// The FP64 LSQR iteration in the reference's order of operations
// (PLSQR_ORDER_REFERENCE): every product, sum and norm is evaluated in the
// order and with the rounding of the reference CPU code built for FP64
// without FMA contraction, so a solve returns the reference's bits.
//
// Why a second path: the Golub-Kahan recurrence of LSQR amplifies rounding
// differences in alpha_k and beta_k (once a Ritz value converges they lose
// all significant digits under a one-ulp change of b, while x itself stays
// put), so per-iteration agreement with the reference on long solves holds
// only for an evaluation with the same rounding.  The default path sums in
// parallel order and is much faster; this one is for bitwise comparisons.
//
//  * products (source/CPUSpMV.c): one thread per line, the line's entries in
//    stored order, t = 0; t = t + val * x[idx] with the multiply and the add
//    rounded apart.  Kernel rows run over K by row, whose entries the device
//    transpose keeps in ascending column order: the order in which the
//    reference's column scatter (CPUSpMV.c:162-183) adds into each row.  The
//    result is folded in as the reference does: dscal, then y += t
//    (aprod_impl.c:138-140, 222-224) and x += (s_k + s_d) (:465-467).
//  * norms (source/mycblas.c:182-222): the scaled sum of squares is a
//    sequential recurrence over the vector.  Its divisions depend only on
//    the running maximum, which is a prefix maximum: two parallel passes find
//    each element's running maximum and turn the element into its term (q*q
//    for an element at or below the running maximum, -q for a new maximum,
//    q = the quotient the reference divides out), and one thread then runs
//    the remaining chain of additions in order.
//  * dknorm (source/lsqr.c:685-690): the x/w update is parallel, its terms
//    go to scratch and one thread adds them in order.
#pragma once

#include "kernels_fp64.cuh"

namespace plsqr {

constexpr int kNrmThreads = 256;
constexpr int kNrmPer = 16;                           // elements per thread
constexpr int kNrmChunk = kNrmThreads * kNrmPer;      // elements per block

// Up to two vectors whose 2-norms one pass computes (y_k and y_d, or v).
struct NrmSeg {
  const double *x;
  int64_t n;
  double *terms;  // [n] scratch
  int b0, nb;     // the segment's blocks [b0, b0 + nb)
};
struct NrmArgs {
  NrmSeg seg[2];
  int nseg;
  double *bmax;   // [blocks] largest |x| of each block's chunk
};

__device__ __forceinline__ int nrm_seg_of(const NrmArgs &a, int b) {
  return (a.nseg > 1 && b >= a.seg[1].b0) ? 1 : 0;
}

// Norm kinds of the chain kernel: beta = ||[y_k; y_d]|| (source/mycblas.c:
// 99-133), alpha = ||v|| (mycblas.c:158-180, one rank).
enum NrmKind : int { kNrmBetaStart = 0, kNrmBeta = 1, kNrmAlpha = 2 };

// Phase 1: the largest |x| of every chunk.  The alpha pass runs only when
// beta > 0 (source/lsqr.c:530-595).
__global__ void __launch_bounds__(kNrmThreads)
    k_nrm_max(NrmArgs a, int kind, const DevState *__restrict__ st) {
  if (kind == kNrmAlpha && !st->s_beta_pos) return;
  __shared__ double smem[kNrmThreads / 32];
  const NrmSeg &s = a.seg[nrm_seg_of(a, blockIdx.x)];
  const int64_t base = (int64_t)(blockIdx.x - s.b0) * kNrmChunk;
  double m = 0.0;
  for (int64_t i = base + threadIdx.x; i < base + kNrmChunk && i < s.n; i += kNrmThreads)
    m = fmax(m, fabs(s.x[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kNrmThreads / 32; ++w) m = fmax(m, smem[w]);
    a.bmax[blockIdx.x] = m;
  }
}

// Phase 2: each element's term of the scaled sum of squares.  scale is the
// largest |x_j| over the earlier elements (0 before the first nonzero): an
// element with |x| > scale starts a new scale (ssq = 1 + ssq * q * q,
// q = scale / |x|), stored as -q; any other nonzero adds (|x| / scale)^2,
// stored as that square; zeros add +0.  -0.0 marks a first nonzero.
__global__ void __launch_bounds__(kNrmThreads)
    k_nrm_terms(NrmArgs a, int kind, const DevState *__restrict__ st) {
  if (kind == kNrmAlpha && !st->s_beta_pos) return;
  __shared__ double smem[kNrmThreads];
  __shared__ double s_prefix;
  const NrmSeg &s = a.seg[nrm_seg_of(a, blockIdx.x)];
  const int rb = blockIdx.x - s.b0;
  // largest |x| of the segment's earlier chunks
  double p = 0.0;
  for (int b = threadIdx.x; b < rb; b += kNrmThreads) p = fmax(p, a.bmax[s.b0 + b]);
  smem[threadIdx.x] = p;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int t = 1; t < kNrmThreads; ++t) p = fmax(p, smem[t]);
    s_prefix = p;
  }
  __syncthreads();
  // exclusive prefix maximum over the threads' runs of kNrmPer elements
  const int64_t i0 = (int64_t)rb * kNrmChunk + (int64_t)threadIdx.x * kNrmPer;
  double m = 0.0;
  for (int k = 0; k < kNrmPer; ++k)
    if (i0 + k < s.n) m = fmax(m, fabs(s.x[i0 + k]));
  smem[threadIdx.x] = m;
  __syncthreads();
  for (int o = 1; o < kNrmThreads; o <<= 1) {  // inclusive max-scan
    const double t = threadIdx.x >= (unsigned)o ? smem[threadIdx.x - o] : 0.0;
    __syncthreads();
    smem[threadIdx.x] = fmax(smem[threadIdx.x], t);
    __syncthreads();
  }
  double run = fmax(s_prefix, threadIdx.x > 0 ? smem[threadIdx.x - 1] : 0.0);
  for (int k = 0; k < kNrmPer; ++k) {
    const int64_t i = i0 + k;
    if (i >= s.n) break;
    const double xi = s.x[i];
    double t = 0.0;
    if (xi != 0.0) {
      const double ax = fabs(xi);
      if (run < ax) {
        t = -ddiv(run, ax);
        run = ax;
      } else {
        const double q = ddiv(ax, run);
        t = dmul(q, q);
      }
    }
    s.terms[i] = t;
  }
}

// Terms staged a chunk at a time: the warp loads the next chunk of terms
// (coalesced, 8 per lane) while lane 0 adds up the current one from shared
// memory, so the chain of additions no longer waits on a global load.
constexpr int kChainChunk = 256;

// The ordered sum of one segment's terms on one thread (lane 0 of the
// segment's warp; the other lanes find the scale and stage the terms);
// source/mycblas.c:182-222: scale * sqrt(ssq), |x[0]| for n = 1, 0 for
// n < 1.  Valid in lane 0.  buf: 2 * kChainChunk doubles of the warp.
__device__ __forceinline__ double nrm_chain(const NrmArgs &a, const NrmSeg &s, double *buf) {
  const int lane = threadIdx.x & 31;
  if (s.n <= 0) return 0.0;
  if (s.n == 1) return fabs(s.x[0]);
  double scale = 0.0;
  for (int b = lane; b < s.nb; b += 32) scale = fmax(scale, a.bmax[s.b0 + b]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) scale = fmax(scale, __shfl_xor_sync(0xffffffffu, scale, o));
  const int64_t n = s.n;
  double ssq = 1.0;
  double r[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int64_t i = k * 32 + lane;
    r[k] = i < n ? s.terms[i] : 0.0;
  }
  for (int64_t c0 = 0; c0 < n; c0 += kChainChunk) {
    double *bc = buf + ((c0 / kChainChunk) & 1) * kChainChunk;
#pragma unroll
    for (int k = 0; k < 8; ++k) bc[k * 32 + lane] = r[k];
    __syncwarp();
    if (c0 + kChainChunk < n) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t i = c0 + kChainChunk + k * 32 + lane;
        r[k] = i < n ? s.terms[i] : 0.0;
      }
    }
    if (lane == 0) {
      const int cnt = (int)(n - c0 < kChainChunk ? n - c0 : kChainChunk);
      int j = 0;
      for (; j + 8 <= cnt; j += 8) {
        double t[8];
        unsigned neg = 0;  // any new scale among the eight (rare: records of a running maximum)
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          t[k] = bc[j + k];
          neg |= (unsigned)(__double2hiint(t[k]) >> 31);
        }
        // the common case keeps one addition per term on the chain (a select
        // between the two updates would put both multiplies on it as well)
        if (!neg) {
#pragma unroll
          for (int k = 0; k < 8; ++k) ssq = dadd(ssq, t[k]);
        } else {
          for (int k = 0; k < 8; ++k) {
            if (signbit(t[k])) ssq = dadd(1.0, dmul(dmul(ssq, -t[k]), -t[k]));
            else ssq = dadd(ssq, t[k]);
          }
        }
      }
      for (; j < cnt; ++j) {
        const double t = bc[j];
        if (signbit(t)) ssq = dadd(1.0, dmul(dmul(ssq, -t), -t));
        else ssq = dadd(ssq, t);
      }
    }
    __syncwarp();
  }
  return lane == 0 ? dmul(scale, __dsqrt_rn(ssq)) : 0.0;
}

// Phase 3: one warp per segment (its lane 0 runs the chain), then the norm
// into the state: beta with
// the anorm update of source/lsqr.c:516-528 (kNrmBeta) or without it (the
// start-up, kNrmBetaStart), or alpha into s_alpha.
__global__ void __launch_bounds__(64) k_nrm_chain(NrmArgs a, int kind, DevState *__restrict__ st) {
  if (kind == kNrmAlpha && !st->s_beta_pos) return;
  __shared__ double res[2];
  __shared__ double buf[2][2 * kChainChunk];
  const int w = threadIdx.x >> 5;
  if (w < a.nseg) {
    const double r = nrm_chain(a, a.seg[w], buf[w]);
    if ((threadIdx.x & 31) == 0) res[w] = r;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (kind == kNrmAlpha) {
    st->s_alpha = __dsqrt_rn(dmul(res[0], res[0]));  // cblas_dnrm2_parallel on one rank
    return;
  }
  const double pk = res[0];
  const double pd = a.nseg > 1 ? __dsqrt_rn(dmul(res[1], res[1])) : 0.0;
  const double beta = __dsqrt_rn(dadd(dmul(pk, pk), dmul(pd, pd)));
  st->beta = beta;
  st->s_beta_pos = beta > 0.0;
  if (kind == kNrmBeta) {
    double temp = d2norm(st->alpha, beta);
    temp = d2norm(temp, st->damp);
    st->anorm = d2norm(st->anorm, temp);
  }
}

// ---------------------------------------------------------------------------
// seq_dot_f64 with the products of eight entries formed ahead of the chain of
// additions (each product is rounded on its own either way, so the sum has
// the same bits); for the long kernel lines.
__device__ __forceinline__ double seq_dot_ahead(const int32_t *__restrict__ idx,
                                                const double *__restrict__ val,
                                                const double *__restrict__ x, int64_t beg,
                                                int64_t end) {
  double t = 0.0;
  int64_t e = beg;
  for (; e + 8 <= end; e += 8) {
    double p[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) p[k] = dmul(__ldg(val + e + k), __ldg(x + __ldg(idx + e + k)));
#pragma unroll
    for (int k = 0; k < 8; ++k) t = dadd(t, p[k]);
  }
  for (; e < end; ++e) t = dadd(t, dmul(val[e], x[idx[e]]));
  return t;
}

// u_k[r] = u_k[r] * s + (K v)[r], u_d[r] = u_d[r] * s + (D v)[r]; one thread
// per row, kernel rows in blocks [0, gk), damping rows in the rest.
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_ref_rows(Csr K, Csr D, const double *__restrict__ v, double *__restrict__ u, int gk,
               int mode, const DevState *__restrict__ st) {
  const double s = mode == kScaleNegAlpha ? -st->alpha : 1.0;
  if ((int)blockIdx.x < gk) {
    for (int r = blockIdx.x * kThreads + threadIdx.x; r < K.n_lines; r += gk * kThreads)
      u[r] = dadd(dmul(u[r], s), seq_dot_ahead(K.idx, K.val, v, K.ptr[r], K.ptr[r + 1]));
    return;
  }
  const int gd = gridDim.x - gk;
  double *ud = u + K.n_lines;
  for (int r = (blockIdx.x - gk) * kThreads + threadIdx.x; r < D.n_lines; r += gd * kThreads)
    ud[r] = dadd(dmul(ud[r], s), seq_dot_f64(D.idx, D.val, v, D.ptr[r], D.ptr[r + 1]));
}

// u *= 1 / beta when beta > 0 (source/lsqr.c:361, 538).
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_ref_scale_u(double *__restrict__ u, int64_t m, const DevState *__restrict__ st) {
  if (!st->s_beta_pos) return;
  const double r = ddiv(1.0, st->beta);
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * kThreads)
    u[i] = dmul(u[i], r);
}

// v[c] = v[c] * s + (s_k + s_d)[c], s_k = (K^T u_k)[c] and s_d = (D^T u_d)[c]
// each summed over the column in stored order; one thread per column.  LSQR:
// s = -beta, skipped when beta == 0 (source/lsqr.c:530-564); start-up: s = 0
// on v = 0 (lsqr.c:311, 366).
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_ref_cols(Csr KC, Csr DC, const double *__restrict__ u, int m_k, double *__restrict__ v,
               int mode, const DevState *__restrict__ st) {
  double s = 1.0;
  if (mode == kScaleNegBeta) {
    if (!st->s_beta_pos) return;
    s = -st->beta;
  } else if (mode == kScaleZero) {
    if (!st->s_beta_pos) return;
    s = 0.0;
  }
  const double *ud = u + m_k;
  for (int c = blockIdx.x * kThreads + threadIdx.x; c < KC.n_lines; c += gridDim.x * kThreads) {
    const double sk = seq_dot_ahead(KC.idx, KC.val, u, KC.ptr[c], KC.ptr[c + 1]);
    const double sd = seq_dot_f64(DC.idx, DC.val, ud, DC.ptr[c], DC.ptr[c + 1]);
    v[c] = dadd(dmul(v[c], s), dadd(sk, sd));
  }
}

// alpha (s_alpha from the norm pass; unchanged when beta == 0), v *= 1/alpha
// when alpha > 0, then the rotation and the x/w update of source/lsqr.c:
// 577-692 with each element's dknorm term, (t3 w)^2, written to dk_terms for
// the ordered sum.  start = 1: the start-up, lsqr.c:375-445 (w = v, x = 0).
template <int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_ref_update(double *__restrict__ v, double *__restrict__ w, double *__restrict__ x,
                 double *__restrict__ se, const double *__restrict__ xref, int n,
                 DevState *__restrict__ st, double *__restrict__ dk_terms,
                 double *__restrict__ parts_err, plsqr_iter *__restrict__ hist, int start) {
  __shared__ double smem[kThreads / 32];
  __shared__ double s_alpha, s_ra;
  __shared__ Step s_step;
  const int beta_pos = st->s_beta_pos;
  if (threadIdx.x == 0) {
    double alpha = beta_pos ? st->s_alpha : (start ? 0.0 : st->alpha);
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
      w[i] = ra != 0.0 ? vi : 0.0;
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
  double e2 = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double vi = v[i];
    if (ra != 0.0) {
      vi = dmul(vi, ra);
      v[i] = vi;
    }
    const double t = w[i];
    const double xi = dadd(dmul(sp.t1, t), x[i]);
    x[i] = xi;
    w[i] = dadd(dmul(sp.t2, t), vi);
    const double tt = dmul(dmul(sp.t3, t), dmul(sp.t3, t));
    if (se) se[i] = dadd(tt, se[i]);
    dk_terms[i] = tt;
    if (xref) {
      const double d = xi - xref[i];
      e2 = fma(d, d, e2);
    }
  }
  if (xref) {
    const double be2 = block_sum<kThreads>(e2, smem);
    if (threadIdx.x == 0) parts_err[blockIdx.x] = be2;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
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

// dknorm^2 = the terms added in element order (source/lsqr.c:685-690), on
// one thread, then the rest of the iteration's scalars (lsqr_tail).
__global__ void __launch_bounds__(32)
    k_ref_tail(DevState *__restrict__ st, const double *__restrict__ dk_terms, int n,
               const double *__restrict__ parts_err, int gp, const double *__restrict__ x,
               plsqr_iter *__restrict__ hist) {
  const int lane = threadIdx.x;
  __shared__ double buf[2 * kChainChunk];
  double e2 = 0.0;
  if (parts_err) {
    for (int b = lane; b < gp; b += 32) e2 += parts_err[b];
    e2 = warp_sum(e2);
  }
  // lane 0 adds the terms in element order; the warp stages them (as in
  // nrm_chain)
  double dk = 0.0;
  double r[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int i = k * 32 + lane;
    r[k] = i < n ? dk_terms[i] : 0.0;
  }
  for (int c0 = 0; c0 < n; c0 += kChainChunk) {
    double *bc = buf + ((c0 / kChainChunk) & 1) * kChainChunk;
#pragma unroll
    for (int k = 0; k < 8; ++k) bc[k * 32 + lane] = r[k];
    __syncwarp();
    if (c0 + kChainChunk < n) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int i = c0 + kChainChunk + k * 32 + lane;
        r[k] = i < n ? dk_terms[i] : 0.0;
      }
    }
    if (lane == 0) {
      const int cnt = n - c0 < kChainChunk ? n - c0 : kChainChunk;
      for (int j = 0; j < cnt; ++j) dk = dadd(bc[j], dk);
    }
    __syncwarp();
  }
  if (lane != 0) return;
  lsqr_tail(*st, dk, e2, x[0], hist);
}

}  // namespace plsqr
