// Independent problems in one persistent launch.
//
// Every problem is a complete FP64 lsqr() (source/lsqr.c:195-917) on its own
// operator [K; D].  The launch is cooperative, so all of its blocks are
// resident at once.  The host plan splits the blocks into groups; group g
// owns blocks [first, first + nb) and a queue of problems that it solves one
// after another.  Inside a group the work of a phase is split over the
// group's warps (kernel rows and columns: nonzero-balanced ranges per warp,
// computed for the group's size) and the phases are separated by a barrier
// in device memory: a counter each block increments once per barrier, and
// waits on until it reaches nb times the barrier's ordinal.  Each wait gives
// up after wait_ns nanoseconds (global timer), sets the launch's error word
// and returns; the other blocks see the word at their next wait, so the
// launch always ends.
//
// Per iteration (four barriers; three in the default mode, see solve_one):
//   A  u = -alpha u + A v            kernel rows (a warp's range, a row per
//                                    lane), damping rows by thread
//   B  beta = ||u||, u /= beta       every block sums the group's partials
//   C  v = -beta v + A^T u           columns (a warp's range, a column per lane)
//   D  alpha = ||v||, v /= alpha, rotation, x/w update, dknorm partials
//   E  (after the barrier) dknorm and the rest of the scalars
// The products form each row and column sum in the reference's order (one
// thread per line), so they are the reference's sums bit for bit; only the
// norms' partial sums are grouped differently.
// Every block keeps its own copy of the scalar state in shared memory and
// computes the same values from the same partial sums; the first block of the
// group writes the history.  Data written by other blocks of the group (u, v,
// x, the partial sums) is read with L2 loads (ld.global.cg): the L1 caches are
// not coherent across blocks.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <queue>
#include <string>
#include <vector>

#include "lsqr_state.cuh"
#include "plsqr_gpu.h"

using namespace plsqr;

// plsqr_gpu.cu: PLSQR_ERR_NUMERIC for NaN, Inf, or magnitudes outside the
// range of the FP64 sums of squares
int magnitude_ok(const double *p, int64_t n, int allow_small = 0);

namespace {

constexpr int kMT = 256;              // threads per block
constexpr int kMW = kMT / 32;         // warps per block

struct MultiProb {
  const int64_t *kr_ptr;  // K by row
  const int32_t *kr_idx;
  const double *kr_val;
  const int64_t *kc_ptr;  // K by column
  const int32_t *kc_idx;
  const double *kc_val;
  const int64_t *dr_ptr;  // D by row
  const int32_t *dr_idx;
  const double *dr_val;
  const int64_t *dc_ptr;  // D by column
  const int32_t *dc_idx;
  const double *dc_val;
  const int32_t *korder; // [m_k] kernel rows, longest first (the lanes of a warp
                         // then sum rows of about the same length)
  const int32_t *kpart;  // [nw + 1] range of korder of each warp of the group
  const int32_t *cpart;  // [nw + 1] column range of each warp of the group
  const double *b;
  double *u, *v, *w, *x;
  // mixed precision (plsqr_multi_set_mixed): FP32 kernel values by row and
  // by column, hi + lo FP32 mirrors of u_k and v, the sweep's correction
  const float *kr_val32, *kc_val32;
  float2 *uhl, *vhl;  // (hi, lo) pairs: one 8-byte gather per nonzero
  double *dx;
  plsqr_iter *hist;  // [iters + 1]
  int32_t m_k, m_d, n, iters, itnlim, pad;
  double damp, atol, btol, ctol;
};

struct MultiGroup {
  int32_t first, nb, q_begin, q_end;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// A bounded wait of thread 0 until *word >= target; 0 on success, else an
// error code (also stored in *err unless another wait stored one first).
__device__ int bounded_wait(const unsigned int *word, unsigned int target, int *err,
                            long long wait_ns) {
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (*(volatile const unsigned int *)word >= target) return 0;
    const int e = *(volatile int *)err;
    if (e) return e;
    if ((long long)(global_ns() - t0) > wait_ns) {
      atomicCAS(err, 0, PLSQR_ERR_TIMEOUT);
      return PLSQR_ERR_TIMEOUT;
    }
    __nanosleep(64);
  }
}

struct Group {
  int rank, nb, first;  // this block's rank in the group, group size, first block
  unsigned int *bar;
  unsigned int epoch;
  int *err;
  long long wait_ns;
};

// Barrier of the group's blocks; false when the launch is being abandoned.
__device__ bool group_sync(Group &g) {
  __shared__ int s_ok;
  if (g.nb == 1) {
    __threadfence();  // the L2 loads after the barrier see this block's stores
    __syncthreads();
    return true;
  }
  __syncthreads();
  ++g.epoch;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(g.bar, 1u);
    s_ok = bounded_wait(g.bar, g.epoch * (unsigned)g.nb, g.err, g.wait_ns) == 0;
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ double ld(const double *p) { return __ldcg(p); }

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of the group's partials parts[first .. first + nb) in a fixed order
// (lane-strided, then a shuffle tree), by warp 0; valid in thread 0.
__device__ double group_parts_sum(const double *parts, const Group &g) {
  double s = 0.0;
  if (threadIdx.x < 32) {
    for (int q = threadIdx.x; q < g.nb; q += 32) s += ld(parts + g.first + q);
    s = wsum(s);
  }
  return s;
}

// Block sum of one value per thread (fixed order); valid in thread 0.
__device__ double block_total(double v, double *red) {
  v = wsum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kMW; ++i) s += red[i];
  __syncthreads();
  return s;
}

// One line times a vector by one thread, in stored order.  kExact: the
// multiply and the add rounded apart, the reference's sums term for term
// (cpuSpMV_CSC accumulates each row over ascending columns, CPUSpMV.c:162-183;
// cpuSpMVTranspose_CSC each column over its stored rows, CPUSpMV.c:203-245;
// the damping rows and columns, CPUSpMV.c:67-70, 270-275).  Otherwise fused
// multiply-adds: half the FP64 instructions (the GB300's FP64 pipe, two per
// clock per SM, bounds these small problems), the rounding of the
// one-problem path.  Vector entries come from L2.
template <bool kExact>
__device__ __forceinline__ double seq_line(const int32_t *__restrict__ idx,
                                           const double *__restrict__ val, const double *vec,
                                           int64_t beg, int64_t end) {
  double t = 0.0;
  for (int64_t e = beg; e < end; ++e) {
    const double a = __ldg(val + e), x = ld(vec + __ldg(idx + e));
    t = kExact ? plsqr::dadd(t, plsqr::dmul(a, x)) : fma(a, x, t);
  }
  return t;
}

// One line of FP32 values times a vector of (hi, lo) FP32 pairs by one
// thread, in stored order: the product's error recovered by a fused
// multiply-add, the sum's by Knuth's two-sum, both collected with the lo
// products in a second float; the FP32 values times the FP64 vector to
// about 2^-44, in FP32 instructions only.
__device__ __forceinline__ double seq_line32(const int32_t *__restrict__ idx,
                                             const float *__restrict__ val, const float2 *xhl,
                                             int64_t beg, int64_t end) {
  float s = 0.0f, c = 0.0f;
  for (int64_t e = beg; e < end; ++e) {
    const int j = __ldg(idx + e);
    const float2 x = __ldcg(xhl + j);
    const float a = __ldg(val + e), h = x.x, l = x.y;
    const float p = __fmul_rn(a, h);
    const float pe = __fmaf_rn(a, h, -p);
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float er = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(er, __fmaf_rn(a, l, pe)));
  }
  return (double)s + (double)c;
}

// FP64 value -> hi + lo FP32 pair
__device__ __forceinline__ void split_store(float2 *hl, int64_t i, double y) {
  const float h = (float)y;
  hl[i] = make_float2(h, (float)(y - (double)h));
}

template <bool kExact>
__device__ __forceinline__ double kernel_row(const MultiProb &P, const double *v, int r) {
  return seq_line<kExact>(P.kr_idx, P.kr_val, v, P.kr_ptr[r], P.kr_ptr[r + 1]);
}
template <bool kExact>
__device__ __forceinline__ double kernel_col(const MultiProb &P, const double *u, int c) {
  return seq_line<kExact>(P.kc_idx, P.kc_val, u, P.kc_ptr[c], P.kc_ptr[c + 1]);
}
template <bool kExact>
__device__ __forceinline__ double damp_col(const MultiProb &P, const double *u, int c) {
  return seq_line<kExact>(P.dc_idx, P.dc_val, u + P.m_k, P.dc_ptr[c], P.dc_ptr[c + 1]);
}

}  // namespace

namespace {

// Shared per-block state of the problem being solved.
struct BlockScalars {
  DevState S;
  double rb, ra;  // 1/beta, 1/alpha (0: leave the vector)
  Step step;
};

// One problem, by all blocks of the group.  Returns false when the launch is
// being abandoned (a wait gave up).  kMixed: `sweeps` refinement sweeps, each
// an LSQR of P.iters iterations for the correction dx on the FP64 residual
// r = b - A x (kernel rows in FP64), with the kernel products in FP32 over
// hi + lo mirrors of u_k and v; x += dx after each sweep.  The history and
// the returned state are the last sweep's.
template <bool kExact, bool kMixed>
__device__ bool solve_one(const MultiProb &P, Group &g, double *parts_u, double *parts_v,
                          double *parts_dk, DevState *out, BlockScalars &sh, double *red,
                          int sweeps) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int gw = g.rank * kMW + (tid >> 5);               // warp of the group
  const int64_t gt = (int64_t)g.rank * kMT + tid;          // thread of the group
  const int64_t gstride = (int64_t)g.nb * kMT;
  const int64_t m = (int64_t)P.m_k + P.m_d;
  double *u = P.u, *v = P.v, *w = P.w;
  double *x = kMixed ? P.dx : P.x;  // the iterate the LSQR updates
  const bool lead = g.rank == 0;
  if (!kMixed) sweeps = 1;
  if (kMixed) {
    for (int64_t i = gt; i < P.n; i += gstride) P.x[i] = 0.0;
  }

  for (int sweep = 0; sweep < sweeps; ++sweep) {
  // ---- start-up: u = b (kMixed: b - A x), v = 0, x = 0 (source/lsqr.c:311-312, 343-409) ----
  if (tid == 0) {
    DevState &S = sh.S;
    memset(&S, 0, sizeof(S));
    S.damp = P.damp;
    S.atol = P.atol;
    S.btol = P.btol;
    S.ctol = P.ctol;
    S.itnlim = P.itnlim;
    S.cs2 = -1.0;
  }
  double sq = 0.0;
  if (kMixed && sweep > 0) {
    // FP64 residual of the current x: kernel rows by warp range, damping rows by thread
    for (int i = P.kpart[gw] + lane; i < P.kpart[gw + 1]; i += 32) {
      const int r = P.korder[i];
      const double y = __ldg(P.b + r) - kernel_row<false>(P, P.x, r);
      u[r] = y;
      sq = fma(y, y, sq);
    }
    for (int64_t r = gt; r < P.m_d; r += gstride) {
      const double y = -seq_line<false>(P.dr_idx, P.dr_val, P.x, P.dr_ptr[r], P.dr_ptr[r + 1]);
      u[P.m_k + r] = y;
      sq = fma(y, y, sq);
    }
  } else {
    for (int64_t i = gt; i < m; i += gstride) {
      const double y = i < P.m_k ? __ldg(P.b + i) : 0.0;
      u[i] = y;
      sq = fma(y, y, sq);
    }
  }
  for (int64_t i = gt; i < P.n; i += gstride) {
    v[i] = 0.0;
    x[i] = 0.0;
  }
  double bs = block_total(sq, red);
  if (tid == 0) parts_u[g.first + g.rank] = bs;
  if (!group_sync(g)) return false;
  // beta = ||b||, u /= beta
  bs = group_parts_sum(parts_u, g);
  if (tid == 0) {
    const double beta = __dsqrt_rn(bs);
    sh.S.beta = beta;
    sh.S.s_beta_pos = beta > 0.0;
    sh.rb = beta > 0.0 ? plsqr::ddiv(1.0, beta) : 0.0;
  }
  __syncthreads();
  if (sh.rb != 0.0)
    for (int64_t i = gt; i < m; i += gstride) {
      const double y = plsqr::dmul(ld(u + i), sh.rb);
      u[i] = y;
      if (kMixed && i < P.m_k) split_store(P.uhl, i, y);
    }
  if (!group_sync(g)) return false;
  // v = A^T u (when beta > 0)
  sq = 0.0;
  if (sh.S.s_beta_pos) {
    for (int c = P.cpart[gw] + lane; c < P.cpart[gw + 1]; c += 32) {
      const double k = kMixed ? seq_line32(P.kc_idx, P.kc_val32, P.uhl, P.kc_ptr[c], P.kc_ptr[c + 1])
                              : kernel_col<kExact>(P, u, c);
      const double t = plsqr::dadd(k, damp_col<kExact>(P, u, c));  // x += (s_k + s_d)
      v[c] = t;
      sq = fma(t, t, sq);
    }
  }
  bs = block_total(sq, red);
  if (tid == 0) parts_v[g.first + g.rank] = bs;
  if (!group_sync(g)) return false;
  // alpha = ||v||, v /= alpha, w = v
  bs = group_parts_sum(parts_v, g);
  if (tid == 0) {
    DevState &S = sh.S;
    const double alpha = S.s_beta_pos ? __dsqrt_rn(bs) : 0.0;
    sh.ra = (S.s_beta_pos && alpha > 0.0) ? plsqr::ddiv(1.0, alpha) : 0.0;
    S.alpha = alpha;
    S.arnorm = plsqr::dmul(alpha, S.beta);
    S.rhobar = alpha;
    S.phibar = S.beta;
    S.bnorm = S.beta;
    S.rnorm = S.beta;
    S.done = S.arnorm == 0.0;
    if (lead && P.hist) {
      plsqr_iter &h = P.hist[0];
      memset(&h, 0, sizeof(h));
      h.alpha = alpha;
      h.beta = S.beta;
      h.rnorm = S.beta;
      h.arnorm = S.arnorm;
      h.test1 = 1.0;
      h.test2 = S.beta > 0.0 ? plsqr::ddiv(alpha, S.beta) : 0.0;
      h.err = -1.0;
    }
  }
  __syncthreads();
  for (int64_t i = gt; i < P.n; i += gstride) {
    double vi = ld(v + i);
    if (sh.ra != 0.0) vi = plsqr::dmul(vi, sh.ra);
    v[i] = vi;
    if (kMixed) split_store(P.vhl, i, vi);
    w[i] = sh.ra != 0.0 ? vi : 0.0;
  }
  if (!group_sync(g)) return false;
  const int iters = sh.S.done ? 0 : P.iters;

  // Default mode: u is kept unscaled between B and the next A, so B needs no
  // pass over u and no barrier of its own: C multiplies its column sums by
  // 1/beta and A scales each u element as it reads it (the same product the
  // reference's scaling rounds).  rb_u: the scale u still carries.  The
  // mixed products read the mirror of the unscaled u_k that A writes.
  double rb_u = 1.0;
  for (int it = 0; it < iters; ++it) {
    // A: u = -alpha u + A v
    const double s1 = -sh.S.alpha;
    sq = 0.0;
    for (int i = P.kpart[gw] + lane; i < P.kpart[gw + 1]; i += 32) {
      const int r = P.korder[i];
      const double ur = kExact ? ld(u + r) : plsqr::dmul(ld(u + r), rb_u);
      const double k = kMixed ? seq_line32(P.kr_idx, P.kr_val32, P.vhl, P.kr_ptr[r], P.kr_ptr[r + 1])
                              : kernel_row<kExact>(P, v, r);
      const double y = plsqr::dadd(plsqr::dmul(s1, ur), k);
      u[r] = y;
      if (kMixed) split_store(P.uhl, r, y);
      sq = fma(y, y, sq);
    }
    for (int64_t r = gt; r < P.m_d; r += gstride) {
      const double t = seq_line<kExact>(P.dr_idx, P.dr_val, v, P.dr_ptr[r], P.dr_ptr[r + 1]);  // CPUSpMV.c:67-70
      double *p = u + P.m_k + r;
      const double ur = kExact ? ld(p) : plsqr::dmul(ld(p), rb_u);
      const double y = plsqr::dadd(plsqr::dmul(s1, ur), t);
      *p = y;
      sq = fma(y, y, sq);
    }
    bs = block_total(sq, red);
    if (tid == 0) parts_u[g.first + g.rank] = bs;
    if (!group_sync(g)) return false;
    // B: beta, anorm (source/lsqr.c:526-528), u /= beta
    bs = group_parts_sum(parts_u, g);
    if (tid == 0) {
      DevState &S = sh.S;
      const double beta = __dsqrt_rn(bs);
      S.beta = beta;
      S.s_beta_pos = beta > 0.0;
      double temp = d2norm(S.alpha, beta);
      temp = d2norm(temp, S.damp);
      S.anorm = d2norm(S.anorm, temp);
      sh.rb = beta > 0.0 ? plsqr::ddiv(1.0, beta) : 0.0;
    }
    __syncthreads();
    if (kExact) {
      if (sh.rb != 0.0)
        for (int64_t i = gt; i < m; i += gstride) u[i] = plsqr::dmul(ld(u + i), sh.rb);
      if (!group_sync(g)) return false;
    } else {
      rb_u = sh.rb != 0.0 ? sh.rb : 1.0;  // beta = 0: u is left as it is
    }
    // C: v = -beta v + A^T u (skipped when beta = 0, source/lsqr.c:530)
    sq = 0.0;
    if (sh.S.s_beta_pos) {
      const double s2 = -sh.S.beta;
      const double rb = sh.rb;
      for (int c = P.cpart[gw] + lane; c < P.cpart[gw + 1]; c += 32) {
        const double k = kMixed ? seq_line32(P.kc_idx, P.kc_val32, P.uhl, P.kc_ptr[c], P.kc_ptr[c + 1])
                                : kernel_col<kExact>(P, u, c);
        double t = plsqr::dadd(k, damp_col<kExact>(P, u, c));
        if (!kExact) t = plsqr::dmul(t, rb);
        const double y = plsqr::dadd(plsqr::dmul(s2, ld(v + c)), t);
        v[c] = y;
        sq = fma(y, y, sq);
      }
    }
    bs = block_total(sq, red);
    if (tid == 0) parts_v[g.first + g.rank] = bs;
    if (!group_sync(g)) return false;
    // D: alpha, v /= alpha, rotation (source/lsqr.c:551-636), x/w update
    bs = group_parts_sum(parts_v, g);
    if (tid == 0) {
      DevState &S = sh.S;
      const double alpha = S.s_beta_pos ? __dsqrt_rn(bs) : S.alpha;
      sh.ra = (S.s_beta_pos && alpha > 0.0) ? plsqr::ddiv(1.0, alpha) : 0.0;
      sh.step = lsqr_step(S, alpha, S.beta);
      S.s_alpha = alpha;
      S.s_rhobar = sh.step.rhobar;
      S.s_phibar = sh.step.phibar;
      S.s_psi = sh.step.psi;
      S.s_phi = sh.step.phi;
      S.s_rho = sh.step.rho;
      S.s_theta = sh.step.theta;
      S.s_tau = sh.step.tau;
    }
    __syncthreads();
    const double ra = sh.ra, t1 = sh.step.t1, t2 = sh.step.t2, t3 = sh.step.t3;
    double dk = 0.0;
    for (int64_t i = gt; i < P.n; i += gstride) {
      double vi = ld(v + i);
      if (ra != 0.0) {
        vi = plsqr::dmul(vi, ra);
        v[i] = vi;
      }
      if (kMixed) split_store(P.vhl, i, vi);
      const double t = w[i];
      x[i] = plsqr::dadd(plsqr::dmul(t1, t), x[i]);
      w[i] = plsqr::dadd(plsqr::dmul(t2, t), vi);
      dk += plsqr::dmul(plsqr::dmul(t3, t), plsqr::dmul(t3, t));
    }
    bs = block_total(dk, red);
    if (tid == 0) parts_dk[g.first + g.rank] = bs;
    if (!group_sync(g)) return false;
    // E: the rest of the scalars and the history record
    bs = group_parts_sum(parts_dk, g);
    if (tid == 0) lsqr_tail(sh.S, bs, 0.0, ld(x), lead ? P.hist : nullptr);
    __syncthreads();
  }
  if (kMixed) {  // x += dx
    for (int64_t i = gt; i < P.n; i += gstride) P.x[i] = P.x[i] + ld(x + i);
    if (!group_sync(g)) return false;
  }
  }  // sweeps
  if (tid == 0 && lead) *out = sh.S;
  return true;
}

// The persistent kernel: block b runs the queue of its group.
template <bool kExact, bool kMixed>
__global__ void __launch_bounds__(kMT, 4)  // 4 blocks per SM (64 registers)
    k_multi_lsqr(const MultiProb *__restrict__ probs, const MultiGroup *__restrict__ groups,
                 const int32_t *__restrict__ queue, const int32_t *__restrict__ block_group,
                 unsigned int *bars, double *parts, DevState *out, int *err, long long wait_ns,
                 int sweeps) {
  __shared__ BlockScalars sh;
  __shared__ double red[kMW];
  const int gi = block_group[blockIdx.x];
  const MultiGroup G = groups[gi];
  Group g{(int)blockIdx.x - G.first, G.nb, G.first, bars + gi, 0u, err, wait_ns};
  const int nblk = gridDim.x;
  for (int q = G.q_begin; q < G.q_end; ++q) {
    const int p = queue[q];
    if (!solve_one<kExact, kMixed>(probs[p], g, parts, parts + nblk, parts + 2 * nblk, out + p,
                                   sh, red, sweeps))
      return;
  }
}

// One bounded wait on a word that nothing writes (thread 0 of one block).
__global__ void k_check_wait(const unsigned int *word, int *err, long long wait_ns) {
  if (threadIdx.x == 0) bounded_wait(word, 1u, err, wait_ns);
}

}  // namespace

// ---- host side -------------------------------------------------------------------
struct plsqr_multi {
  plsqr_opts opts;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int count = 0, sm_count = 0, blocks_per_sm = 0, blocks = 0;
  std::vector<MultiProb> desc;  // device pointers
  std::vector<int32_t> n, iters;
  std::vector<int64_t> hist_off;  // first history record of each problem
  int64_t hist_total = 0, x_total = 0;
  std::vector<int32_t> group_of, group_blocks;
  MultiProb *d_probs = nullptr;
  MultiGroup *d_groups = nullptr;
  int32_t *d_queue = nullptr, *d_block_group = nullptr;
  unsigned int *d_bars = nullptr;  // one barrier word per launched group
  int n_bars = 0;
  unsigned int *d_zero = nullptr;
  double *d_parts = nullptr;
  DevState *d_out = nullptr;
  plsqr_iter *d_hist = nullptr;
  int *d_err = nullptr;
  std::vector<void *> allocs;
  int64_t device_bytes = 0;
  long long wait_ns = 1000000000LL;
  int exact = 0;  // products in the reference's rounding (DMUL + DADD)
  int sweeps = 0;  // > 0: FP32-inner / FP64-outer sweeps (plsqr_multi_set_mixed)
  double seconds = 0.0;
  char last_error[512] = {0};
};

namespace {

void set_error(plsqr_multi *mp, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(mp->last_error, sizeof mp->last_error, fmt, ap);
  va_end(ap);
}

#define MK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      set_error(mp, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return PLSQR_ERR_CUDA;                                                          \
    }                                                                                 \
  } while (0)

template <class T>
int upload(plsqr_multi *mp, T **dst, const T *src, size_t count) {
  void *p = nullptr;
  MK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
  mp->allocs.push_back(p);
  mp->device_bytes += (int64_t)(std::max<size_t>(count, 1) * sizeof(T));
  if (src && count) MK(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
  *dst = (T *)p;
  return PLSQR_OK;
}

// A compressed-sparse operand with int64 pointers, checked on the host
// (no index may reach the device out of range).
int checked_lines(const plsqr_sparse *a, int32_t rows, int32_t cols, bool by_col,
                  std::vector<int64_t> &ptr) {
  if ((!a->ptr32 && !a->ptr64) || (a->ptr32 && a->ptr64)) return PLSQR_ERR_ARG;
  if (a->num_row != rows || a->num_col != cols || a->nnz < 0) return PLSQR_ERR_ARG;
  const int32_t nl = by_col ? cols : rows, ni = by_col ? rows : cols;
  ptr.resize((size_t)nl + 1);
  for (int32_t i = 0; i <= nl; ++i) ptr[(size_t)i] = a->ptr32 ? a->ptr32[i] : a->ptr64[i];
  if (ptr[0] != 0 || ptr[(size_t)nl] != a->nnz) return PLSQR_ERR_FORMAT;
  for (int32_t i = 0; i < nl; ++i)
    if (ptr[(size_t)i + 1] < ptr[(size_t)i]) return PLSQR_ERR_FORMAT;
  if (a->nnz > 0 && (!a->idx || !a->val)) return PLSQR_ERR_ARG;
  for (int64_t e = 0; e < a->nnz; ++e)
    if (a->idx[e] < 0 || a->idx[e] >= ni) return PLSQR_ERR_FORMAT;
  return magnitude_ok(a->val, a->nnz, 1);
}

void split_by_nnz(const std::vector<int64_t> &pre, int parts, std::vector<int32_t> &out) {
  const int32_t nl = (int32_t)pre.size() - 1;
  out.assign((size_t)parts + 1, 0);
  const int64_t tot = pre.back();
  for (int w = 1; w < parts; ++w) {
    const int64_t target = (int64_t)((long double)tot * w / parts);
    const int32_t r = (int32_t)(std::lower_bound(pre.begin(), pre.end(), target) - pre.begin());
    out[(size_t)w] = std::max(std::min(r, nl), out[(size_t)w - 1]);
  }
  out[(size_t)parts] = nl;
}

// Planner cost model: an iteration streams the operator twice (12 bytes per
// nonzero each time) and a few vector passes, at an equal share of the HBM
// bandwidth per block, plus four barriers whose cost grows with the group.
struct CostModel {
  double bw_block;  // bytes/s one block streams
  double work(int64_t nnz, int64_t m, int64_t n) const {
    return 24.0 * (double)nnz + 56.0 * (double)(m + n);
  }
  double time(double bytes, int iters, int nb) const {
    const double sync = nb == 1 ? 4 * 0.5e-6 : 4 * (2.5e-6 + 0.02e-6 * nb);
    return iters * (bytes / (nb * bw_block) + sync);
  }
};

}  // namespace

// Groups and queues: with at least as many blocks as problems every problem
// gets its own group, and the spare blocks go one at a time to the problem
// with the longest modelled time while that shortens it; otherwise the
// problems are packed longest first onto single-block groups, each onto the
// group with the least modelled work so far.
static void plan(const std::vector<double> &bytes, const std::vector<int32_t> &iters, int blocks,
                 double bw_block, std::vector<int32_t> &group_of, std::vector<int32_t> &nb,
                 std::vector<std::vector<int32_t>> &queues) {
  const int P = (int)bytes.size();
  CostModel cm{bw_block};
  group_of.assign((size_t)P, 0);
  nb.clear();
  queues.clear();
  if (P <= blocks) {
    nb.assign((size_t)P, 1);
    std::priority_queue<std::pair<double, int>> pq;
    for (int p = 0; p < P; ++p) pq.push({cm.time(bytes[(size_t)p], iters[(size_t)p], 1), p});
    int spare = blocks - P;
    while (spare > 0 && !pq.empty()) {
      auto top = pq.top();
      pq.pop();
      const int p = top.second;
      const double t1 = cm.time(bytes[(size_t)p], iters[(size_t)p], nb[(size_t)p] + 1);
      if (t1 >= top.first) continue;  // more blocks would not help this one
      ++nb[(size_t)p];
      --spare;
      pq.push({t1, p});
    }
    for (int p = 0; p < P; ++p) {
      group_of[(size_t)p] = p;
      queues.push_back({p});
    }
    return;
  }
  std::vector<int> order((size_t)P);
  for (int p = 0; p < P; ++p) order[(size_t)p] = p;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return cm.time(bytes[(size_t)a], iters[(size_t)a], 1) > cm.time(bytes[(size_t)b], iters[(size_t)b], 1);
  });
  nb.assign((size_t)blocks, 1);
  queues.assign((size_t)blocks, {});
  std::priority_queue<std::pair<double, int>, std::vector<std::pair<double, int>>,
                      std::greater<std::pair<double, int>>>
      load;
  for (int g = 0; g < blocks; ++g) load.push({0.0, g});
  for (int p : order) {
    auto top = load.top();
    load.pop();
    queues[(size_t)top.second].push_back(p);
    group_of[(size_t)p] = top.second;
    load.push({top.first + cm.time(bytes[(size_t)p], iters[(size_t)p], 1), top.second});
  }
}

// ---- C ABI ---------------------------------------------------------------------
extern "C" void plsqr_default_problem(plsqr_problem *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->lsqr_iteration = 100;
  p->itnlim = 1000;  // source/lsqr.c:47-51
  p->atol = 1e-10;
  p->btol = 1e-10;
  p->conlim = 100;
}

extern "C" void plsqr_multi_destroy(plsqr_multi *mp) {
  if (!mp) return;
  cudaSetDevice(mp->opts.device);
  for (void *p : mp->allocs) cudaFree(p);
  if (mp->ev0) cudaEventDestroy(mp->ev0);
  if (mp->ev1) cudaEventDestroy(mp->ev1);
  if (mp->stream) cudaStreamDestroy(mp->stream);
  delete mp;
}

extern "C" const char *plsqr_multi_last_error(const plsqr_multi *mp) {
  return mp ? mp->last_error : "";
}

static int multi_build(plsqr_multi *mp, const plsqr_problem *probs) {
  const int P = mp->count;
  MK(cudaSetDevice(mp->opts.device));
  MK(cudaStreamCreateWithFlags(&mp->stream, cudaStreamNonBlocking));
  MK(cudaEventCreate(&mp->ev0));
  MK(cudaEventCreate(&mp->ev1));
  int coop = 0;
  MK(cudaDeviceGetAttribute(&mp->sm_count, cudaDevAttrMultiProcessorCount, mp->opts.device));
  MK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, mp->opts.device));
  if (!coop) {
    set_error(mp, "device does not support cooperative launches");
    return PLSQR_ERR_NODEV;
  }
  int occ = 0;
  int occ2 = 0;
  int occ3 = 0;
  MK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_multi_lsqr<false, false>, kMT, 0));
  MK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, k_multi_lsqr<true, false>, kMT, 0));
  MK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ3, k_multi_lsqr<false, true>, kMT, 0));
  occ = std::min({occ, occ2, occ3});
  mp->blocks_per_sm = std::max(1, std::min(occ, 4));
  mp->blocks = mp->sm_count * mp->blocks_per_sm;
  // host copies: pointers as int64, K by row
  std::vector<std::vector<int64_t>> kc(P), dr(P), dc(P), kr(P);
  std::vector<std::vector<int32_t>> kri(P);
  std::vector<std::vector<double>> krv(P);
  std::vector<double> bytes((size_t)P);
  mp->n.resize((size_t)P);
  mp->iters.resize((size_t)P);
  for (int p = 0; p < P; ++p) {
    const plsqr_problem &q = probs[p];
    const int32_t m_k = q.k_csc.num_row, n = q.k_csc.num_col, m_d = q.d_csr.num_row;
    int rc;
    if (m_k < 0 || n < 1 || m_d < 0 || q.lsqr_iteration < 0 || (m_k > 0 && !q.b_k)) {
      set_error(mp, "problem %d: bad sizes or arguments", p);
      return PLSQR_ERR_ARG;
    }
    if ((rc = checked_lines(&q.k_csc, m_k, n, true, kc[(size_t)p])) ||
        (rc = checked_lines(&q.d_csr, m_d, n, false, dr[(size_t)p])) ||
        (rc = checked_lines(&q.d_csc, m_d, n, true, dc[(size_t)p]))) {
      set_error(mp, "problem %d: inconsistent operator", p);
      return rc;
    }
    if ((rc = magnitude_ok(q.b_k, m_k))) {
      set_error(mp, "problem %d: b_k holds NaN, Inf or magnitudes outside [2^-500, 2^500]", p);
      return rc;
    }
    if (q.d_csc.nnz != q.d_csr.nnz) return PLSQR_ERR_FORMAT;
    kr[(size_t)p].resize((size_t)m_k + 1);
    kri[(size_t)p].resize((size_t)q.k_csc.nnz);
    krv[(size_t)p].resize((size_t)q.k_csc.nnz);
    if ((rc = plsqr_transpose(n, m_k, kc[(size_t)p].data(), q.k_csc.idx, q.k_csc.val,
                              kr[(size_t)p].data(), kri[(size_t)p].data(), krv[(size_t)p].data())))
      return rc;
    mp->n[(size_t)p] = n;
    mp->iters[(size_t)p] = q.lsqr_iteration;
    bytes[(size_t)p] = CostModel{1.0}.work(q.k_csc.nnz + q.d_csr.nnz, (int64_t)m_k + m_d, n);
  }
  std::vector<int32_t> nb;
  std::vector<std::vector<int32_t>> queues;
  plan(bytes, mp->iters, mp->blocks, 6.0e12 / mp->blocks, mp->group_of, nb, queues);
  const int G = (int)nb.size();
  mp->group_blocks = nb;
  std::vector<MultiGroup> groups((size_t)G);
  std::vector<int32_t> queue, block_group((size_t)mp->blocks, 0);
  int first = 0;
  for (int g = 0; g < G; ++g) {
    groups[(size_t)g] = MultiGroup{first, nb[(size_t)g], (int32_t)queue.size(), 0};
    queue.insert(queue.end(), queues[(size_t)g].begin(), queues[(size_t)g].end());
    groups[(size_t)g].q_end = (int32_t)queue.size();
    for (int b = 0; b < nb[(size_t)g]; ++b) block_group[(size_t)(first + b)] = g;
    first += nb[(size_t)g];
  }
  // blocks the plan left unused run an empty queue
  if (first < mp->blocks) {
    groups.push_back(MultiGroup{first, mp->blocks - first, 0, 0});
    for (int b = first; b < mp->blocks; ++b) block_group[(size_t)b] = G;
  }
  // operators, vectors and per-warp ranges
  mp->desc.resize((size_t)P);
  mp->hist_off.resize((size_t)P);
  mp->hist_total = 0;
  mp->x_total = 0;
  int rc;
  for (int p = 0; p < P; ++p) {
    const plsqr_problem &q = probs[p];
    MultiProb &d = mp->desc[(size_t)p];
    memset(&d, 0, sizeof(d));
    const int32_t m_k = q.k_csc.num_row, n = q.k_csc.num_col, m_d = q.d_csr.num_row;
    const int nw = nb[(size_t)mp->group_of[(size_t)p]] * kMW;
    std::vector<int32_t> kp, cp, ko((size_t)m_k);
    {  // kernel rows longest first; the warps' ranges balanced in that order
      const std::vector<int64_t> &rp = kr[(size_t)p];
      for (int32_t r = 0; r < m_k; ++r) ko[(size_t)r] = r;
      std::stable_sort(ko.begin(), ko.end(), [&](int32_t a, int32_t b) {
        return rp[(size_t)a + 1] - rp[(size_t)a] > rp[(size_t)b + 1] - rp[(size_t)b];
      });
      std::vector<int64_t> pre((size_t)m_k + 1, 0);
      for (int32_t i = 0; i < m_k; ++i)
        pre[(size_t)i + 1] = pre[(size_t)i] + (rp[(size_t)ko[(size_t)i] + 1] - rp[(size_t)ko[(size_t)i]]);
      split_by_nnz(pre, nw, kp);
    }
    std::vector<int64_t> pre((size_t)n + 1);
    for (int32_t c = 0; c <= n; ++c)
      pre[(size_t)c] = kc[(size_t)p][(size_t)c] + dc[(size_t)p][(size_t)c];
    split_by_nnz(pre, nw, cp);
    const int64_t m = (int64_t)m_k + m_d;
    int64_t *kr_ptr, *kc_ptr, *dr_ptr, *dc_ptr;
    int32_t *kr_idx, *kc_idx, *dr_idx, *dc_idx, *kpart, *cpart, *korder;
    double *kr_val, *kc_val, *dr_val, *dc_val, *b, *u, *v, *w, *x, *dx;
    float *kr_val32, *kc_val32;
    float2 *uhl, *vhl;
    // FP32 values of the mixed-precision sweeps, rounded to nearest
    std::vector<float> krf(krv[(size_t)p].begin(), krv[(size_t)p].end());
    std::vector<float> kcf(q.k_csc.val, q.k_csc.val + q.k_csc.nnz);
    if ((rc = upload(mp, &kr_ptr, kr[(size_t)p].data(), kr[(size_t)p].size())) ||
        (rc = upload(mp, &kr_idx, kri[(size_t)p].data(), kri[(size_t)p].size())) ||
        (rc = upload(mp, &kr_val, krv[(size_t)p].data(), krv[(size_t)p].size())) ||
        (rc = upload(mp, &kc_ptr, kc[(size_t)p].data(), kc[(size_t)p].size())) ||
        (rc = upload(mp, &kc_idx, q.k_csc.idx, (size_t)q.k_csc.nnz)) ||
        (rc = upload(mp, &kc_val, q.k_csc.val, (size_t)q.k_csc.nnz)) ||
        (rc = upload(mp, &dr_ptr, dr[(size_t)p].data(), dr[(size_t)p].size())) ||
        (rc = upload(mp, &dr_idx, q.d_csr.idx, (size_t)q.d_csr.nnz)) ||
        (rc = upload(mp, &dr_val, q.d_csr.val, (size_t)q.d_csr.nnz)) ||
        (rc = upload(mp, &dc_ptr, dc[(size_t)p].data(), dc[(size_t)p].size())) ||
        (rc = upload(mp, &dc_idx, q.d_csc.idx, (size_t)q.d_csc.nnz)) ||
        (rc = upload(mp, &dc_val, q.d_csc.val, (size_t)q.d_csc.nnz)) ||
        (rc = upload(mp, &korder, ko.data(), ko.size())) ||
        (rc = upload(mp, &kpart, kp.data(), kp.size())) ||
        (rc = upload(mp, &cpart, cp.data(), cp.size())) ||
        (rc = upload(mp, &b, q.b_k, (size_t)m_k)) ||
        (rc = upload<double>(mp, &u, nullptr, (size_t)m)) ||
        (rc = upload<double>(mp, &v, nullptr, (size_t)n)) ||
        (rc = upload<double>(mp, &w, nullptr, (size_t)n)) ||
        (rc = upload<double>(mp, &x, nullptr, (size_t)n)) ||
        (rc = upload<double>(mp, &dx, nullptr, (size_t)n)) ||
        (rc = upload(mp, &kr_val32, krf.data(), krf.size())) ||
        (rc = upload(mp, &kc_val32, kcf.data(), kcf.size())) ||
        (rc = upload<float2>(mp, &uhl, nullptr, (size_t)m_k)) ||
        (rc = upload<float2>(mp, &vhl, nullptr, (size_t)n)))
      return rc;
    d.kr_ptr = kr_ptr, d.kr_idx = kr_idx, d.kr_val = kr_val;
    d.kc_ptr = kc_ptr, d.kc_idx = kc_idx, d.kc_val = kc_val;
    d.dr_ptr = dr_ptr, d.dr_idx = dr_idx, d.dr_val = dr_val;
    d.dc_ptr = dc_ptr, d.dc_idx = dc_idx, d.dc_val = dc_val;
    d.korder = korder, d.kpart = kpart, d.cpart = cpart;
    d.b = b, d.u = u, d.v = v, d.w = w, d.x = x;
    d.kr_val32 = kr_val32, d.kc_val32 = kc_val32, d.uhl = uhl, d.vhl = vhl;
    d.dx = dx;
    d.m_k = m_k, d.m_d = m_d, d.n = n, d.iters = q.lsqr_iteration, d.itnlim = q.itnlim;
    d.damp = q.damp, d.atol = q.atol, d.btol = q.btol;
    d.ctol = q.conlim > 0.0 ? 1.0 / q.conlim : 0.0;
    mp->hist_off[(size_t)p] = mp->hist_total;
    mp->hist_total += (int64_t)q.lsqr_iteration + 1;
    mp->x_total += n;
    kr[(size_t)p].clear(), kr[(size_t)p].shrink_to_fit();
    kri[(size_t)p].clear(), kri[(size_t)p].shrink_to_fit();
    krv[(size_t)p].clear(), krv[(size_t)p].shrink_to_fit();
  }
  if ((rc = upload<plsqr_iter>(mp, &mp->d_hist, nullptr, (size_t)mp->hist_total))) return rc;
  for (int p = 0; p < P; ++p) mp->desc[(size_t)p].hist = mp->d_hist + mp->hist_off[(size_t)p];
  if ((rc = upload(mp, &mp->d_probs, mp->desc.data(), mp->desc.size())) ||
      (rc = upload(mp, &mp->d_groups, groups.data(), groups.size())) ||
      (rc = upload(mp, &mp->d_queue, queue.data(), queue.size())) ||
      (rc = upload(mp, &mp->d_block_group, block_group.data(), block_group.size())) ||
      (rc = upload<unsigned int>(mp, &mp->d_bars, nullptr, groups.size())) ||
      ((mp->n_bars = (int)groups.size()), false) ||
      (rc = upload<unsigned int>(mp, &mp->d_zero, nullptr, 1)) ||
      (rc = upload<double>(mp, &mp->d_parts, nullptr, (size_t)3 * mp->blocks)) ||
      (rc = upload<DevState>(mp, &mp->d_out, nullptr, (size_t)P)) ||
      (rc = upload<int>(mp, &mp->d_err, nullptr, 1)))
    return rc;
  MK(cudaMemset(mp->d_zero, 0, sizeof(unsigned int)));
  MK(cudaMemset(mp->d_err, 0, sizeof(int)));
  return PLSQR_OK;
}

extern "C" int plsqr_multi_create(const plsqr_problem *probs, int32_t count,
                                  const plsqr_opts *opts, plsqr_multi **out) {
  if (!out || !probs || count < 1 || count > (1 << 20)) return PLSQR_ERR_ARG;
  *out = nullptr;
  int32_t ndev = 0;
  plsqr_device_count(&ndev);
  plsqr_opts o;
  plsqr_default_opts(&o);
  if (opts) o = *opts;
  if (ndev < 1 || o.device < 0 || o.device >= ndev) return PLSQR_ERR_NODEV;
  plsqr_multi *mp = new plsqr_multi();
  mp->opts = o;
  mp->count = count;
  const int rc = multi_build(mp, probs);
  if (rc) {
    plsqr_multi_destroy(mp);
    return rc;
  }
  *out = mp;
  return PLSQR_OK;
}

extern "C" int plsqr_multi_info_get(const plsqr_multi *mp, plsqr_multi_info *info) {
  if (!mp || !info) return PLSQR_ERR_ARG;
  memset(info, 0, sizeof(*info));
  info->count = mp->count;
  info->blocks = mp->blocks;
  info->groups = (int32_t)mp->group_blocks.size();
  info->blocks_per_sm = mp->blocks_per_sm;
  info->device_bytes = mp->device_bytes;
  info->wait_ns = mp->wait_ns;
  info->seconds = mp->seconds;
  return PLSQR_OK;
}

extern "C" int plsqr_multi_plan(const plsqr_multi *mp, int32_t *group, int32_t *group_blocks) {
  if (!mp) return PLSQR_ERR_ARG;
  for (int p = 0; p < mp->count; ++p) {
    if (group) group[p] = mp->group_of[(size_t)p];
    if (group_blocks)
      group_blocks[p] = p < (int)mp->group_blocks.size() ? mp->group_blocks[(size_t)p] : 0;
  }
  return PLSQR_OK;
}

extern "C" int plsqr_multi_set_wait(plsqr_multi *mp, int64_t wait_ns) {
  if (!mp || wait_ns < 1000) return PLSQR_ERR_ARG;
  mp->wait_ns = wait_ns;
  return PLSQR_OK;
}

extern "C" int plsqr_multi_set_exact(plsqr_multi *mp, int32_t exact) {
  if (!mp || (exact != 0 && exact != 1)) return PLSQR_ERR_ARG;
  if (exact && mp->sweeps) {
    set_error(mp, "exact products are FP64: turn mixed precision off first");
    return PLSQR_ERR_ARG;
  }
  mp->exact = exact;
  return PLSQR_OK;
}

extern "C" int plsqr_multi_set_mixed(plsqr_multi *mp, int32_t sweeps) {
  if (!mp || sweeps < 0 || sweeps > 64) return PLSQR_ERR_ARG;
  if (sweeps && mp->exact) {
    set_error(mp, "mixed precision needs the default (non-exact) products");
    return PLSQR_ERR_ARG;
  }
  mp->sweeps = sweeps;
  return PLSQR_OK;
}

extern "C" int plsqr_multi_solve(plsqr_multi *mp, double *x, plsqr_iter *hist,
                                 plsqr_result *res) {
  if (!mp) return PLSQR_ERR_ARG;
  MK(cudaSetDevice(mp->opts.device));
  cudaStream_t s = mp->stream;
  MK(cudaMemsetAsync(mp->d_bars, 0, sizeof(unsigned int) * mp->n_bars, s));
  MK(cudaMemsetAsync(mp->d_err, 0, sizeof(int), s));
  MK(cudaMemsetAsync(mp->d_hist, 0, sizeof(plsqr_iter) * mp->hist_total, s));
  long long wait = mp->wait_ns;
  int sweeps = mp->sweeps;
  void *args[] = {&mp->d_probs, &mp->d_groups, &mp->d_queue, &mp->d_block_group,
                  &mp->d_bars,  &mp->d_parts,  &mp->d_out,   &mp->d_err,
                  &wait,        &sweeps};
  const void *kern = sweeps      ? (const void *)k_multi_lsqr<false, true>
                     : mp->exact ? (const void *)k_multi_lsqr<true, false>
                                 : (const void *)k_multi_lsqr<false, false>;
  MK(cudaEventRecord(mp->ev0, s));
  MK(cudaLaunchCooperativeKernel(kern, dim3(mp->blocks), dim3(kMT), args, 0, s));
  MK(cudaEventRecord(mp->ev1, s));
  MK(cudaEventSynchronize(mp->ev1));
  float ms = 0.f;
  MK(cudaEventElapsedTime(&ms, mp->ev0, mp->ev1));
  mp->seconds = ms * 1e-3;
  int err = 0;
  MK(cudaMemcpy(&err, mp->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    set_error(mp, "a group barrier wait gave up after %lld ns", (long long)mp->wait_ns);
    return err;
  }
  if (x) {
    int64_t off = 0;
    for (int p = 0; p < mp->count; ++p) {
      MK(cudaMemcpyAsync(x + off, mp->desc[(size_t)p].x, sizeof(double) * mp->n[(size_t)p],
                         cudaMemcpyDeviceToHost, s));
      off += mp->n[(size_t)p];
    }
  }
  if (hist)
    MK(cudaMemcpyAsync(hist, mp->d_hist, sizeof(plsqr_iter) * mp->hist_total,
                       cudaMemcpyDeviceToHost, s));
  std::vector<DevState> st((size_t)mp->count);
  MK(cudaMemcpyAsync(st.data(), mp->d_out, sizeof(DevState) * mp->count, cudaMemcpyDeviceToHost,
                     s));
  MK(cudaStreamSynchronize(s));
  if (res)
    for (int p = 0; p < mp->count; ++p) {
      const DevState &c = st[(size_t)p];
      plsqr_result &r = res[p];
      memset(&r, 0, sizeof(r));
      r.istop = c.istop;
      r.itn = c.itn;
      r.anorm = c.anorm;
      r.acond = c.acond;
      r.rnorm = c.rnorm;
      r.arnorm_out = c.test2;
      r.xnorm = c.xnorm;
      r.arnorm = c.arnorm;
      r.bnorm = c.bnorm;
      r.dxmax = c.dxmax;
      r.maxdx = c.maxdx;
      r.seconds = mp->seconds;
      r.seconds_total = mp->seconds;
    }
  return PLSQR_OK;
}

extern "C" int plsqr_multi_check_wait(plsqr_multi *mp, int64_t wait_ns) {
  if (!mp || wait_ns < 1000 || wait_ns > 10000000000LL) return PLSQR_ERR_ARG;
  MK(cudaSetDevice(mp->opts.device));
  MK(cudaMemsetAsync(mp->d_err, 0, sizeof(int), mp->stream));
  k_check_wait<<<1, 32, 0, mp->stream>>>(mp->d_zero, mp->d_err, (long long)wait_ns);
  MK(cudaGetLastError());
  int err = 0;
  MK(cudaMemcpyAsync(&err, mp->d_err, sizeof(int), cudaMemcpyDeviceToHost, mp->stream));
  MK(cudaStreamSynchronize(mp->stream));
  MK(cudaMemsetAsync(mp->d_err, 0, sizeof(int), mp->stream));
  MK(cudaStreamSynchronize(mp->stream));
  return err;
}

extern "C" int plsqr_multi_plan_host(const double *bytes, const int32_t *iters, int32_t count,
                                     int32_t blocks, double bw_block, int32_t *group,
                                     int32_t *group_blocks, int32_t *n_groups) {
  if (!bytes || !iters || count < 1 || blocks < 1 || !(bw_block > 0.0) || !group ||
      !group_blocks || !n_groups)
    return PLSQR_ERR_ARG;
  std::vector<double> b(bytes, bytes + count);
  std::vector<int32_t> it(iters, iters + count), g, nb;
  std::vector<std::vector<int32_t>> q;
  plan(b, it, blocks, bw_block, g, nb, q);
  for (int p = 0; p < count; ++p) group[p] = g[(size_t)p];
  for (size_t i = 0; i < nb.size(); ++i) group_blocks[i] = nb[i];
  *n_groups = (int32_t)nb.size();
  return PLSQR_OK;
}
