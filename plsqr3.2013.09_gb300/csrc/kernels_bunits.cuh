// k-wide products of the batched solver on the unit layout (units.cuh, built
// with lane_lines): passes over KW = 4 or 8 columns of the block (a block of
// 16 or 32 right-hand sides in passes of 8).
//
// The team form (kernels_batched.cuh) streams the matrix as int32 index +
// FP32 value (8 bytes a nonzero) and gathers 4*KW bytes of the block's row
// from L2 for every nonzero; for narrow blocks that leaves the product far
// from the matrix stream (a block of 4: 8.7 ms an iteration on the 96x96x32
// problem, against 2.55 ms for one right-hand side on the unit layout).
// Here the block's FP32 rows of one slab (6,144 rows: 192 KB for KW = 8) are
// staged in shared memory, the matrix is read as 16-bit slab-local index +
// FP32 value (6 bytes), and lane j of a warp streams line j of its unit, so
// every lane keeps its own KW sums and writes them once:
//
//   partial[(s * n_lines + l) * KW + j] = sum over segment (s, l) of val * X[idx][j]
//
// Each step's 8 products are summed in FP32 per column and added to the
// line's running sum with the error-free two-sum (hi + lo), as in the team
// form; the combine kernels add the slabs' partials in slab order in FP64.
#pragma once

#include "kernels_batched.cuh"
#include "units.cuh"

namespace plsqr {

constexpr int kBUnitThreads = 1024;
constexpr int kBUnitSlab = 6144;  // rows of the block per slab: 192 KB at KW = 8

template <int KW>
__global__ void __launch_bounds__(kBUnitThreads, 1)
    k_bunits(UnitsArgs<float> A, int *__restrict__ next, const float *__restrict__ xf, int kp,
             int col0, double *__restrict__ partial) {
  static_assert(KW == 4 || KW == 8, "passes of 4 or 8 columns");
  constexpr int V4 = KW / 4;  // float4 pieces of a row
  constexpr int P = UnitPieces<float>::P;
  extern __shared__ __align__(16) float4 xs4[];
  __shared__ int s_left;
  const int lane = threadIdx.x & 31;
  const uint4 *idx8 = reinterpret_cast<const uint4 *>(A.idx);
  const uint4 *val16 = reinterpret_cast<const uint4 *>(A.val);
  const int plane = min(A.slab, A.n_idx);  // rows of the staged slab's planes
  int s = (int)(((int64_t)blockIdx.x * A.n_slabs) / gridDim.x);
  for (int visit = 0; visit < A.n_slabs; ++visit, s = (s + 1 == A.n_slabs) ? 0 : s + 1) {
    const int u0 = A.unit_begin[s], nu = A.unit_begin[s + 1] - u0;
    if (threadIdx.x == 0) s_left = *reinterpret_cast<volatile int *>(next + s) < nu;
    __syncthreads();
    const bool left = s_left;  // the same decision in every thread of the block
    __syncthreads();           // read before thread 0 writes the next slab's
    if (!left) continue;
    const int64_t xbase = (int64_t)s * A.slab;
    const int len = (int)min((int64_t)A.slab, (int64_t)A.n_idx - xbase);
    // columns col0 .. col0 + KW - 1 of the block xf[n_idx][kp]; piece t of
    // row r at xs4[t * plane + r]: a wavefront's random rows then spread over
    // all 8 groups of 4 banks (rows of 32 bytes side by side would start on
    // only 4 of them)
    const float4 *src = reinterpret_cast<const float4 *>(xf + xbase * kp + col0);
    for (int i = threadIdx.x; i < len * V4; i += kBUnitThreads)
      xs4[(i % V4) * plane + i / V4] = __ldg(src + (int64_t)(i / V4) * (kp / 4) + i % V4);
    __syncthreads();
    double *part = partial + (int64_t)s * A.n_lines * KW;
    for (;;) {
      int u = 0;
      if (lane == 0) u = atomicAdd(next + s, 1);
      u = __shfl_sync(0xffffffffu, u, 0);
      if (u >= nu) break;
      u += u0;
      const int q = A.q[u];
      const int64_t base = A.slot0[u];
      const int l = A.line[(int64_t)u * kUnitLines + lane];
      chk(base + (int64_t)q * 32 <= A.n_slots, kChkSlot);
      float hi[KW], lo[KW];
#pragma unroll
      for (int j = 0; j < KW; ++j) hi[j] = lo[j] = 0.f;
      for (int k = 0; k < q; ++k) {
        const int kp = k + A.pf_dist;
        if (A.pf_dist > 0 && kp < q) {  // a later step into L2
          asm volatile("prefetch.global.L2 [%0];" ::"l"(idx8 + base + (int64_t)kp * 32 + lane));
          for (int pc = 0; pc < A.pf_pieces; ++pc)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(val16 + base * P +
                                                          (int64_t)(kp * P + pc) * 32 + lane));
        }
        if (!chk(base + (int64_t)k * 32 + lane < A.n_slots, kChkSlot)) continue;
        const uint4 g = __ldg(idx8 + base + (int64_t)k * 32 + lane);
        float v[8];
        unit_vals(A.val, base, k, lane, v);
        if (!chk(group_in(g, len), kChkGather)) continue;
        const unsigned id[8] = {g.x & 0xffffu, g.x >> 16, g.y & 0xffffu, g.y >> 16,
                                g.z & 0xffffu, g.z >> 16, g.w & 0xffffu, g.w >> 16};
        float c[KW];
#pragma unroll
        for (int j = 0; j < KW; ++j) c[j] = 0.f;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
#pragma unroll
          for (int t = 0; t < V4; ++t) {
            const float4 x = xs4[t * plane + id[e]];
            c[4 * t] = fmaf(v[e], x.x, c[4 * t]);
            c[4 * t + 1] = fmaf(v[e], x.y, c[4 * t + 1]);
            c[4 * t + 2] = fmaf(v[e], x.z, c[4 * t + 2]);
            c[4 * t + 3] = fmaf(v[e], x.w, c[4 * t + 3]);
          }
        }
#pragma unroll
        for (int j = 0; j < KW; ++j) two_sum_add(hi[j], lo[j], c[j]);
      }
      if (l >= 0 && chk(l < A.n_lines, kChkLine)) {
        double2 *p = reinterpret_cast<double2 *>(part + (int64_t)l * KW);
#pragma unroll
        for (int j = 0; j < KW; j += 2)
          p[j / 2] = make_double2((double)hi[j] + (double)lo[j],
                                  (double)hi[j + 1] + (double)lo[j + 1]);
      }
    }
    __syncthreads();  // every warp is done with the slab before the next is staged
  }
}

// A x of the units form, columns col0 .. col0 + KW - 1 of the block
// u[m][kp]: U_k[r][j] = s_j U_k[r][j] + the sum of partial[s][r][j - col0]
// over the slabs in slab order, and the damping rows U_d[r][j] = s_j
// U_d[r][j] + lambda_j (D V)[r][j] in FP64, in one grid-stride pass; sums of
// squares to parts[block * kp + j]; with `finish` (the block's last pass) the
// last block forms every beta_j (rows_finish).
template <int KW>
__global__ void __launch_bounds__(kBatchThreads)
    k_bunits_rows(const double *__restrict__ partial, int n_slabs, int m_k, Csr D, int k, int kp,
                  int col0, const double *__restrict__ v64, double *__restrict__ u,
                  const double *__restrict__ lambda, int mode, DevState *__restrict__ st,
                  BatchCoef *__restrict__ cf, double *__restrict__ parts, int finish) {
  __shared__ double red[kBatchThreads];
  // each thread keeps one right-hand side: the block and the grid stride
  // are multiples of KW
  const int j = col0 + (threadIdx.x & (KW - 1));
  const double sc = (j < k && mode == kScaleNegAlpha) ? -st[j].alpha : 1.0;
  const double lam = (j < k && lambda) ? lambda[j] : 1.0;
  const int64_t tk = (int64_t)m_k * KW, total = tk + (int64_t)D.n_lines * KW;
  double sq = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kBatchThreads + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * kBatchThreads) {
    const int64_t r = i / KW;  // a row of [K; D]
    double a;
    if (i < tk) {
      a = 0.0;
      for (int sl = 0; sl < n_slabs; ++sl) a += __ldcs(partial + (int64_t)sl * tk + i);
    } else {
      double t = 0.0;
      for (int64_t e = D.ptr[r - m_k]; e < D.ptr[r - m_k + 1]; ++e)
        t = fma(D.val[e], v64[(int64_t)D.idx[e] * kp + j], t);
      a = dmul(lam, t);
    }
    if (j < k) {
      double *p = u + r * kp + j;
      const double y = dadd(dmul(sc, *p), a);
      *p = y;
      sq = fma(y, y, sq);
    }
  }
  const double b = batch_block_sum(sq, KW, red);
  if ((int)threadIdx.x < KW) parts[(int64_t)blockIdx.x * kp + col0 + threadIdx.x] = b;
  if (!finish || !batch_last_block(&cf->count)) return;
  rows_finish(parts, gridDim.x, kp, k, mode, st, cf);
}

// A^T y of the units form, columns col0 .. col0 + KW - 1 of the block
// v[n][kp]: V[c][j] = s_j V[c][j] + (the slabs' partials in slab order) +
// lambda_j (D^T U_d)[c][j], FP64; with `finish` the last block finishes the
// product (cols_finish), as k_bslab_cols does.
template <int KW>
__global__ void __launch_bounds__(kBatchThreads)
    k_bunits_cols(const double *__restrict__ partial, int n_slabs, Csr DC, int m_k, int n,
                  int k, int kp, int col0, const double *__restrict__ u64,
                  double *__restrict__ v, const double *__restrict__ lambda, int mode,
                  DevState *__restrict__ st, BatchCoef *__restrict__ cf,
                  double *__restrict__ parts, int finish) {
  __shared__ double red[kBatchThreads];
  const int j = col0 + (threadIdx.x & (KW - 1));
  double sc = 1.0;
  bool act = j < k;
  if (act && (mode == kScaleNegBeta || mode == kScaleZero)) {
    act = st[j].s_beta_pos && !(mode == kScaleNegBeta && st[j].done);
    sc = mode == kScaleZero ? 0.0 : -st[j].beta;
  }
  const double lam = (j < k && lambda) ? lambda[j] : 1.0;
  const double *ud = u64 + (int64_t)m_k * kp;
  const int64_t total = (int64_t)n * KW;
  double sq = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kBatchThreads + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * kBatchThreads) {
    const int64_t c = i / KW;
    double a = 0.0;
    for (int sl = 0; sl < n_slabs; ++sl) a += __ldcs(partial + (int64_t)sl * total + i);
    double d = 0.0;
    for (int64_t e = DC.ptr[c]; e < DC.ptr[c + 1]; ++e)
      d = fma(DC.val[e], ud[(int64_t)DC.idx[e] * kp + j], d);
    if (act) {
      double *p = v + c * kp + j;
      const double y = dadd(dmul(sc, *p), dadd(a, dmul(lam, d)));
      *p = y;
      sq = fma(y, y, sq);
    }
  }
  const double b = batch_block_sum(sq, KW, red);
  if ((int)threadIdx.x < KW) parts[(int64_t)blockIdx.x * kp + col0 + threadIdx.x] = b;
  if (!finish || !batch_last_block(&cf->count)) return;
  cols_finish(parts, gridDim.x, kp, k, mode, st, cf);
}

}  // namespace plsqr
