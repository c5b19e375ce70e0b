// Slab layout of the kernel matrix and the products built on it.
//
// A product gathers a vector (v for A x, u_k for A^T y) at the matrix's
// indices.  The index space is cut into slabs of S entries that fit in shared
// memory (S = 24,576 FP64 values = 192 KB).  Every line (row for A x, column
// for A^T y) is stored slab by slab: the entries of line l whose index falls
// in slab s form the segment (s, l), with a 16-bit slab-local index, padded
// with zero entries to a multiple of 8 so that a lane loads 8 indices and their
// values with 16-byte loads.  Segments are stored slab-major:
//
//   ptr[s * (n_lines + 1) + l]   start of segment (s, l) in idx / val
//   idx[e]  uint16, val[e]  T    entries (10 bytes per FP64 nonzero, 6 per FP32)
//
// k_slab_spmv: block b works on slab s = b / B: it copies x[s*S, (s+1)*S) into
// shared memory once, then its warps stream the segments of a contiguous,
// nonzero-balanced range of lines and write partial[s][l].  The gathers hit
// shared memory instead of scattering over L2.  k_combine_rows /
// k_combine_cols add the partials of the slabs in slab order (so results are
// deterministic), add the damping part, apply the LSQR scale and write the
// per-block sums of squares the norm kernels finish.
#pragma once

#include "kernels_fp64.cuh"

namespace plsqr {

template <typename T>
struct SlabCsr {
  const int64_t *ptr;   // [n_slabs * (n_lines + 1)]
  const int32_t *order; // [n_slabs * n_lines] lines of each block range, longest segment first
  const uint16_t *idx;  // slab-local indices
  const T *val;
  int32_t n_lines;      // lines (rows for A x, columns for A^T y)
  int32_t n_slabs;
  int32_t slab;         // S
  int32_t n_idx;        // length of the gathered vector
};

// ---- construction (setup only) --------------------------------------------

// cnt[s * n_lines + l] = entries of line l in slab s, rounded up to 8.
static __global__ void k_slab_count(const int64_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                                    int n_lines, int n_slabs, int slab, int64_t *__restrict__ cnt) {
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n_lines; l += gridDim.x * blockDim.x) {
    int64_t c[64];
    for (int s = 0; s < n_slabs; ++s) c[s] = 0;
    for (int64_t e = ptr[l]; e < ptr[l + 1]; ++e) c[idx[e] / slab]++;
    for (int s = 0; s < n_slabs; ++s) cnt[(int64_t)s * n_lines + l] = (c[s] + 7) & ~int64_t(7);
  }
}

// Stored position of the segment's entry o (segment length len, a multiple
// of 8) when a product streams the segment with tgroup lanes: each chunk of
// tgroup groups of 8 (ng groups in a shorter last chunk) is transposed so
// that lane l's group holds the chunk's entries l, l + ng, l + 2 ng, ....
// At every step of the product the group's lanes then read consecutive
// entries: for a kernel row, mostly consecutive columns, which fall in
// distinct shared-memory banks.  tgroup <= 1 keeps the order.
__host__ __device__ __forceinline__ int64_t slab_pos(int64_t o, int64_t len, int tgroup) {
  if (tgroup <= 1) return o;
  const int64_t cw = (int64_t)tgroup * 8, c0 = (o / cw) * cw;
  const int64_t ng = (len - c0) / 8 < tgroup ? (len - c0) / 8 : tgroup;
  const int64_t w = o - c0;
  return c0 + (w % ng) * 8 + w / ng;
}

// Scatter line l's entries into its segments; pad with (index 0, value 0).
template <typename T>
__global__ void k_slab_fill(const int64_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                            const double *__restrict__ val, int n_lines, int n_slabs, int slab,
                            const int64_t *__restrict__ sptr, int tgroup,
                            uint16_t *__restrict__ sidx, T *__restrict__ sval) {
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n_lines; l += gridDim.x * blockDim.x) {
    int64_t cur[64];
    for (int s = 0; s < n_slabs; ++s) cur[s] = 0;
    for (int64_t e = ptr[l]; e < ptr[l + 1]; ++e) {
      const int s = idx[e] / slab;
      const int64_t b = sptr[(int64_t)s * (n_lines + 1) + l];
      const int64_t o = b + slab_pos(cur[s]++, sptr[(int64_t)s * (n_lines + 1) + l + 1] - b, tgroup);
      sidx[o] = (uint16_t)(idx[e] - s * slab);
      sval[o] = (T)val[e];
    }
    for (int s = 0; s < n_slabs; ++s) {
      const int64_t b = sptr[(int64_t)s * (n_lines + 1) + l];
      const int64_t len = sptr[(int64_t)s * (n_lines + 1) + l + 1] - b;
      for (int64_t o = cur[s]; o < len; ++o) {
        const int64_t q = b + slab_pos(o, len, tgroup);
        sidx[q] = 0;
        sval[q] = (T)0;
      }
    }
  }
}

// ---- products -----------------------------------------------------------------

__device__ __forceinline__ void load8(const double *v, int64_t g, double (&o)[8]) {
  const double2 *p = reinterpret_cast<const double2 *>(v) + 4 * g;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const double2 a = __ldg(p + j);
    o[2 * j] = a.x;
    o[2 * j + 1] = a.y;
  }
}
__device__ __forceinline__ void load8(const float *v, int64_t g, float (&o)[8]) {
  const float4 *p = reinterpret_cast<const float4 *>(v) + 2 * g;
  const float4 a = __ldg(p), b = __ldg(p + 1);
  o[0] = a.x;
  o[1] = a.y;
  o[2] = a.z;
  o[3] = a.w;
  o[4] = b.x;
  o[5] = b.y;
  o[6] = b.z;
  o[7] = b.w;
}

// partial[s * n_lines + l] = sum over segment (s, l) of val * x_slab[idx].
// Blocks are slab-major: slab s = blockIdx.x / bps, range r = blockIdx.x % bps;
// lpart[s * (bps + 1) + r] .. [.. + 1] is the range's first and end line.  A
// group of kGroup lanes streams one segment (each lane one 16-byte group of 8
// indices per step) and reduces it in log2(kGroup) shuffles, so that a short
// segment does not pay a full 5-step warp reduction on the FP64 pipe.
// FP32 slabs are 96 KB, so two blocks share an SM: the register budget must
// allow it (32 registers per thread at 1024 threads).  That budget leaves no
// room for deeper software pipelining, so each lane also prefetches its
// indices and values of the step after next into L2 (no registers): the
// FP32 products 1.57 -> 1.44 ms (A x) and 1.52 -> 1.39 ms (A^T y), the FP64
// A^T y 2.86 -> 2.81 ms on the 96x96x32 problem (three steps ahead, and the
// same prefetch in the per-row A x kernel, measured slower).
template <typename T, int kThreads, int kGroup>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1)
    k_slab_spmv(SlabCsr<T> A, const int32_t *__restrict__ lpart, int bps, const T *__restrict__ x,
                T *__restrict__ partial) {
  static_assert(kGroup == 4 || kGroup == 8 || kGroup == 16 || kGroup == 32, "4 to 32 lanes");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *xs = reinterpret_cast<T *>(smem_raw);
  const int s = blockIdx.x / bps, r = blockIdx.x - s * bps;
  const int64_t base = (int64_t)s * A.slab;
  const int len = (int)min((int64_t)A.slab, (int64_t)A.n_idx - base);
  for (int i = threadIdx.x; i < len; i += kThreads) xs[i] = x[base + i];
  __syncthreads();
  const int sub = threadIdx.x & (kGroup - 1);        // lane within the group
  const int grp = threadIdx.x / kGroup;              // group within the block
  constexpr int kGroups = kThreads / kGroup;
  const int64_t *ptr = A.ptr + (int64_t)s * (A.n_lines + 1);
  const int l1 = lpart[s * (bps + 1) + r + 1];
  const uint4 *idx8 = reinterpret_cast<const uint4 *>(A.idx);
  const int32_t *order = A.order + (int64_t)s * A.n_lines;
  // The lines of the range are visited longest segment first, so the groups
  // of a warp walk segments of about the same length.  Every group runs the
  // same number of loop trips so the shuffles below see their whole group.
  const int l0 = lpart[s * (bps + 1) + r];
  for (int lb = l0; lb < l1; lb += kGroups) {
    const int k = lb + grp;
    const int l = k < l1 ? order[k] : 0;
    T acc0 = 0, acc1 = 0;
    if (k < l1) {
      const int64_t g0 = ptr[l] >> 3, g1 = ptr[l + 1] >> 3;  // groups of 8 entries
      int64_t g = g0 + sub;
      // two steps in flight; the FP32 build spills a few values at its 32
      // registers per thread and still measured faster than one step
      for (; g + kGroup < g1; g += 2 * kGroup) {
        if (g + 4 * kGroup < g1) {  // the step after next into L2
          asm volatile("prefetch.global.L2 [%0];" ::"l"(idx8 + g + 4 * kGroup));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(A.val + (g + 4 * kGroup) * 8));
        }
        const uint4 q = __ldg(idx8 + g), p = __ldg(idx8 + g + kGroup);
        T v[8], w[8];
        load8(A.val, g, v);
        load8(A.val, g + kGroup, w);
        acc0 = fmaT(v[0], xs[q.x & 0xffff], acc0);
        acc1 = fmaT(v[1], xs[q.x >> 16], acc1);
        acc0 = fmaT(v[2], xs[q.y & 0xffff], acc0);
        acc1 = fmaT(v[3], xs[q.y >> 16], acc1);
        acc0 = fmaT(v[4], xs[q.z & 0xffff], acc0);
        acc1 = fmaT(v[5], xs[q.z >> 16], acc1);
        acc0 = fmaT(v[6], xs[q.w & 0xffff], acc0);
        acc1 = fmaT(v[7], xs[q.w >> 16], acc1);
        acc0 = fmaT(w[0], xs[p.x & 0xffff], acc0);
        acc1 = fmaT(w[1], xs[p.x >> 16], acc1);
        acc0 = fmaT(w[2], xs[p.y & 0xffff], acc0);
        acc1 = fmaT(w[3], xs[p.y >> 16], acc1);
        acc0 = fmaT(w[4], xs[p.z & 0xffff], acc0);
        acc1 = fmaT(w[5], xs[p.z >> 16], acc1);
        acc0 = fmaT(w[6], xs[p.w & 0xffff], acc0);
        acc1 = fmaT(w[7], xs[p.w >> 16], acc1);
      }
      for (; g < g1; g += kGroup) {
        const uint4 q = __ldg(idx8 + g);
        T v[8];
        load8(A.val, g, v);
        acc0 = fmaT(v[0], xs[q.x & 0xffff], acc0);
        acc1 = fmaT(v[1], xs[q.x >> 16], acc1);
        acc0 = fmaT(v[2], xs[q.y & 0xffff], acc0);
        acc1 = fmaT(v[3], xs[q.y >> 16], acc1);
        acc0 = fmaT(v[4], xs[q.z & 0xffff], acc0);
        acc1 = fmaT(v[5], xs[q.z >> 16], acc1);
        acc0 = fmaT(v[6], xs[q.w & 0xffff], acc0);
        acc1 = fmaT(v[7], xs[q.w >> 16], acc1);
      }
    }
    T t = acc0 + acc1;
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (sub == 0 && k < l1) partial[(int64_t)s * A.n_lines + l] = t;
  }
}

// The same product as a persistent kernel: one block per SM slot; blocks
// take lines of a slab from the slab's counter in next[] (chunk * 32 / kGroup
// consecutive lines per warp and grab, a group's line per pass, in the slab's
// longest-segment-first order, A.order with one range per slab), so that
// every warp stays busy until the slab runs out; the block then stages the next slab that still has lines (counters
// shared by all blocks, so fast SMs take over the work of slow ones) and
// passes each slab once.  next[] is zeroed before every launch.  A
// segment's partial comes from one group whichever block takes it, with the
// same lanes and order: the results equal the static kernel's bit for bit.
template <typename T, int kThreads, int kGroup>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1)
    k_slab_spmv_dyn(SlabCsr<T> A, int *__restrict__ next, int chunk, const T *__restrict__ x,
                    T *__restrict__ partial) {
  static_assert(kGroup == 4 || kGroup == 8 || kGroup == 16 || kGroup == 32, "4 to 32 lanes");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *xs = reinterpret_cast<T *>(smem_raw);
  __shared__ int s_left;
  constexpr int kPerWarp = 32 / kGroup;
  const int lane = threadIdx.x & 31;
  const int sub = threadIdx.x & (kGroup - 1);
  const int gw = lane / kGroup;  // group within the warp
  const uint4 *idx8 = reinterpret_cast<const uint4 *>(A.idx);
  int s = (int)(((int64_t)blockIdx.x * A.n_slabs) / gridDim.x);
  for (int visit = 0; visit < A.n_slabs; ++visit, s = (s + 1 == A.n_slabs) ? 0 : s + 1) {
    if (threadIdx.x == 0) s_left = *reinterpret_cast<volatile int *>(next + s) < A.n_lines;
    __syncthreads();
    const bool left = s_left;  // the same decision in every thread of the block
    __syncthreads();           // read before thread 0 writes the next slab's
    if (!left) continue;
    const int64_t base = (int64_t)s * A.slab;
    const int len = (int)min((int64_t)A.slab, (int64_t)A.n_idx - base);
    for (int i = threadIdx.x; i < len; i += kThreads) xs[i] = x[base + i];
    __syncthreads();
    const int64_t *ptr = A.ptr + (int64_t)s * (A.n_lines + 1);
    const int32_t *order = A.order + (int64_t)s * A.n_lines;
    int k0 = 0, c = chunk;  // this warp's grab: lines [k0, k0 + chunk * kPerWarp)
    for (;;) {
      if (c == chunk) {
        if (lane == 0) k0 = atomicAdd(next + s, chunk * kPerWarp);
        k0 = __shfl_sync(0xffffffffu, k0, 0);
        c = 0;
      }
      if (k0 >= A.n_lines) break;
      const int k = k0 + gw;
      k0 += kPerWarp;
      ++c;
      const int l = k < A.n_lines ? order[k] : 0;
      T acc0 = 0, acc1 = 0;
      if (k < A.n_lines) {
        const int64_t g0 = ptr[l] >> 3, g1 = ptr[l + 1] >> 3;
        int64_t g = g0 + sub;
        for (; g + kGroup < g1; g += 2 * kGroup) {
          if (g + 4 * kGroup < g1) {
            asm volatile("prefetch.global.L2 [%0];" ::"l"(idx8 + g + 4 * kGroup));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(A.val + (g + 4 * kGroup) * 8));
          }
          const uint4 q = __ldg(idx8 + g), p = __ldg(idx8 + g + kGroup);
          T v[8], w[8];
          load8(A.val, g, v);
          load8(A.val, g + kGroup, w);
          acc0 = fmaT(v[0], xs[q.x & 0xffff], acc0);
          acc1 = fmaT(v[1], xs[q.x >> 16], acc1);
          acc0 = fmaT(v[2], xs[q.y & 0xffff], acc0);
          acc1 = fmaT(v[3], xs[q.y >> 16], acc1);
          acc0 = fmaT(v[4], xs[q.z & 0xffff], acc0);
          acc1 = fmaT(v[5], xs[q.z >> 16], acc1);
          acc0 = fmaT(v[6], xs[q.w & 0xffff], acc0);
          acc1 = fmaT(v[7], xs[q.w >> 16], acc1);
          acc0 = fmaT(w[0], xs[p.x & 0xffff], acc0);
          acc1 = fmaT(w[1], xs[p.x >> 16], acc1);
          acc0 = fmaT(w[2], xs[p.y & 0xffff], acc0);
          acc1 = fmaT(w[3], xs[p.y >> 16], acc1);
          acc0 = fmaT(w[4], xs[p.z & 0xffff], acc0);
          acc1 = fmaT(w[5], xs[p.z >> 16], acc1);
          acc0 = fmaT(w[6], xs[p.w & 0xffff], acc0);
          acc1 = fmaT(w[7], xs[p.w >> 16], acc1);
        }
        for (; g < g1; g += kGroup) {
          const uint4 q = __ldg(idx8 + g);
          T v[8];
          load8(A.val, g, v);
          acc0 = fmaT(v[0], xs[q.x & 0xffff], acc0);
          acc1 = fmaT(v[1], xs[q.x >> 16], acc1);
          acc0 = fmaT(v[2], xs[q.y & 0xffff], acc0);
          acc1 = fmaT(v[3], xs[q.y >> 16], acc1);
          acc0 = fmaT(v[4], xs[q.z & 0xffff], acc0);
          acc1 = fmaT(v[5], xs[q.z >> 16], acc1);
          acc0 = fmaT(v[6], xs[q.w & 0xffff], acc0);
          acc1 = fmaT(v[7], xs[q.w >> 16], acc1);
        }
      }
      T t = acc0 + acc1;
#pragma unroll
      for (int o = kGroup / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (sub == 0 && k < A.n_lines) partial[(int64_t)s * A.n_lines + l] = t;
    }
    __syncthreads();  // every warp is done with xs before the next slab is staged
  }
}

// u_k[r] = scale*u_k[r] + sum_s partial[s][r] (blocks [0, gk)); u_d[r] =
// scale*u_d[r] + (D v)[r] (blocks [gk, grid)); per-block sums of squares.
// P: type of the slab partials, T: type of the vectors (the mixed solver
// combines FP32 partials into FP64 vectors).
template <typename P, typename T, int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_combine_rows(const P *__restrict__ partial, int n_slabs, int m_k, Csr D,
                   const T *__restrict__ v, T *__restrict__ u, int gk, int mode,
                   const DevState *__restrict__ st, double *__restrict__ parts) {
  __shared__ double smem[kThreads / 32];
  double s = 1.0;
  if (mode == kScaleNegAlpha) s = -st->alpha;
  double sq = 0.0;
  if ((int)blockIdx.x < gk) {
    for (int r = blockIdx.x * kThreads + threadIdx.x; r < m_k; r += gk * kThreads) {
      T t = 0;
      for (int q = 0; q < n_slabs; ++q) t += (T)partial[(int64_t)q * m_k + r];
      const T y = scaled_add(s, u[r], t);
      u[r] = y;
      sq = fma((double)y, (double)y, sq);
    }
  } else {
    const int gd = gridDim.x - gk;
    T *ud = u + m_k;
    for (int r = (blockIdx.x - gk) * kThreads + threadIdx.x; r < D.n_lines; r += gd * kThreads) {
      const T y = scaled_add(s, ud[r], damp_row(D, v, r));
      ud[r] = y;
      sq = fma((double)y, (double)y, sq);
    }
  }
  const double b = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0 && parts) parts[blockIdx.x] = b;
}

// Damping column c times u_d in stored order (FP64: mul and add rounded apart
// as in CPUSpMV.c:270-275).
__device__ __forceinline__ double damp_col(const Csr &DC, const double *__restrict__ ud, int c) {
  return seq_dot_f64(DC.idx, DC.val, ud, DC.ptr[c], DC.ptr[c + 1]);
}
__device__ __forceinline__ float damp_col(const Csr &DC, const float *__restrict__ ud, int c) {
  float t = 0.f;
  for (int64_t e = DC.ptr[c]; e < DC.ptr[c + 1]; ++e) t = fmaf((float)DC.val[e], ud[DC.idx[e]], t);
  return t;
}

// v[c] = scale*v[c] + (sum_s partial[s][c] + (D^T u_d)[c]); per-block sums
// of squares.  LSQR mode: skipped when beta == 0 (source/lsqr.c:530).
template <typename P, typename T, int kThreads>
__global__ void __launch_bounds__(kThreads)
    k_combine_cols(const P *__restrict__ partial, int n_slabs, int n, Csr DC,
                   const T *__restrict__ u, int m_k, T *__restrict__ v, int mode,
                   const DevState *__restrict__ st, double *__restrict__ parts) {
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
  double sq = 0.0;
  for (int c = blockIdx.x * kThreads + threadIdx.x; c < n; c += gridDim.x * kThreads) {
    T t = 0;
    for (int q = 0; q < n_slabs; ++q) t += (T)partial[(int64_t)q * n + c];
    const T y = scaled_add(s, v[c], t + damp_col(DC, ud, c));  // x += (s_k + s_d)
    v[c] = y;
    sq = fma((double)y, (double)y, sq);
  }
  const double b = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0 && parts) parts[blockIdx.x] = b;
}

}  // namespace plsqr
