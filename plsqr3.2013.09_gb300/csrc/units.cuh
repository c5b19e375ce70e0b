// Unit layout of the kernel matrix, for the FP64 products on slabs.
//
// The slab layout (slab.cuh) hands each line's segment to a group of 8
// lanes; a segment of ~57 groups of 8 entries then leaves the group's last
// step partly empty, and on GB300, where the FP64 pipe binds this product, a
// warp instruction costs the pipe the same whether 32 or 25 of its lanes
// work (28.4 of 32 active on the 96x96x32 problem).  Here a warp takes a
// unit: 32 consecutive lines of a slab in longest-segment-first order.  The
// unit's stream is the concatenation of its lines' groups of 8 entries (G
// groups, each line's segment padded to a multiple of 8 entries, as in the
// slab layout); lane j streams groups [j*q, (j+1)*q), q = ceil(G / 32), so
// every lane works at every step but in the unit's last few slots.  Slot
// (k, j), lane j's k-th group, is stored at unit position k * 32 + j, so at
// every step the 32 lanes read 32 consecutive slots:
//
//   idx[(slot0 + k*32 + j) * 8 + e]              uint16, entry e of the group
//   val[(slot0*4 + (k*4 + p)*32 + j) * 2 + w]    FP64, entry e = 2p + w
//
// (four coalesced 16-byte loads of the values per step).  A lane sums its
// groups into the line they belong to; a line wholly inside one lane's run
// is written by that lane, and a line spread over lanes is summed by the
// unit's lane of the same index, from the lanes' parts in lane order, so the
// result is deterministic.  Units are taken from a per-slab counter by
// persistent blocks, as in k_slab_spmv_dyn.
#pragma once

#include "slab.cuh"

namespace plsqr {

constexpr int kUnitLines = 32;  // lines per unit: one per lane of the summing step

struct UnitsArgs {
  const uint16_t *idx;         // [slots * 8]
  const double *val;           // [slots * 8]
  const int64_t *slot0;        // [units] first slot of each unit
  const int32_t *q;            // [units] groups per lane
  const int32_t *c;            // [units * (kUnitLines + 1)] first group of each line in the unit's stream
  const int32_t *line;         // [units * kUnitLines] line index, -1 past the slab's last line
  const int32_t *unit_begin;   // [n_slabs + 1] first unit of each slab
  int32_t n_lines, n_slabs, slab, n_idx;
};

// Setup: entry o of segment (s, l) to its slot.  seg_unit / seg_pos give
// the unit of segment (s, l) and the line's position in it; the arrays were
// zeroed, so padding slots and entries stay (index 0, value 0).
static __global__ void k_units_fill(const int64_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                                    const double *__restrict__ val, int n_lines, int n_slabs,
                                    int slab, const int32_t *__restrict__ seg_unit,
                                    const int32_t *__restrict__ seg_pos, UnitsArgs U,
                                    uint16_t *__restrict__ sidx, double *__restrict__ sval) {
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n_lines; l += gridDim.x * blockDim.x) {
    int64_t cur[64];
    for (int s = 0; s < n_slabs; ++s) cur[s] = 0;
    for (int64_t e = ptr[l]; e < ptr[l + 1]; ++e) {
      const int s = idx[e] / slab;
      const int64_t o = cur[s]++;
      const int64_t sl = (int64_t)s * n_lines + l;
      const int u = seg_unit[sl], li = seg_pos[sl];
      const int64_t t = U.c[(int64_t)u * (kUnitLines + 1) + li] + o / 8;
      const int64_t q = U.q[u];
      const int64_t j = t / q, k = t - j * q;
      const int64_t base = U.slot0[u];
      const int w = (int)(o & 7);
      sidx[(base + k * 32 + j) * 8 + w] = (uint16_t)(idx[e] - s * slab);
      sval[(base * 4 + (k * 4 + w / 2) * 32 + j) * 2 + (w & 1)] = val[e];
    }
  }
}

// partial[s * n_lines + l] = sum over segment (s, l) of val * x_slab[idx].
// One block per SM (the 192 KB slab of x plus the summing area); the unit's
// loads for the step after next are prefetched into L2.
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 1)
    k_slab_units(UnitsArgs A, int *__restrict__ next, const double *__restrict__ x,
                 double *__restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *xs = reinterpret_cast<double *>(smem_raw);
  // per warp: each lane's first and last line and its sums for them, after
  // the slab (min(slab, n_idx) entries: the size the launch gives)
  double *pf_all = xs + min(A.slab, A.n_idx);
  double *pl_all = pf_all + kThreads;
  int *lf_all = reinterpret_cast<int *>(pl_all + kThreads);
  int *ll_all = lf_all + kThreads;
  __shared__ int s_left;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *pf = pf_all + warp * 32, *pl = pl_all + warp * 32;
  int *lf = lf_all + warp * 32, *ll = ll_all + warp * 32;
  const uint4 *idx8 = reinterpret_cast<const uint4 *>(A.idx);
  const double2 *val2 = reinterpret_cast<const double2 *>(A.val);
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
    for (int i = threadIdx.x; i < len; i += kThreads) xs[i] = x[xbase + i];
    __syncthreads();
    double *part = partial + (int64_t)s * A.n_lines;
    for (;;) {
      int u = 0;
      if (lane == 0) u = atomicAdd(next + s, 1);
      u = __shfl_sync(0xffffffffu, u, 0);
      if (u >= nu) break;
      u += u0;
      const int q = A.q[u];
      const int64_t base = A.slot0[u];
      const int32_t *c = A.c + (int64_t)u * (kUnitLines + 1);
      const int32_t *ln = A.line + (int64_t)u * kUnitLines;
      const int G = c[kUnitLines];
      const int sj = lane * q;
      int li = kUnitLines, nb = 0x7fffffff;
      if (sj < G) {  // the line holding this lane's first group (empty lines skipped)
        li = 0;
        while (c[li + 1] <= sj) ++li;
        nb = c[li + 1];
      }
      const int li_first = li;
      double acc0 = 0.0, acc1 = 0.0, p_first = 0.0, p_last = 0.0;
      int li_last = kUnitLines;
      for (int k = 0; k < q; ++k) {
        const int t = sj + k;
        if (t == nb && t < G) {  // this lane's run enters the next line
          const double a = acc0 + acc1;
          if (li == li_first) p_first = a;
          else part[ln[li]] = a;  // a line wholly inside the run
          acc0 = acc1 = 0.0;
          ++li;
          while (c[li + 1] <= t) ++li;
          nb = c[li + 1];
        }
        if (k + 2 < q) {  // the step after next into L2
          asm volatile("prefetch.global.L2 [%0];" ::"l"(idx8 + base + (int64_t)(k + 2) * 32 + lane));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(val2 + base * 4 +
                                                        (int64_t)((k + 2) * 4) * 32 + lane));
        }
        const uint4 g = __ldg(idx8 + base + (int64_t)k * 32 + lane);
        const double2 *vp = val2 + base * 4 + (int64_t)(k * 4) * 32 + lane;
        const double2 v0 = __ldg(vp), v1 = __ldg(vp + 32), v2 = __ldg(vp + 64), v3 = __ldg(vp + 96);
        acc0 = fma(v0.x, xs[g.x & 0xffff], acc0);
        acc1 = fma(v0.y, xs[g.x >> 16], acc1);
        acc0 = fma(v1.x, xs[g.y & 0xffff], acc0);
        acc1 = fma(v1.y, xs[g.y >> 16], acc1);
        acc0 = fma(v2.x, xs[g.z & 0xffff], acc0);
        acc1 = fma(v2.y, xs[g.z >> 16], acc1);
        acc0 = fma(v3.x, xs[g.w & 0xffff], acc0);
        acc1 = fma(v3.y, xs[g.w >> 16], acc1);
      }
      if (sj < G) {
        const double a = acc0 + acc1;
        if (li == li_first) {
          p_first = a;
        } else {
          p_last = a;
          li_last = li;
        }
      }
      lf[lane] = li_first;
      ll[lane] = li_last;
      pf[lane] = p_first;
      pl[lane] = p_last;
      __syncwarp();
      // line `lane` of the unit: its parts in lane order
      const int l = ln[lane];
      if (l >= 0) {
        const int c0 = c[lane], c1 = c[lane + 1];
        if (c0 == c1) {
          part[l] = 0.0;
        } else {
          const int a = c0 / q, b = (c1 - 1) / q;
          if (a != b || lf[a] == lane || ll[a] == lane) {
            double t = lf[a] == lane ? pf[a] : pl[a];
            for (int j = a + 1; j <= b; ++j) t += lf[j] == lane ? pf[j] : pl[j];
            part[l] = t;
          }
        }
      }
      __syncwarp();  // the summing area is rewritten by the next unit
    }
    __syncthreads();  // every warp is done with xs before the next slab is staged
  }
}

// Shared memory of k_slab_units: the slab plus 24 bytes per thread.
__host__ __device__ constexpr size_t units_smem(size_t slab_entries, int threads) {
  return slab_entries * sizeof(double) + (size_t)threads * (2 * sizeof(double) + 2 * sizeof(int));
}

}  // namespace plsqr
