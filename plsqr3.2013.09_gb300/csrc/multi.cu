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
// Per iteration (four barriers):
//   A  u = -alpha u + A v            kernel rows by warp, damping rows by thread
//   B  beta = ||u||, u /= beta       every block sums the group's partials
//   C  v = -beta v + A^T u           columns by warp
//   D  alpha = ||v||, v /= alpha, rotation, x/w update, dknorm partials
//   E  (after the barrier) dknorm and the rest of the scalars
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
  const int32_t *kpart;  // [nw + 1] kernel-row range of each warp of the group
  const int32_t *cpart;  // [nw + 1] column range of each warp of the group
  const double *b;
  double *u, *v, *w, *x;
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
  __syncthreads();
  if (g.nb == 1) return true;
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

// Dot product of a line with a vector block-wide by one warp: lane-strided
// entries, shuffle tree.  Vector entries come from L2.
__device__ __forceinline__ double line_dot(const int32_t *__restrict__ idx,
                                           const double *__restrict__ val, const double *vec,
                                           int64_t beg, int64_t end, int lane) {
  double a0 = 0.0, a1 = 0.0;
  int64_t e = beg + lane;
  for (; e + 32 < end; e += 64) {
    a0 = fma(__ldg(val + e), ld(vec + __ldg(idx + e)), a0);
    a1 = fma(__ldg(val + e + 32), ld(vec + __ldg(idx + e + 32)), a1);
  }
  if (e < end) a0 = fma(__ldg(val + e), ld(vec + __ldg(idx + e)), a0);
  return a0 + a1;
}

}  // namespace
