// Unit layout of the kernel matrix, for the products on slabs: FP64, and
// FP32 for the mixed solver's inner sweeps.
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
//   val[(slot0*P + (k*P + p)*32 + j) * E + w]    entry e = E p + w
//
// with E = 16 / sizeof(T) values per 16-byte piece and P = 8 / E pieces per
// group: FP64 four pieces of two, FP32 (the mixed solver's inner products)
// two of four, coalesced 16-byte loads either way.  A lane sums its
// groups into the line they belong to; a line wholly inside one lane's run
// is written by that lane, and a line spread over lanes is summed by the
// unit's lane of the same index, from the lanes' parts in lane order, so the
// result is deterministic.  Units are taken from a per-slab counter by
// persistent blocks, as in k_slab_spmv_dyn.
#pragma once

#include <type_traits>

#include "check.cuh"
#include "slab.cuh"

namespace plsqr {

constexpr int kUnitLines = 32;  // lines per unit: one per lane of the summing step

template <typename T>
struct UnitsArgs {
  const uint16_t *idx;         // [slots * 8]
  const T *val;                // [slots * 8]
  const int64_t *slot0;        // [units] first slot of each unit
  const int32_t *q;            // [units] groups per lane
  const int32_t *c;            // [units * (kUnitLines + 1)] first group of each line in the unit's stream
  const int32_t *line;         // [units * kUnitLines] line index, -1 past the slab's last line
  const int32_t *unit_begin;   // [n_slabs + 1] first unit of each slab
  int32_t n_lines, n_slabs, slab, n_idx;
  int32_t pf_dist;    // steps ahead of the L2 prefetch (0: none)
  int32_t pf_pieces;  // value pieces prefetched per lane: 1 or all P
  int64_t n_slots;    // slots of the layout (bounds of the checked build)
};

// The 8 slab-local indices of a group, all inside the staged slab of len.
__device__ __forceinline__ bool group_in(uint4 g, int len) {
  const unsigned m = max(max(max(g.x & 0xffffu, g.x >> 16), max(g.y & 0xffffu, g.y >> 16)),
                         max(max(g.z & 0xffffu, g.z >> 16), max(g.w & 0xffffu, g.w >> 16)));
  return m < (unsigned)len;
}

// Values per 16-byte piece of a group, and pieces per group.
template <typename T>
struct UnitPieces {
  static constexpr int E = 16 / (int)sizeof(T);
  static constexpr int P = 8 / E;
};

// Setup: entry o of segment (s, l) to its slot.  seg_unit / seg_pos give
// the unit of segment (s, l) and the line's position in it; the arrays were
// zeroed, so padding slots and entries stay (index 0, value 0).  FP32
// values are the FP64 ones rounded to nearest.
template <typename T>
__global__ void k_units_fill(const int64_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                             const double *__restrict__ val, int n_lines, int n_slabs, int slab,
                             const int32_t *__restrict__ seg_unit, const int32_t *__restrict__ seg_pos,
                             UnitsArgs<T> U, uint16_t *__restrict__ sidx, T *__restrict__ sval) {
  constexpr int E = UnitPieces<T>::E, P = UnitPieces<T>::P;
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
      if (!chk(k < q && j < 32 && base + k * 32 + j < U.n_slots, kChkFill)) continue;
      sidx[(base + k * 32 + j) * 8 + w] = (uint16_t)(idx[e] - s * slab);
      sval[(base * P + (k * P + w / E) * 32 + j) * E + w % E] = (T)val[e];
    }
  }
}

// partial[s * n_lines + l] = sum over segment (s, l) of val * x_slab[idx],
// in FP64 for either value type.  1,024 threads: one block per SM (a slab
// of x of up to 192 KB plus the summing area); 512 threads: two blocks per
// SM on slabs of half that.
// Each lane prefetches its loads of a later step into L2 (by default all
// of the next step's).
// Exact order of one wave of 8 lanes over 8 bank groups: lane j's entry w,
// of bank group g[j][w], is gathered in round rd[j][w], a lane's rounds all
// distinct, and a bank group with d entries in the wave used at most
// ceil(d / 8) times a round, the fewest possible.  A proper 8-edge-colouring
// of the bipartite multigraph lanes x virtual groups (a group's entries cut
// into virtual groups of 8, so that no vertex has more than 8 edges), built
// edge by edge: colour a free at the lane, b free at the group; where a is
// taken at the group, the path from the group alternating a and b has its
// colours swapped first (Konig's construction; the path cannot reach the
// lane, so a is then free at both ends).  Returns false, leaving the
// caller's greedy order, if a path or a search runs past its bound (a path
// has at most the wave's 64 edges).
__host__ __device__ inline bool colour_wave(const unsigned char (&g)[8][8], unsigned char (&rd)[8][8]) {
  constexpr unsigned char kNone = 0xff;
  unsigned char vid[8][8], seen[8], at_l[8][8], at_v[64][8], path[64];
  for (int q = 0; q < 8; ++q) seen[q] = 0;
  for (int j = 0; j < 8; ++j)
    for (int w = 0; w < 8; ++w) {
      const int q = g[j][w] & 7;
      vid[j][w] = (unsigned char)(q * 8 + seen[q]++ / 8);
    }
  for (int j = 0; j < 8; ++j)
    for (int c = 0; c < 8; ++c) at_l[j][c] = kNone;
  for (int v = 0; v < 64; ++v)
    for (int c = 0; c < 8; ++c) at_v[v][c] = kNone;
  for (int j = 0; j < 8; ++j)
    for (int w = 0; w < 8; ++w) {
      const int v = vid[j][w];
      int a = 0, b = 0;
      while (a < 8 && at_l[j][a] != kNone) ++a;
      while (b < 8 && at_v[v][b] != kNone) ++b;
      if (a == 8 || b == 8) return false;
      if (at_v[v][a] != kNone) {
        int len = 0, x = v, col = a;
        bool at_group = true;
        for (;;) {
          const unsigned char e = at_group ? at_v[x][col] : at_l[x][col];
          if (e == kNone) break;
          if (len == 64) return false;
          path[len++] = e;
          x = at_group ? e / 8 : vid[e / 8][e % 8];
          at_group = !at_group;
          col = col == a ? b : a;
        }
        for (int i = 0; i < len; ++i) {  // the path's edges leave their colours
          const int e = path[i], c = (i & 1) ? b : a;
          at_l[e / 8][c] = kNone;
          at_v[vid[e / 8][e % 8]][c] = kNone;
        }
        for (int i = 0; i < len; ++i) {  // and take the other one
          const int e = path[i], c = (i & 1) ? a : b;
          at_l[e / 8][c] = (unsigned char)e;
          at_v[vid[e / 8][e % 8]][c] = (unsigned char)e;
        }
      }
      at_l[j][a] = (unsigned char)(j * 8 + w);
      at_v[v][a] = (unsigned char)(j * 8 + w);
    }
  for (int j = 0; j < 8; ++j)
    for (int c = 0; c < 8; ++c) {
      const int e = at_l[j][c];
      if (e == kNone || e / 8 != j) return false;
      rd[j][e % 8] = (unsigned char)c;
    }
  return true;
}

// Setup, optional: order each lane's 8 entries of every step so that the
// lanes one shared-memory wavefront serves (16 for 8-byte entries: FP64, or
// FP32 hi + lo pairs; 32 for 4-byte ones) gather from distinct banks where
// they can.  The kernel's e-th gather of a step reads entry e of every
// lane's group; the entries of a group may come in any order (they are
// summed into the lane's line either way).  Greedy, a warp per unit and a
// thread per step: for e = 0..7, lane by lane, the lane's remaining entry
// whose bank the wavefront has used least so far.  banks: the bank groups an
// entry's gather can fall in (index mod banks): lanes_per_wave for 4- and
// 8-byte gathers, 8 for the 16-byte pieces of the batched k-wide products,
// whose waves of 8 lanes over 8 bank groups take the exact order of
// colour_wave instead.
template <typename T>
__global__ void k_units_banks(UnitsArgs<T> U, int n_units, int lanes_per_wave, int banks,
                              uint16_t *__restrict__ sidx, T *__restrict__ sval) {
  constexpr int E = UnitPieces<T>::E, P = UnitPieces<T>::P;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int u = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n_units; u += warps) {
    const int q = U.q[u];
    const int64_t base = U.slot0[u];
    if (!chk(base + (int64_t)q * 32 <= U.n_slots, kChkFill)) continue;
    for (int k = lane; k < q; k += 32)
      for (int h = 0; h < 32; h += lanes_per_wave) {
        uint16_t id[32][8];
        T v[32][8];
        unsigned char used[32];
        for (int j = 0; j < lanes_per_wave; ++j) {
          used[j] = 0;
          for (int w = 0; w < 8; ++w) {
            id[j][w] = sidx[(base + (int64_t)k * 32 + h + j) * 8 + w];
            v[j][w] = sval[(base * P + ((int64_t)k * P + w / E) * 32 + h + j) * E + w % E];
          }
        }
        if (lanes_per_wave == 8 && banks == 8) {
          unsigned char gq[8][8], rd[8][8];
          for (int j = 0; j < 8; ++j)
            for (int w = 0; w < 8; ++w) gq[j][w] = (unsigned char)(id[j][w] & 7);
          if (colour_wave(gq, rd)) {
            for (int j = 0; j < 8; ++j)
              for (int w = 0; w < 8; ++w) {
                const int e = rd[j][w];
                sidx[(base + (int64_t)k * 32 + h + j) * 8 + e] = id[j][w];
                sval[(base * P + ((int64_t)k * P + e / E) * 32 + h + j) * E + e % E] = v[j][w];
              }
            continue;
          }
        }
        for (int e = 0; e < 8; ++e) {
          int cnt[32];
          for (int b = 0; b < banks; ++b) cnt[b] = 0;
          for (int j = 0; j < lanes_per_wave; ++j) {
            int best = -1, bc = 1 << 30;
            for (int w = 0; w < 8; ++w)
              if (!((used[j] >> w) & 1) && cnt[id[j][w] % banks] < bc) {
                bc = cnt[id[j][w] % banks];
                best = w;
              }
            used[j] |= (unsigned char)(1u << best);
            ++cnt[id[j][best] % banks];
            sidx[(base + (int64_t)k * 32 + h + j) * 8 + e] = id[j][best];
            sval[(base * P + ((int64_t)k * P + e / E) * 32 + h + j) * E + e % E] = v[j][best];
          }
        }
      }
  }
}

// One step of a lane: its group's 8 values (P coalesced 16-byte loads).
__device__ __forceinline__ void unit_vals(const double *val, int64_t base, int k, int lane,
                                          double (&v)[8]) {
  const double2 *p = reinterpret_cast<const double2 *>(val) + base * 4 + (int64_t)(k * 4) * 32 + lane;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double2 a = __ldg(p + 32 * i);
    v[2 * i] = a.x;
    v[2 * i + 1] = a.y;
  }
}
__device__ __forceinline__ void unit_vals(const float *val, int64_t base, int k, int lane,
                                          float (&v)[8]) {
  const float4 *p = reinterpret_cast<const float4 *>(val) + base * 2 + (int64_t)(k * 2) * 32 + lane;
  const float4 a = __ldg(p), b = __ldg(p + 32);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
  v[4] = b.x;
  v[5] = b.y;
  v[6] = b.z;
  v[7] = b.w;
}

// A lane's running sum of one line.  FP64 values: two chains of fused
// multiply-adds.  FP32 values (the mixed solver): each group's 8 products
// summed in FP32, the group sums added in FP64, so that a line of thousands
// of entries streamed by one lane keeps FP64 accuracy in its sum (a plain
// FP32 running sum cost the mixed solver 7% more iterations to 1e-6 on the
// 96x96x32 problem); the FP64 pipe is otherwise idle in the FP32 product.
// FP32 values with the gathered vector as hi + lo FP32 pairs (kHiLo): each
// product's rounding error recovered by a fused multiply-add, each
// addition's by the error-free sum of two floats (Knuth), the errors and the
// lo products summed in a second float: the product of the FP32 values with
// the FP64 vector to about 2^-44, in FP32 instructions only.
template <typename T, bool kHiLo = false, int kChains = 2>
struct UnitSum;
template <>
struct UnitSum<double, false, 2> {
  double a0 = 0.0, a1 = 0.0;
  __device__ __forceinline__ void add8(const double (&v)[8], const double *xs, uint4 g) {
    a0 = fma(v[0], xs[g.x & 0xffff], a0);
    a1 = fma(v[1], xs[g.x >> 16], a1);
    a0 = fma(v[2], xs[g.y & 0xffff], a0);
    a1 = fma(v[3], xs[g.y >> 16], a1);
    a0 = fma(v[4], xs[g.z & 0xffff], a0);
    a1 = fma(v[5], xs[g.z >> 16], a1);
    a0 = fma(v[6], xs[g.w & 0xffff], a0);
    a1 = fma(v[7], xs[g.w >> 16], a1);
  }
  __device__ __forceinline__ double total() const { return a0 + a1; }
  __device__ __forceinline__ void reset() { a0 = a1 = 0.0; }
};
// four chains: half the dependent fused multiply-adds per step
template <>
struct UnitSum<double, false, 4> {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  __device__ __forceinline__ void add8(const double (&v)[8], const double *xs, uint4 g) {
    a0 = fma(v[0], xs[g.x & 0xffff], a0);
    a1 = fma(v[1], xs[g.x >> 16], a1);
    a2 = fma(v[2], xs[g.y & 0xffff], a2);
    a3 = fma(v[3], xs[g.y >> 16], a3);
    a0 = fma(v[4], xs[g.z & 0xffff], a0);
    a1 = fma(v[5], xs[g.z >> 16], a1);
    a2 = fma(v[6], xs[g.w & 0xffff], a2);
    a3 = fma(v[7], xs[g.w >> 16], a3);
  }
  __device__ __forceinline__ double total() const { return (a0 + a1) + (a2 + a3); }
  __device__ __forceinline__ void reset() { a0 = a1 = a2 = a3 = 0.0; }
};
template <>
struct UnitSum<float, false, 2> {
  double a = 0.0;
  __device__ __forceinline__ void add8(const float (&v)[8], const float *xs, uint4 g) {
    float g0 = v[0] * xs[g.x & 0xffff], g1 = v[1] * xs[g.x >> 16];
    g0 = fmaf(v[2], xs[g.y & 0xffff], g0);
    g1 = fmaf(v[3], xs[g.y >> 16], g1);
    g0 = fmaf(v[4], xs[g.z & 0xffff], g0);
    g1 = fmaf(v[5], xs[g.z >> 16], g1);
    g0 = fmaf(v[6], xs[g.w & 0xffff], g0);
    g1 = fmaf(v[7], xs[g.w >> 16], g1);
    a += (double)(g0 + g1);
  }
  __device__ __forceinline__ double total() const { return a; }
  __device__ __forceinline__ void reset() { a = 0.0; }
};
template <>
struct UnitSum<float, true, 2> {
  float s = 0.0f, c = 0.0f;  // running sum and its collected errors
  // rounded intrinsics: no contraction of a product into a later addition
  __device__ __forceinline__ void add1(float v, float2 x) {
    const float p = __fmul_rn(v, x.x);
    const float pe = __fmaf_rn(v, x.x, -p);  // v * x.x - p, exactly
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));  // s + p - t
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, __fmaf_rn(v, x.y, pe)));
  }
  __device__ __forceinline__ void add8(const float (&v)[8], const float2 *xs, uint4 g) {
    add1(v[0], xs[g.x & 0xffff]);
    add1(v[1], xs[g.x >> 16]);
    add1(v[2], xs[g.y & 0xffff]);
    add1(v[3], xs[g.y >> 16]);
    add1(v[4], xs[g.z & 0xffff]);
    add1(v[5], xs[g.z >> 16]);
    add1(v[6], xs[g.w & 0xffff]);
    add1(v[7], xs[g.w >> 16]);
  }
  __device__ __forceinline__ double total() const { return (double)s + (double)c; }
  __device__ __forceinline__ void reset() { s = c = 0.0f; }
};

// The gathered vector's entry type in shared memory.
template <typename T, bool kHiLo>
using UnitX = typename std::conditional<kHiLo, float2, T>::type;

// x_lo (kHiLo only): the low halves of the FP32 pairs x + x_lo.
template <typename T, int kThreads, bool kHiLo = false, int kChains = 2>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads)
    k_slab_units(UnitsArgs<T> A, int *__restrict__ next, const T *__restrict__ x,
                 const T *__restrict__ x_lo, double *__restrict__ partial) {
  static_assert(!kHiLo || sizeof(T) == 4, "hi + lo pairs are FP32");
  using X = UnitX<T, kHiLo>;
  constexpr int P = UnitPieces<T>::P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  X *xs = reinterpret_cast<X *>(smem_raw);
  // per warp: each lane's first and last line and its FP64 sums for them,
  // after the slab (min(slab, n_idx) entries: the size the launch gives,
  // rounded up to 2 so that the sums after an FP32 slab stay aligned)
  double *pf_all = reinterpret_cast<double *>(xs + ((min(A.slab, A.n_idx) + 1) & ~1));
  double *pl_all = pf_all + kThreads;
  int *lf_all = reinterpret_cast<int *>(pl_all + kThreads);
  int *ll_all = lf_all + kThreads;
  __shared__ int s_left;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *pf = pf_all + warp * 32, *pl = pl_all + warp * 32;
  int *lf = lf_all + warp * 32, *ll = ll_all + warp * 32;
  const uint4 *idx8 = reinterpret_cast<const uint4 *>(A.idx);
  const uint4 *val16 = reinterpret_cast<const uint4 *>(A.val);
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
    if constexpr (kHiLo) {
      for (int i = threadIdx.x; i < len; i += kThreads) xs[i] = make_float2(x[xbase + i], x_lo[xbase + i]);
    } else {
      for (int i = threadIdx.x; i < len; i += kThreads) xs[i] = x[xbase + i];
    }
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
      chk(base + (int64_t)q * 32 <= A.n_slots, kChkSlot);
      if (sj < G) {  // the line holding this lane's first group (empty lines skipped)
        li = 0;
        while (c[li + 1] <= sj && chk(li + 1 < kUnitLines, kChkLine)) ++li;
        nb = c[li + 1];
      }
      const int li_first = li;
      UnitSum<T, kHiLo, kChains> acc;
      double p_first = 0.0, p_last = 0.0;
      int li_last = kUnitLines;
      for (int k = 0; k < q; ++k) {
        const int t = sj + k;
        if (t == nb && t < G) {  // this lane's run enters the next line
          const double a = acc.total();
          if (li == li_first) p_first = a;
          else if (chk(ln[li] >= 0 && ln[li] < A.n_lines, kChkLine)) part[ln[li]] = a;  // a line wholly inside the run
          acc.reset();
          ++li;
          while (chk(li < kUnitLines, kChkLine) && c[li + 1] <= t) ++li;
          nb = c[li + 1];
        }
        const int kp = k + A.pf_dist;
        if (A.pf_dist > 0 && kp < q) {  // a later step into L2
          asm volatile("prefetch.global.L2 [%0];" ::"l"(idx8 + base + (int64_t)kp * 32 + lane));
          for (int pc = 0; pc < A.pf_pieces; ++pc)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(val16 + base * P +
                                                          (int64_t)(kp * P + pc) * 32 + lane));
        }
        if (!chk(base + (int64_t)k * 32 + lane < A.n_slots, kChkSlot)) continue;
        const uint4 g = __ldg(idx8 + base + (int64_t)k * 32 + lane);
        T v[8];
        unit_vals(A.val, base, k, lane, v);
        if (chk(group_in(g, len), kChkGather)) acc.add8(v, xs, g);
      }
      if (sj < G) {
        const double a = acc.total();
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
      if (l >= 0 && chk(l < A.n_lines, kChkLine)) {
        const int c0 = c[lane], c1 = c[lane + 1];
        if (c0 == c1) {
          part[l] = 0;
        } else {
          const int a = c0 / q, b = (c1 - 1) / q;
          if (!chk(a >= 0 && b < 32 && a <= b, kChkLane)) {
          } else if (a != b || lf[a] == lane || ll[a] == lane) {
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

// Shared memory of k_slab_units: the slab plus 2 FP64 sums and 2 line
// indices per thread.
template <typename T, bool kHiLo = false>
__host__ __device__ constexpr size_t units_smem(size_t slab_entries, int threads) {
  return ((slab_entries + 1) & ~size_t(1)) * sizeof(UnitX<T, kHiLo>) +
         (size_t)threads * (2 * sizeof(double) + 2 * sizeof(int));
}

}  // namespace plsqr
