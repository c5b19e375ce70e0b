// Construction of the slab layout (slab.cuh) on the device, at context
// creation: count entries per (slab, line), lay the segments out slab-major
// with 8-entry padding, scatter, and cut every slab's lines into
// nonzero-balanced ranges, one per block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "plsqr_internal.h"
#include "slab.cuh"
#include "units.cuh"

using namespace plsqr;

#define CK(call)                                                               \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ctx_set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call,            \
                    cudaGetErrorString(e_));                                   \
      return PLSQR_ERR_CUDA;                                                   \
    }                                                                          \
  } while (0)

namespace {
constexpr int kMaxSlabs = 64;  // k_slab_count / k_slab_fill keep one counter per slab
}

int slab_dyn_blocks(const plsqr_ctx *ctx, bool fp32) {
  // defaults measured on the 96x96x32 problem: the FP64 A^T y product
  // 2.81 -> 2.66 ms persistent; the FP32 products slower persistent
  int on = fp32 ? 0 : 1;
  if (const char *e = getenv(fp32 ? "PLSQR_SLAB_SCHED_F" : "PLSQR_SLAB_SCHED"))
    if (e[0] == '0' || e[0] == '1') on = e[0] - '0';
  // resident blocks per SM: one 192 KB FP64 slab, two 96 KB FP32 slabs
  return on ? ctx->sm_count * (fp32 ? 2 : 1) : 0;
}

template <typename T>
int build_slab(plsqr_ctx *ctx, const DevLines &L, int32_t n_idx, int32_t slab, int blocks,
               DevSlab<T> *out, int tgroup, int dyn_blocks) {
  const int n_lines = L.n_lines;
  const int n_slabs = std::max(1, (n_idx + slab - 1) / slab);
  if (n_slabs > kMaxSlabs) return PLSQR_ERR_ARG;
  int rc;
  int64_t *cnt = nullptr;
  const int64_t cells = (int64_t)n_slabs * n_lines;
  if ((rc = dev_alloc(ctx, &cnt, (size_t)std::max<int64_t>(cells, 1)))) return rc;
  const int g = std::max(1, std::min(ctx->sm_count * 8, (n_lines + 255) / 256));
  k_slab_count<<<g, 256, 0, ctx->stream>>>(L.ptr, L.idx, n_lines, n_slabs, slab, cnt);
  CK(cudaGetLastError());
  std::vector<int64_t> hc((size_t)std::max<int64_t>(cells, 1));
  CK(cudaMemcpyAsync(hc.data(), cnt, sizeof(int64_t) * cells, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, cnt);
  // slab-major segment starts
  std::vector<int64_t> sp((size_t)n_slabs * (n_lines + 1));
  int64_t run = 0;
  for (int s = 0; s < n_slabs; ++s) {
    for (int l = 0; l < n_lines; ++l) {
      sp[(size_t)s * (n_lines + 1) + l] = run;
      run += hc[(size_t)s * n_lines + l];
    }
    sp[(size_t)s * (n_lines + 1) + n_lines] = run;
  }
  out->n_lines = n_lines;
  out->n_slabs = n_slabs;
  out->slab = slab;
  out->n_idx = n_idx;
  out->nnz_padded = run;
  if ((rc = dev_alloc(ctx, &out->ptr, sp.size())) || (rc = dev_alloc(ctx, &out->idx, (size_t)run)) ||
      (rc = dev_alloc(ctx, &out->val, (size_t)run)) ||
      (rc = dev_alloc(ctx, &out->partial, (size_t)std::max<int64_t>(cells, 1))))
    return rc;
  CK(cudaMemcpy(out->ptr, sp.data(), sizeof(int64_t) * sp.size(), cudaMemcpyHostToDevice));
  k_slab_fill<T><<<g, 256, 0, ctx->stream>>>(L.ptr, L.idx, L.val, n_lines, n_slabs, slab, out->ptr,
                                             tgroup, out->idx, out->val);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  // blocks per slab: `blocks` in total (several waves of small, nonzero-
  // balanced line ranges; measured better than one wave of large ones)
  int bps = std::max(1, (blocks + n_slabs - 1) / n_slabs);
  if (const char *e = getenv("PLSQR_SLAB_BLOCKS"))
    if (atoi(e) > 0) bps = std::max(1, atoi(e) / n_slabs);
  if (dyn_blocks > 0) {  // persistent form: one range, the whole slab sorted
    bps = 1;
    out->dyn_blocks = dyn_blocks;
    out->chunk = 4;
    if (const char *e = getenv("PLSQR_SLAB_CHUNK"))
      if (atoi(e) >= 1 && atoi(e) <= 64) out->chunk = atoi(e);
    if ((rc = dev_alloc(ctx, &out->next, (size_t)n_slabs))) return rc;
  }
  out->bps = bps;
  std::vector<int32_t> lp((size_t)n_slabs * (bps + 1));
  for (int s = 0; s < n_slabs; ++s) {
    const int64_t *seg = sp.data() + (size_t)s * (n_lines + 1);
    const int64_t b0 = seg[0], tot = seg[n_lines] - b0;
    int32_t *o = lp.data() + (size_t)s * (bps + 1);
    o[0] = 0;
    for (int r = 1; r < bps; ++r) {
      const int64_t target = b0 + (int64_t)((long double)tot * r / bps);
      const int64_t *it = std::lower_bound(seg, seg + n_lines + 1, target);
      o[r] = std::max<int32_t>(o[r - 1], (int32_t)std::min<int64_t>(it - seg, n_lines));
    }
    o[bps] = n_lines;
  }
  // visit order inside every block range: longest segment first, ties by line
  std::vector<int32_t> ord((size_t)n_slabs * n_lines);
  for (int s = 0; s < n_slabs; ++s) {
    const int64_t *seg = sp.data() + (size_t)s * (n_lines + 1);
    int32_t *o = ord.data() + (size_t)s * n_lines;
    for (int l = 0; l < n_lines; ++l) o[l] = l;
    const int32_t *b = lp.data() + (size_t)s * (bps + 1);
    for (int r = 0; r < bps; ++r)
      std::stable_sort(o + b[r], o + b[r + 1], [&](int32_t a, int32_t c) {
        return seg[a + 1] - seg[a] > seg[c + 1] - seg[c];
      });
  }
  if ((rc = dev_alloc(ctx, &out->lpart, lp.size())) || (rc = dev_alloc(ctx, &out->order, ord.size())))
    return rc;
  CK(cudaMemcpy(out->lpart, lp.data(), sizeof(int32_t) * lp.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(out->order, ord.data(), sizeof(int32_t) * ord.size(), cudaMemcpyHostToDevice));
  // the launching translation unit sets the kernel's shared-memory limit
  out->smem = sizeof(T) * (size_t)std::min(slab, n_idx);
  return PLSQR_OK;
}

template int build_slab<double>(plsqr_ctx *, const DevLines &, int32_t, int32_t, int,
                                DevSlab<double> *, int, int);
template int build_slab<float>(plsqr_ctx *, const DevLines &, int32_t, int32_t, int,
                               DevSlab<float> *, int, int);

// The unit layout (units.cuh) of a by-line matrix: segments counted as for
// the slab layout, lines of each slab sorted longest segment first and cut
// into units of kUnitLines, every unit's groups assigned to 32 lanes.
//
// lane_lines: lane j of a unit streams line j alone (q = the unit's longest
// segment in groups, the shorter ones padded with zero entries), for the
// k-wide products of the batched solver, whose lanes then need no summing
// across lanes.
template <typename T>
int build_units(plsqr_ctx *ctx, const DevLines &L, int32_t n_idx, int32_t slab,
                DevUnitsT<T> *out, bool hilo, bool lane_lines) {
  const int n_lines = L.n_lines;
  const int n_slabs = std::max(1, (n_idx + slab - 1) / slab);
  if (n_slabs > kMaxSlabs) return PLSQR_ERR_ARG;
  int rc;
  const int64_t cells = (int64_t)n_slabs * n_lines;
  int64_t *cnt = nullptr;
  if ((rc = dev_alloc(ctx, &cnt, (size_t)std::max<int64_t>(cells, 1)))) return rc;
  const int g = std::max(1, std::min(ctx->sm_count * 8, (n_lines + 255) / 256));
  k_slab_count<<<g, 256, 0, ctx->stream>>>(L.ptr, L.idx, n_lines, n_slabs, slab, cnt);
  CK(cudaGetLastError());
  std::vector<int64_t> hc((size_t)std::max<int64_t>(cells, 1));
  CK(cudaMemcpyAsync(hc.data(), cnt, sizeof(int64_t) * cells, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, cnt);
  // units: per slab, lines longest segment first (ties by line), 32 at a time
  std::vector<int32_t> ubeg((size_t)n_slabs + 1, 0), uq, uc, uline, seg_unit((size_t)cells),
      seg_pos((size_t)cells);
  std::vector<int64_t> uslot;
  int64_t slots = 0;
  std::vector<int32_t> ord((size_t)n_lines);
  // lines per unit: kUnitLines, or fewer (PLSQR_UNIT_LINES; the unit's other
  // line slots stay empty) for shorter units and a shorter launch tail
  int lpu = kUnitLines;
  if (const char *e = getenv("PLSQR_UNIT_LINES"))
    if (atoi(e) >= 1 && atoi(e) <= kUnitLines && !lane_lines) lpu = atoi(e);
  for (int s = 0; s < n_slabs; ++s) {
    const int64_t *cs = hc.data() + (size_t)s * n_lines;
    for (int l = 0; l < n_lines; ++l) ord[(size_t)l] = l;
    std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return cs[a] > cs[b]; });
    ubeg[(size_t)s] = (int32_t)uq.size();
    for (int i0 = 0; i0 < n_lines; i0 += lpu) {
      const int u = (int)uq.size();
      int64_t run = 0, qmax = 0;
      if (lane_lines)
        for (int i = 0; i < lpu && i0 + i < n_lines; ++i)
          qmax = std::max<int64_t>(qmax, cs[ord[(size_t)i0 + i]] / 8);
      for (int i = 0; i < kUnitLines; ++i) {
        uc.push_back((int32_t)(lane_lines ? i * qmax : run));
        if (i < lpu && i0 + i < n_lines) {
          const int l = ord[(size_t)i0 + i];
          uline.push_back(l);
          seg_unit[(size_t)s * n_lines + l] = u;
          seg_pos[(size_t)s * n_lines + l] = i;
          run += cs[l] / 8;
        } else {
          uline.push_back(-1);
        }
      }
      if (lane_lines) run = kUnitLines * qmax;
      uc.push_back((int32_t)run);
      if (run > INT32_MAX / 2) return PLSQR_ERR_ARG;
      const int64_t q = lane_lines ? qmax : (run + 31) / 32;
      uq.push_back((int32_t)q);
      uslot.push_back(slots);
      slots += 32 * q;
    }
  }
  ubeg[(size_t)n_slabs] = (int32_t)uq.size();
  out->n_lines = n_lines;
  out->n_slabs = n_slabs;
  out->slab = slab;
  out->n_idx = n_idx;
  out->n_units = (int32_t)uq.size();
  out->slots = slots;
  int32_t *d_seg_unit = nullptr, *d_seg_pos = nullptr;
  if ((rc = dev_alloc(ctx, &out->idx, (size_t)slots * 8)) ||
      (rc = dev_alloc(ctx, &out->val, (size_t)slots * 8)) ||
      (rc = dev_alloc(ctx, &out->slot0, uslot.size())) || (rc = dev_alloc(ctx, &out->q, uq.size())) ||
      (rc = dev_alloc(ctx, &out->c, uc.size())) || (rc = dev_alloc(ctx, &out->line, uline.size())) ||
      (rc = dev_alloc(ctx, &out->unit_begin, ubeg.size())) ||
      (rc = dev_alloc(ctx, &out->next, (size_t)n_slabs)) ||
      (rc = dev_alloc(ctx, &out->partial, (size_t)std::max<int64_t>(cells, 1))) ||
      (rc = dev_alloc(ctx, &d_seg_unit, seg_unit.size())) ||
      (rc = dev_alloc(ctx, &d_seg_pos, seg_pos.size())))
    return rc;
  CK(cudaMemsetAsync(out->idx, 0, sizeof(uint16_t) * 8 * (size_t)std::max<int64_t>(slots, 1),
                     ctx->stream));
  CK(cudaMemsetAsync(out->val, 0, sizeof(T) * 8 * (size_t)std::max<int64_t>(slots, 1),
                     ctx->stream));
  CK(cudaMemcpy(out->slot0, uslot.data(), sizeof(int64_t) * uslot.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(out->q, uq.data(), sizeof(int32_t) * uq.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(out->c, uc.data(), sizeof(int32_t) * uc.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(out->line, uline.data(), sizeof(int32_t) * uline.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(out->unit_begin, ubeg.data(), sizeof(int32_t) * ubeg.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_seg_unit, seg_unit.data(), sizeof(int32_t) * seg_unit.size(),
                cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_seg_pos, seg_pos.data(), sizeof(int32_t) * seg_pos.size(), cudaMemcpyHostToDevice));
  const UnitsArgs<T> U{out->idx,       out->val, out->slot0, out->q, out->c, out->line,
                       out->unit_begin, n_lines,  n_slabs,    slab,   n_idx,  0,
                       0,               slots};
  k_units_fill<<<g, 256, 0, ctx->stream>>>(L.ptr, L.idx, L.val, n_lines, n_slabs, slab, d_seg_unit,
                                           d_seg_pos, U, out->idx, out->val);
  CK(cudaGetLastError());
  // The entries of every step ordered for distinct shared-memory banks: by
  // default for the FP32 hi + lo pairs (inner iteration 2.62 -> 2.56 ms on
  // the 96x96x32 problem), not for FP64 (measured no change) nor the FP32
  // mirror alone; PLSQR_UNIT_BANKS=0/1 overrides.
  // The lane-per-line layout of the batched k-wide products gathers 16-byte
  // pieces of rows staged piece-major: a wavefront serves 8 lanes, over 8
  // groups of 4 banks (row mod 8); ordered by default (on the 48x48x32
  // problem 10.4 shared-memory wavefronts per gather unordered, 7.5 with the
  // 32 lanes balanced as one wave, against 4 at best).
  bool banks = (sizeof(T) == 4 && hilo) || lane_lines;
  if (const char *e = getenv("PLSQR_UNIT_BANKS")) banks = atoi(e) == 1;
  if (banks) {
    const int wave = lane_lines ? 8 : (sizeof(T) == 8 || hilo) ? 16 : 32;
    const int groups = lane_lines ? 8 : wave;
    const int nu = (int)uq.size();
    k_units_banks<<<std::max(1, (nu + 3) / 4), 128, 0, ctx->stream>>>(U, nu, wave, groups,
                                                                     out->idx, out->val);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, d_seg_unit);
  dev_free(ctx, d_seg_pos);
  // PLSQR_UNIT_THREADS=512: two blocks per SM where two slabs fit in shared memory
  out->hilo = hilo && sizeof(T) == 4;
  auto smem = [&](int threads) {
    return out->hilo ? units_smem<T, true>((size_t)std::min(slab, n_idx), threads)
                     : units_smem<T, false>((size_t)std::min(slab, n_idx), threads);
  };
  out->threads = 1024;
  if (const char *e = getenv("PLSQR_UNIT_THREADS"))
    if (atoi(e) == 512 && 2 * (smem(512) + 1024) <= 228 * 1024) out->threads = 512;
  out->blocks = ctx->sm_count * (1024 / out->threads);
  // PLSQR_UNIT_CHAINS=4: four FP64 accumulator chains per lane instead of two
  out->chains = 2;
  if (const char *e = getenv("PLSQR_UNIT_CHAINS"))
    if (atoi(e) == 4) out->chains = 4;
  // Each lane prefetches all its loads of the next step into L2 (on the
  // 96x96x32 problem against the step after next, first value piece only:
  // FP64 A x 2.32 -> 2.29 ms, FP32 A x 1.28 -> 1.22 ms; two steps of all
  // pieces are on par, four or more steps of all pieces slower: 4,864 warps
  // prefetching 10 KB each begin to evict one another's lines from L2).
  // PLSQR_UNIT_PREFETCH=d,p: d steps ahead (0: none), p value pieces.
  out->pf_dist = 1;
  out->pf_pieces = UnitPieces<T>::P;
  if (const char *e = getenv("PLSQR_UNIT_PREFETCH")) {
    int d = 1, pc = UnitPieces<T>::P;
    if (sscanf(e, "%d,%d", &d, &pc) >= 1 && d >= 0 && d <= 16) out->pf_dist = d;
    if (pc >= 1 && pc <= UnitPieces<T>::P) out->pf_pieces = pc;
  }
  out->smem = smem(out->threads);
  return PLSQR_OK;
}
template int build_units<double>(plsqr_ctx *, const DevLines &, int32_t, int32_t,
                                 DevUnitsT<double> *, bool, bool);
template int build_units<float>(plsqr_ctx *, const DevLines &, int32_t, int32_t,
                                DevUnitsT<float> *, bool, bool);

template <typename T>
bool units_fit(int32_t n_idx, int32_t slab, bool hilo) {
  const size_t e = (size_t)std::min(slab, n_idx);
  const size_t smem = hilo && sizeof(T) == 4 ? units_smem<T, true>(e, 1024) : units_smem<T, false>(e, 1024);
  return slab >= 1 && slab <= 65536 && (n_idx + slab - 1) / slab <= kMaxSlabs && smem <= 227 * 1024;
}
unsigned slab_check_word(bool reset) { return plsqr::check_word(reset); }

template bool units_fit<double>(int32_t, int32_t, bool);
template bool units_fit<float>(int32_t, int32_t, bool);

// Plan the slab paths.  slab_ok: every dimension fits kMaxSlabs slabs of
// 24,576 FP32 values, so the mixed solver's inner products use FP32 layouts.
// FP64: both products on slabs of 20,480 values in the unit layout
// (units.cuh): on the 96x96x32 problem A^T y 2.66 -> 2.26 ms and A x 2.57 ->
// 2.29 ms against the segment-per-group slab kernel and the per-row kernel
// k_aprod1 (16-bit indices, every lane busy, the gathered vector in shared
// memory).  PLSQR_SLABS overrides: 0 none, 1 both orientations (default),
// 2 A^T y only; PLSQR_SLAB_UNITS=0 the slab kernel instead of the units.
int slab_plan(plsqr_ctx *ctx) {
  ctx->use_slabs = ctx->use_slabs_rows = ctx->use_units = ctx->use_units_rows = false;
  const int fslab = 24576;
  ctx->slab_ok = ctx->nnz_k > 0 && (ctx->n + fslab - 1) / fslab <= kMaxSlabs &&
                 (ctx->m_k + fslab - 1) / fslab <= kMaxSlabs;
  const int sm = ctx->sm_count, half = kMaxParts / 2;
  ctx->gc1k = std::max(1, std::min({sm * 2, (ctx->m_k + 255) / 256, half}));
  ctx->gc1d = std::max(1, std::min({sm * 2, (ctx->m_d + 255) / 256, half}));
  ctx->gc2 = std::max(1, std::min({sm * 4, (ctx->n + 255) / 256, kMaxParts}));
  // a mixed-precision context solves with its FP32 layouts (mixed.cu) and
  // runs FP64 products only for plsqr_aprod calls: no FP64 layouts by default
  int mode = ctx->opts.precision == PLSQR_PREC_MIXED ? 0 : 1;
  if (const char *e = getenv("PLSQR_SLABS")) mode = atoi(e);
  int slab = 20480;  // 160 KB of FP64 per block (24,576: A x + A^T y 1.5% slower)
  if (const char *s = getenv("PLSQR_SLAB_SIZE"))
    if (atoi(s) >= 1024 && atoi(s) <= 28672) slab = atoi(s);
  const bool rows_fit = (ctx->n + slab - 1) / slab <= kMaxSlabs;
  const bool cols_fit = (ctx->m_k + slab - 1) / slab <= kMaxSlabs;
  if (ctx->nnz_k == 0 || mode <= 0) return PLSQR_OK;
  int rc;
  // the unit layout unless PLSQR_SLAB_UNITS=0 (or the slab and its summing
  // area do not fit in shared memory)
  int units = 1;
  if (const char *e = getenv("PLSQR_SLAB_UNITS")) units = atoi(e) != 0;
  if (mode == 1 && rows_fit) {
    if (units && units_smem<double>((size_t)std::min(slab, ctx->n), 1024) <= 227 * 1024) {
      if ((rc = build_units(ctx, ctx->K, ctx->n, slab, &ctx->u_rows))) return rc;
      ctx->use_units_rows = true;
    } else if ((rc = build_slab<double>(ctx, ctx->K, ctx->n, slab, 16 * ctx->sm_count, &ctx->s_rows,
                                        0, slab_dyn_blocks(ctx, false)))) {
      return rc;
    }
    ctx->use_slabs_rows = true;
  }
  if ((mode == 1 || mode == 2) && cols_fit) {
    if (units && units_smem<double>((size_t)std::min(slab, ctx->m_k), 1024) <= 227 * 1024) {
      if ((rc = build_units(ctx, ctx->KC, ctx->m_k, slab, &ctx->u_cols))) return rc;
      ctx->use_units = true;
    } else if ((rc = build_slab<double>(ctx, ctx->KC, ctx->m_k, slab, 16 * ctx->sm_count,
                                        &ctx->s_cols, 0, slab_dyn_blocks(ctx, false)))) {
      return rc;
    }
    ctx->use_slabs = true;
  }
  return PLSQR_OK;
}
