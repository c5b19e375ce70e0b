// Construction of the slab layout (slab.cuh) on the device, at context
// creation: count entries per (slab, line), lay the segments out slab-major
// with 8-entry padding, scatter, and cut every slab's lines into
// nonzero-balanced ranges, one per block.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "plsqr_internal.h"
#include "slab.cuh"

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

// Plan the slab paths.  slab_ok: every dimension fits kMaxSlabs slabs of
// 24,576 FP32 values, so the mixed solver's inner products use FP32 slabs.
// FP64: A^T y uses slabs of 24,576 values (its gathers of u_k scatter over
// L2, and shared memory serves them faster); A x keeps the per-line kernel
// (its gathers of v hit nearby columns and already run near the HBM
// roofline, while slab segments would add FP64 reductions).  PLSQR_SLABS
// overrides: 0 none, 1 both orientations, 2 A^T y only (default).
int slab_plan(plsqr_ctx *ctx) {
  ctx->use_slabs = ctx->use_slabs_rows = false;
  const int fslab = 24576;
  ctx->slab_ok = ctx->nnz_k > 0 && (ctx->n + fslab - 1) / fslab <= kMaxSlabs &&
                 (ctx->m_k + fslab - 1) / fslab <= kMaxSlabs;
  const int sm = ctx->sm_count, half = kMaxParts / 2;
  ctx->gc1k = std::max(1, std::min({sm * 2, (ctx->m_k + 255) / 256, half}));
  ctx->gc1d = std::max(1, std::min({sm * 2, (ctx->m_d + 255) / 256, half}));
  ctx->gc2 = std::max(1, std::min({sm * 4, (ctx->n + 255) / 256, kMaxParts}));
  int mode = 2;
  if (const char *e = getenv("PLSQR_SLABS")) mode = atoi(e);
  int slab = 24576;  // 192 KB of FP64 per block
  if (const char *s = getenv("PLSQR_SLAB_SIZE"))
    if (atoi(s) >= 1024 && atoi(s) <= 28672) slab = atoi(s);
  const bool rows_fit = (ctx->n + slab - 1) / slab <= kMaxSlabs;
  const bool cols_fit = (ctx->m_k + slab - 1) / slab <= kMaxSlabs;
  if (ctx->nnz_k == 0 || mode <= 0) return PLSQR_OK;
  int rc;
  if (mode == 1 && rows_fit) {
    if ((rc = build_slab<double>(ctx, ctx->K, ctx->n, slab, 16 * ctx->sm_count, &ctx->s_rows, 0,
                                 slab_dyn_blocks(ctx, false))))
      return rc;
    ctx->use_slabs_rows = true;
  }
  if ((mode == 1 || mode == 2) && cols_fit) {
    if ((rc = build_slab<double>(ctx, ctx->KC, ctx->m_k, slab, 16 * ctx->sm_count, &ctx->s_cols, 0,
                                 slab_dyn_blocks(ctx, false))))
      return rc;
    ctx->use_slabs = true;
  }
  return PLSQR_OK;
}
