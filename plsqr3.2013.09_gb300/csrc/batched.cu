// Several right-hand sides on one operator: k LSQR solves in lock step
// (kernels_batched.cuh), with the refinement form of the mixed solver
//
//   X = 0
//   repeat `sweeps` times:
//     R  = [B; 0] - A_j X_j                 FP64 kernel values, per column j
//     DX = LSQR(A_hi, R), `inner` iterations, one k-wide product per matrix read
//     X += DX
//
// where A_j = [K; lambda_j D].  The inner iteration is four steps captured
// as one CUDA graph: A x, scaling of u, A^T y, scaling of v with the x/w update
// and the scalar tail.  The product variant of each direction (the team form:
// gather width, lanes per line, nonzeros in flight; the slab form; the units
// form of kernels_bunits.cuh, in passes of 8 columns) is picked by timing the
// candidates on the operator and cached per (line-length histogram, block
// width).  With retire_every the host looks at the solves every few
// iterations, lets the finished ones go and packs the rest into the
// narrowest block width that holds them.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "kernels_batched.cuh"
#include "kernels_bunits.cuh"
#include "kernels_f32.cuh"
#include "plsqr_internal.h"

using namespace plsqr;

#define CK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      ctx_set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call,              \
                    cudaGetErrorString(e_));                                     \
      return PLSQR_ERR_CUDA;                                                     \
    }                                                                            \
  } while (0)

struct BatchState;

namespace {

// ---- product variants ------------------------------------------------------
using LaunchFn = void (*)(plsqr_ctx *, const BatchState &, int, cudaStream_t);

struct Variant {
  int vw, lpr, u;
  LaunchFn rows, cols;
};

}  // namespace

struct BatchState {
  int kp = 0;  // block width the vectors are sized for
  int kw = 4;  // block width of the current solve (a power of two <= kp)
  float *k_hi = nullptr, *kc_hi = nullptr;
  bool own_hi = false;
  double *U = nullptr, *V = nullptr, *W = nullptr, *X = nullptr, *DX = nullptr;
  double *B = nullptr, *XR = nullptr, *LAM = nullptr, *stage = nullptr;
  float *Uf = nullptr, *Vf = nullptr;
  double *tmp = nullptr;  // repacking buffer of the retirement (max(m, n) * kp)
  DevState *st = nullptr;
  BatchCoef *cf = nullptr;
  double *parts = nullptr, *parts_dk = nullptr, *parts_err = nullptr;
  int32_t *wrows = nullptr, *wcols = nullptr;
  int gk = 1, gd = 1, gc = 1, gres = 1, gvec = 1;
  int k = 0;  // right-hand sides of the current solve
  bool has_ref = false;
  int var_rows = -1, var_cols = -1;
  double ms_rows = 0.0, ms_cols = 0.0;
  int tuned = 0;
  std::string shape;  // line-length histogram signature of the operator
  plsqr_iter *hist = nullptr;
  int64_t hist_cap = 0;
  int hist_stride = 1;
  cudaGraphExec_t graph = nullptr;
  std::string graph_key;
  // slab form: team slots and grids per block width
  struct SlabPlan {
    int32_t *rows = nullptr, *cols = nullptr;
    int g_rows = 0, g_cols = 0;
  };
  std::map<int, SlabPlan> slab;
  // units form: FP32 unit layouts of K by row and by column, one lane per
  // line, and the partial sums of one pass of 4 or 8 columns
  DevUnitsT<float> ur, uc;
  bool units_tried = false, units_ok = false;
  double *upart = nullptr;
  int gur = 1, guc = 1;  // grids of the combine kernels
  int n_parts = 0;          // capacity of parts (per right-hand side)
  bool lines_sorted = true;  // every kernel row and column ascending (slab form)
};

namespace {

template <int VW, int LPR, int U>
void launch_rows(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  k_bprod_rows<VW, LPR, U><<<B.gk + B.gd, kBatchThreads, 0, s>>>(
      CsrT<float>{ctx->K.ptr, ctx->K.idx, B.k_hi, ctx->K.n_lines}, ctx->D.csr(), B.wrows, B.gk,
      B.kw, B.k, B.Vf, B.V, B.U, B.LAM, mode, B.st, B.cf, B.parts);
}
template <int VW, int LPR, int U>
void launch_cols(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  k_bprod_cols<VW, LPR, U><<<B.gc, kBatchThreads, 0, s>>>(
      CsrT<float>{ctx->KC.ptr, ctx->KC.idx, B.kc_hi, ctx->KC.n_lines}, ctx->DC.csr(), B.wcols,
      B.kw, B.k, B.Uf, B.U, ctx->m_k, B.V, B.LAM, mode, B.st, B.cf, B.parts);
}

template <int T>
void launch_slab_rows_t(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  const BatchState::SlabPlan &P = B.slab.at(B.kw);
  k_bslab_rows<T><<<P.g_rows, kSlabThreads, kSlabBytes, s>>>(
      CsrT<float>{ctx->K.ptr, ctx->K.idx, B.k_hi, ctx->K.n_lines}, P.rows, ctx->n, B.k, B.Vf,
      B.U, mode, B.st, B.parts);
  k_bdamp_rows<<<B.gd, kBatchThreads, 0, s>>>(ctx->D.csr(), ctx->m_k, B.kw, B.k, B.V, B.U, B.LAM,
                                              mode, B.st, B.cf, B.parts, P.g_rows);
}
template <int T>
void launch_slab_cols_t(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  const BatchState::SlabPlan &P = B.slab.at(B.kw);
  k_bslab_cols<T><<<P.g_cols, kSlabThreads, kSlabBytes, s>>>(
      CsrT<float>{ctx->KC.ptr, ctx->KC.idx, B.kc_hi, ctx->KC.n_lines}, ctx->DC.csr(), P.cols,
      ctx->m_k, B.k, B.Uf, B.U, B.V, B.LAM, mode, B.st, B.cf, B.parts);
}
void launch_slab_rows(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  switch (B.kw) {
    case 4: return launch_slab_rows_t<1>(ctx, B, mode, s);
    case 8: return launch_slab_rows_t<2>(ctx, B, mode, s);
    case 16: return launch_slab_rows_t<4>(ctx, B, mode, s);
    default: return launch_slab_rows_t<8>(ctx, B, mode, s);
  }
}
void launch_slab_cols(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  switch (B.kw) {
    case 4: return launch_slab_cols_t<1>(ctx, B, mode, s);
    case 8: return launch_slab_cols_t<2>(ctx, B, mode, s);
    case 16: return launch_slab_cols_t<4>(ctx, B, mode, s);
    default: return launch_slab_cols_t<8>(ctx, B, mode, s);
  }
}

UnitsArgs<float> units_args(const DevUnitsT<float> &U) {
  return UnitsArgs<float>{U.idx,     U.val,     U.slot0, U.q,     U.c,       U.line,       U.unit_begin,
                          U.n_lines, U.n_slabs, U.slab,  U.n_idx, U.pf_dist, U.pf_pieces, U.slots};
}
template <int KW>
size_t bunits_smem(const DevUnitsT<float> &U) {
  return sizeof(float) * KW * (size_t)std::min(U.slab, U.n_idx);
}
// Blocks of 4: one pass of 4 columns; wider blocks: passes of 8 columns over
// the right-hand sides in use (the padding columns past k are left alone),
// the last pass finishing the product.
template <int KW>
void launch_units_rows_t(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  const DevUnitsT<float> &U = B.ur;
  const int last = std::max(0, (B.k - 1) / KW) * KW;
  for (int c0 = 0; c0 <= last; c0 += KW) {
    cudaMemsetAsync(U.next, 0, sizeof(int) * U.n_slabs, s);
    k_bunits<KW><<<U.blocks, kBUnitThreads, bunits_smem<KW>(U), s>>>(units_args(U), U.next, B.Vf,
                                                                     B.kw, c0, B.upart);
    k_bunits_rows<KW><<<B.gur, kBatchThreads, 0, s>>>(B.upart, U.n_slabs, ctx->m_k, ctx->D.csr(),
                                                       B.k, B.kw, c0, B.V, B.U, B.LAM, mode, B.st,
                                                       B.cf, B.parts, c0 == last);
  }
}
template <int KW>
void launch_units_cols_t(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  const DevUnitsT<float> &U = B.uc;
  const int last = std::max(0, (B.k - 1) / KW) * KW;
  for (int c0 = 0; c0 <= last; c0 += KW) {
    cudaMemsetAsync(U.next, 0, sizeof(int) * U.n_slabs, s);
    k_bunits<KW><<<U.blocks, kBUnitThreads, bunits_smem<KW>(U), s>>>(units_args(U), U.next, B.Uf,
                                                                     B.kw, c0, B.upart);
    k_bunits_cols<KW><<<B.guc, kBatchThreads, 0, s>>>(B.upart, U.n_slabs, ctx->DC.csr(),
                                                       ctx->m_k, ctx->n, B.k, B.kw, c0, B.U, B.V,
                                                       B.LAM, mode, B.st, B.cf, B.parts,
                                                       c0 == last);
  }
}
void launch_units_rows(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  if (B.kw == 4) return launch_units_rows_t<4>(ctx, B, mode, s);
  return launch_units_rows_t<8>(ctx, B, mode, s);
}
void launch_units_cols(plsqr_ctx *ctx, const BatchState &B, int mode, cudaStream_t s) {
  if (B.kw == 4) return launch_units_cols_t<4>(ctx, B, mode, s);
  return launch_units_cols_t<8>(ctx, B, mode, s);
}

#define VARIANT(vw, lpr, u) \
  Variant { vw, lpr, u, launch_rows<vw, lpr, u>, launch_cols<vw, lpr, u> }
// lpr = 0: the slab form (float4 gathers from shared memory, kw/4 lanes per
// line, kSlabLines lines per team)
const Variant kVariants[] = {
    VARIANT(4, 8, 2),  VARIANT(4, 8, 4),  VARIANT(4, 16, 2), VARIANT(4, 16, 4),
    VARIANT(4, 32, 2), VARIANT(4, 32, 4), VARIANT(2, 16, 2), VARIANT(2, 16, 4),
    VARIANT(2, 32, 2), VARIANT(2, 32, 4), VARIANT(2, 8, 2),  VARIANT(2, 8, 4),
    Variant{4, 0, 0, launch_slab_rows, launch_slab_cols},
    // lpr = -1: the units form (kernels_bunits.cuh): blocks of 4, or passes
    // of 8 columns
    Variant{4, -1, 0, launch_units_rows, launch_units_cols},
};
#undef VARIANT
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));

bool variant_ok(int v, int kp) {
  if (v < 0 || v >= kNumVariants) return false;
  const Variant &V = kVariants[v];
  if (V.lpr == 0) return true;
  if (V.lpr < 0) return kp % 4 == 0 && kp <= kBatchMax;
  return kp % V.vw == 0 && kp / V.vw <= V.lpr;
}

// Team slots of the slab form: lines dealt longest first to all teams in
// turn, forward then backward (snake), so the teams' nonzero totals are
// close; slots[(block*teams + team)*kSlabLines + t], -1 where none.
int deal_lines(const std::vector<int64_t> &len, int teams_per_block, std::vector<int32_t> &slots) {
  const int64_t n = (int64_t)len.size();
  const int per_block = teams_per_block * kSlabLines;
  const int grid = (int)std::max<int64_t>(1, (n + per_block - 1) / per_block);
  const int64_t teams = (int64_t)grid * teams_per_block;
  std::vector<int32_t> order((size_t)n);
  for (int64_t i = 0; i < n; ++i) order[(size_t)i] = (int32_t)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return len[(size_t)a] > len[(size_t)b]; });
  slots.assign((size_t)teams * kSlabLines, -1);
  int64_t next = 0;
  for (int t = 0; t < kSlabLines && next < n; ++t)
    for (int64_t i = 0; i < teams && next < n; ++i) {
      const int64_t team = (t % 2 == 0) ? i : teams - 1 - i;
      slots[(size_t)(team * kSlabLines + t)] = order[(size_t)next++];
    }
  return grid;
}

int width_for(int k) {
  int kp = 4;
  while (kp < k) kp <<= 1;
  return kp;
}

// Line-length histogram of an operator: per power-of-two length class, the
// share of nonzeros in sixteenths.
std::string length_signature(const std::vector<int64_t> &ptr) {
  const int64_t n = (int64_t)ptr.size() - 1, nnz = ptr.back();
  int64_t cls[40] = {0};
  for (int64_t i = 0; i < n; ++i) {
    const int64_t len = ptr[(size_t)i + 1] - ptr[(size_t)i];
    int c = 0;
    while ((int64_t(1) << c) < len && c < 39) ++c;
    cls[c] += len;
  }
  std::string s;
  for (int c = 0; c < 40; ++c) {
    const int q = nnz > 0 ? (int)((cls[c] * 16 + nnz / 2) / nnz) : 0;
    if (q > 0) s += std::to_string(c) + ":" + std::to_string(q) + ",";
  }
  return s;
}

// (signature | kp) -> (rows variant, cols variant), process-wide
std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune_cache;

void nnz_partition(const std::vector<int64_t> &pre, int parts, std::vector<int32_t> &out) {
  const int32_t n = (int32_t)pre.size() - 1;
  out.assign((size_t)parts + 1, 0);
  const int64_t nnz = pre.back();
  for (int w = 1; w < parts; ++w) {
    const int64_t target = (int64_t)((long double)nnz * w / parts);
    int32_t r = (int32_t)(std::lower_bound(pre.begin(), pre.end(), target) - pre.begin());
    out[(size_t)w] = std::max(std::min(r, n), out[(size_t)w - 1]);
  }
  out[(size_t)parts] = n;
}

}  // namespace

// flag = 1 if some line has its indices out of ascending order (the slab
// form walks each line's entries as one ascending run).
static __global__ void k_check_sorted(const int64_t *__restrict__ ptr,
                                      const int32_t *__restrict__ idx, int n_lines,
                                      int *__restrict__ flag) {
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n_lines; l += gridDim.x * blockDim.x)
    for (int64_t e = ptr[l] + 1; e < ptr[l + 1]; ++e)
      if (idx[e] < idx[e - 1]) {
        *flag = 1;
        break;
      }
}

void batch_free(plsqr_ctx *ctx) {
  if (!ctx || !ctx->batch) return;
  if (ctx->batch->graph) cudaGraphExecDestroy(ctx->batch->graph);
  delete ctx->batch;  // device buffers are in ctx->allocs
  ctx->batch = nullptr;
}

static void free_vectors(plsqr_ctx *ctx, BatchState *B) {
  for (void *p : {(void *)B->U, (void *)B->V, (void *)B->W, (void *)B->X, (void *)B->DX,
                  (void *)B->B, (void *)B->XR, (void *)B->stage, (void *)B->Uf, (void *)B->Vf,
                  (void *)B->tmp})
    dev_free(ctx, p);
  B->U = B->V = B->W = B->X = B->DX = B->B = B->XR = B->stage = B->tmp = nullptr;
  B->Uf = B->Vf = nullptr;
  B->kp = 0;
}

// Device buffers for blocks of width kp, the FP32 kernel values and the
// per-warp line ranges of the products.
static int batch_setup(plsqr_ctx *ctx);


static int batch_prepare(plsqr_ctx *ctx, int kp) {
  int rc;
  if (ctx->lines_released) {
    ctx_set_error(ctx, "the batched solver reads K by row and by column, which this context "
                       "released (opts.lean)");
    return PLSQR_ERR_STATE;
  }
  if (!ctx->batch) {
    ctx->batch = new BatchState();
    if ((rc = batch_setup(ctx))) {
      batch_free(ctx);  // its device buffers stay in ctx->allocs until destroy
      return rc;
    }
  }
  BatchState *B = ctx->batch;
  if (B->kp >= kp) return PLSQR_OK;
  if (B->graph) cudaGraphExecDestroy(B->graph);
  B->graph = nullptr;
  B->graph_key.clear();
  free_vectors(ctx, B);
  const size_t m = (size_t)ctx->m_k + ctx->m_d, n = (size_t)ctx->n, mk = (size_t)ctx->m_k;
  const size_t big = std::max(std::max(m, n), (size_t)1);
  if ((rc = dev_alloc(ctx, &B->U, m * kp)) || (rc = dev_alloc(ctx, &B->V, n * kp)) ||
      (rc = dev_alloc(ctx, &B->W, n * kp)) || (rc = dev_alloc(ctx, &B->X, n * kp)) ||
      (rc = dev_alloc(ctx, &B->DX, n * kp)) || (rc = dev_alloc(ctx, &B->B, mk * kp)) ||
      (rc = dev_alloc(ctx, &B->XR, n * kp)) || (rc = dev_alloc(ctx, &B->stage, big * kp)) ||
      (rc = dev_alloc(ctx, &B->Uf, mk * kp)) || (rc = dev_alloc(ctx, &B->Vf, n * kp)))
    return rc;
  CK(cudaMemsetAsync(B->U, 0, sizeof(double) * m * kp, ctx->stream));
  CK(cudaMemsetAsync(B->V, 0, sizeof(double) * n * kp, ctx->stream));
  CK(cudaMemsetAsync(B->Uf, 0, sizeof(float) * mk * kp, ctx->stream));
  CK(cudaMemsetAsync(B->Vf, 0, sizeof(float) * n * kp, ctx->stream));
  B->kp = kp;
  return PLSQR_OK;
}

static int batch_setup(plsqr_ctx *ctx) {
  int rc;
  {
    BatchState *B = ctx->batch;
    if ((rc = dev_alloc(ctx, &B->k_hi, (size_t)ctx->nnz_k)) ||
        (rc = dev_alloc(ctx, &B->kc_hi, (size_t)ctx->nnz_k)) ||
        (rc = dev_alloc(ctx, &B->st, kBatchMax)) || (rc = dev_alloc(ctx, &B->cf, 1)) ||
        (rc = dev_alloc(ctx, &B->LAM, kBatchMax)))
      return rc;
    B->own_hi = true;
    const int g = ctx->sm_count * 8;
    k_split_hilo<<<g, 256, 0, ctx->stream>>>(ctx->K.val, ctx->nnz_k, B->k_hi, nullptr);
    k_split_hilo<<<g, 256, 0, ctx->stream>>>(ctx->KC.val, ctx->nnz_k, B->kc_hi, nullptr);
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(B->cf, 0, sizeof(BatchCoef), ctx->stream));
    const std::vector<double> ones(kBatchMax, 1.0);
    CK(cudaMemcpy(B->LAM, ones.data(), sizeof(double) * kBatchMax, cudaMemcpyHostToDevice));
    // grids: kTeamBlocksPerSm resident blocks of 256 threads per SM for the
    // team products (their launch bounds), one block per SM on the damping rows
    B->gk = kTeamBlocksPerSm * ctx->sm_count;
    B->gd = ctx->sm_count;
    B->gc = kTeamBlocksPerSm * ctx->sm_count;
    B->gres = 8 * ctx->sm_count;
    B->gvec = 8 * ctx->sm_count;
    std::vector<int64_t> kr((size_t)ctx->m_k + 1), kc((size_t)ctx->n + 1), dc((size_t)ctx->n + 1);
    CK(cudaMemcpy(kr.data(), ctx->K.ptr, sizeof(int64_t) * kr.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(kc.data(), ctx->KC.ptr, sizeof(int64_t) * kc.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dc.data(), ctx->DC.ptr, sizeof(int64_t) * dc.size(), cudaMemcpyDeviceToHost));
    B->shape = "r" + length_signature(kr) + "c" + length_signature(kc);
    std::vector<int64_t> pre((size_t)ctx->n + 1);
    for (size_t c = 0; c < pre.size(); ++c) pre[c] = kc[c] + (dc[c] - dc[0]);
    std::vector<int32_t> wr, wc;
    nnz_partition(kr, B->gk * (kBatchThreads / 32), wr);
    nnz_partition(pre, B->gc * (kBatchThreads / 32), wc);
    int np = std::max(std::max(B->gk + B->gd, B->gc), std::max(B->gres, B->gvec));
    // slab form: team slots for every block width
    std::vector<int64_t> rl((size_t)ctx->m_k), cl((size_t)ctx->n);
    for (int32_t r = 0; r < ctx->m_k; ++r) rl[(size_t)r] = kr[(size_t)r + 1] - kr[(size_t)r];
    for (int32_t c = 0; c < ctx->n; ++c) cl[(size_t)c] = kc[(size_t)c + 1] - kc[(size_t)c];
    for (int kw = 4; kw <= kBatchMax; kw *= 2) {
      BatchState::SlabPlan P;
      std::vector<int32_t> sr, sc;
      P.g_rows = deal_lines(rl, kSlabThreads / (kw / 4), sr);
      P.g_cols = deal_lines(cl, kSlabThreads / (kw / 4), sc);
      if ((rc = dev_alloc(ctx, &P.rows, sr.size())) || (rc = dev_alloc(ctx, &P.cols, sc.size())))
        return rc;
      CK(cudaMemcpy(P.rows, sr.data(), sizeof(int32_t) * sr.size(), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(P.cols, sc.data(), sizeof(int32_t) * sc.size(), cudaMemcpyHostToDevice));
      np = std::max(np, std::max(P.g_rows + B->gd, P.g_cols));
      B->slab[kw] = P;
    }
    CK(cudaFuncSetAttribute(k_bslab_rows<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_rows<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_rows<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_rows<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_cols<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_cols<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_cols<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    CK(cudaFuncSetAttribute(k_bslab_cols<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSlabBytes));
    B->n_parts = np;
    int *flag = nullptr;
    if ((rc = dev_alloc(ctx, &flag, 1))) return rc;
    CK(cudaMemset(flag, 0, sizeof(int)));
    k_check_sorted<<<ctx->sm_count * 8, 256>>>(ctx->K.ptr, ctx->K.idx, ctx->m_k, flag);
    k_check_sorted<<<ctx->sm_count * 8, 256>>>(ctx->KC.ptr, ctx->KC.idx, ctx->n, flag);
    CK(cudaGetLastError());
    int h = 0;
    CK(cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost));
    dev_free(ctx, flag);
    B->lines_sorted = h == 0;
    if ((rc = dev_alloc(ctx, &B->wrows, wr.size())) || (rc = dev_alloc(ctx, &B->wcols, wc.size())) ||
        (rc = dev_alloc(ctx, &B->parts, (size_t)np * kBatchMax)) ||
        (rc = dev_alloc(ctx, &B->parts_dk, (size_t)np * kBatchMax)) ||
        (rc = dev_alloc(ctx, &B->parts_err, (size_t)np * kBatchMax)))
      return rc;
    CK(cudaMemcpy(B->wrows, wr.data(), sizeof(int32_t) * wr.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B->wcols, wc.data(), sizeof(int32_t) * wc.size(), cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return PLSQR_OK;
}

// The units form's layouts, built on first use: slabs of kBUnitSlab rows of
// the block (192 KB of shared memory at 8 right-hand sides), where both
// dimensions fit the unit layout's slab count; PLSQR_BATCH_UNITS=0 leaves
// them out.
static int batch_units(plsqr_ctx *ctx) {
  BatchState *B = ctx->batch;
  if (B->units_tried) return PLSQR_OK;
  B->units_tried = true;
  const int S = kBUnitSlab;
  if (const char *e = getenv("PLSQR_BATCH_UNITS"))
    if (atoi(e) == 0) return PLSQR_OK;
  if (ctx->nnz_k == 0 || !units_fit<float>(ctx->n, S) || !units_fit<float>(ctx->m_k, S))
    return PLSQR_OK;
  int rc;
  if ((rc = build_units<float>(ctx, ctx->K, ctx->n, S, &B->ur, false, true)) ||
      (rc = build_units<float>(ctx, ctx->KC, ctx->m_k, S, &B->uc, false, true)))
    return rc;
  // the k-wide partials replace the layouts' own
  dev_free(ctx, B->ur.partial);
  dev_free(ctx, B->uc.partial);
  B->ur.partial = B->uc.partial = nullptr;
  B->ur.blocks = B->uc.blocks = ctx->sm_count;
  const size_t cells = std::max((size_t)B->ur.n_slabs * ctx->m_k, (size_t)B->uc.n_slabs * ctx->n);
  if ((rc = dev_alloc(ctx, &B->upart, cells * 8))) return rc;
  const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  CK(cudaFuncSetAttribute(k_bunits<4>, attr,
                          (int)std::max(bunits_smem<4>(B->ur), bunits_smem<4>(B->uc))));
  CK(cudaFuncSetAttribute(k_bunits<8>, attr,
                          (int)std::max(bunits_smem<8>(B->ur), bunits_smem<8>(B->uc))));
  B->gur = 8 * ctx->sm_count;
  B->guc = 8 * ctx->sm_count;
  B->units_ok = true;
  return PLSQR_OK;
}

// Variant v can run on this operator at block width kp: the slab form needs
// every line in ascending order, the units form its layouts (built here).
static int variant_usable(plsqr_ctx *ctx, int v, int kp, bool *ok) {
  *ok = variant_ok(v, kp);
  if (!*ok) return PLSQR_OK;
  BatchState *B = ctx->batch;
  if (kVariants[v].lpr == 0) *ok = B->lines_sorted;
  if (kVariants[v].lpr < 0) {
    int rc;
    if ((rc = batch_units(ctx))) return rc;
    *ok = B->units_ok;
  }
  return PLSQR_OK;
}

unsigned batched_check_word(bool reset) { return plsqr::check_word(reset); }

// ---- variant choice ---------------------------------------------------------
static int time_product(plsqr_ctx *ctx, BatchState *B, LaunchFn f, int mode, int reps,
                        double *ms) {
  f(ctx, *B, mode, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int i = 0; i < reps; ++i) f(ctx, *B, mode, ctx->stream);
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(ctx->ev1));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
  *ms = (double)t / reps;
  return PLSQR_OK;
}

// Variants of the two products for the current block width: the requested
// ones, else the cached choice for this operator shape and width, else the
// fastest of the candidates timed here (plain products, a few launches each).
static int batch_choose(plsqr_ctx *ctx, int want_rows, int want_cols) {
  BatchState *B = ctx->batch;
  const std::string key = B->shape + "|" + std::to_string(B->kw);
  B->tuned = 0;
  int vr = want_rows, vc = want_cols;
  if (vr < 0 || vc < 0) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      if (vr < 0) vr = it->second.first;
      if (vc < 0) vc = it->second.second;
    }
  }
  int rc;
  // a choice this operator cannot run (a cached one, made on another
  // operator of the same shape) is timed again; the units form's layouts are
  // built here, outside any graph capture
  for (int *v : {&vr, &vc}) {
    bool ok = false;
    if (*v >= 0 && (rc = variant_usable(ctx, *v, B->kw, &ok))) return rc;
    if (!ok) *v = -1;
  }
  double best_r = 1e30, best_c = 1e30;
  if (vr < 0 || vc < 0) {
    for (int v = 0; v < kNumVariants; ++v) {
      bool ok = false;
      if ((rc = variant_usable(ctx, v, B->kw, &ok))) return rc;
      if (!ok) continue;
      double t;
      if (vr < 0) {
        if ((rc = time_product(ctx, B, kVariants[v].rows, kScaleOne, 3, &t))) return rc;
        if (t < best_r) best_r = t, B->var_rows = v;
      }
      if (vc < 0) {
        if ((rc = time_product(ctx, B, kVariants[v].cols, kScaleOne, 3, &t))) return rc;
        if (t < best_c) best_c = t, B->var_cols = v;
      }
    }
    if (vr < 0) vr = B->var_rows, B->ms_rows = best_r;
    if (vc < 0) vc = B->var_cols, B->ms_cols = best_c;
    B->tuned = 1;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = std::make_pair(vr, vc);
  }
  B->var_rows = vr;
  B->var_cols = vc;
  return PLSQR_OK;
}

// ---- one inner iteration ------------------------------------------------------
static int enqueue_iteration(plsqr_ctx *ctx, BatchState *B, cudaStream_t s) {
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  kVariants[B->var_rows].rows(ctx, *B, kScaleNegAlpha, s);
  k_bscale_u<<<B->gvec, kBatchThreads, 0, s>>>(B->U, B->Uf, ctx->m_k, m, B->kw, B->cf);
  kVariants[B->var_cols].cols(ctx, *B, kScaleNegBeta, s);
  k_bupdate<<<B->gvec, kBatchThreads, 0, s>>>(B->V, B->Vf, B->W, B->DX, B->X,
                                               B->has_ref ? B->XR : nullptr, ctx->n, B->kw, B->k,
                                               B->cf, B->st, B->parts_dk, B->parts_err, 0, B->hist,
                                               B->hist_stride);
  CK(cudaGetLastError());
  return PLSQR_OK;
}

static int ensure_graph(plsqr_ctx *ctx, BatchState *B) {
  char key[256];
  snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%p/%d", B->var_rows, B->var_cols, B->kw, B->k,
           (int)B->has_ref, (void *)B->hist, B->hist_stride);
  if (B->graph && B->graph_key == key) return PLSQR_OK;
  if (B->graph) cudaGraphExecDestroy(B->graph);
  B->graph = nullptr;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_iteration(ctx, B, ctx->stream);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CK(e);
  e = cudaGraphInstantiate(&B->graph, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  B->graph_key = key;
  return PLSQR_OK;
}

// X[:, j] = 0 for the right-hand sides j whose bit is set in `mask`.
static __global__ void k_bzero_cols(double *__restrict__ x, int64_t rows, int kw,
                                    unsigned int mask) {
  const int64_t total = rows * kw;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    if ((mask >> (i % kw)) & 1u) x[i] = 0.0;
}

// ---- C ABI ----------------------------------------------------------------------
extern "C" void plsqr_default_batch_args(plsqr_batch_args *a) {
  if (!a) return;
  memset(a, 0, sizeof(*a));
  a->k = 1;
  a->sweeps = 4;
  a->inner = 50;
  a->variant_rows = -1;
  a->variant_cols = -1;
  a->atol = 1e-10;  // source/lsqr.c:47-51
  a->btol = 1e-10;
  a->conlim = 100;
}

extern "C" int plsqr_batch_variant(int32_t index, int32_t *vw, int32_t *lanes_per_line,
                                   int32_t *unroll) {
  if (index < 0 || index >= kNumVariants) return PLSQR_ERR_ARG;
  if (vw) *vw = kVariants[index].vw;
  if (lanes_per_line) *lanes_per_line = kVariants[index].lpr;
  if (unroll) *unroll = kVariants[index].u;
  return PLSQR_OK;
}

static void fill_info(const BatchState *B, plsqr_batch_info *info) {
  if (!info) return;
  memset(info, 0, sizeof(*info));
  info->k = B->k;
  info->kp = B->kw;
  info->variant_rows = B->var_rows;
  info->variant_cols = B->var_cols;
  info->tuned = B->tuned;
  info->ms_rows = B->ms_rows;
  info->ms_cols = B->ms_cols;
}

extern "C" int plsqr_batch_lsqr(plsqr_ctx *ctx, const plsqr_batch_args *a, double *x,
                                plsqr_iter *hist, plsqr_result *res, plsqr_batch_info *info) {
  if (!ctx || !a || !a->b_k) return PLSQR_ERR_ARG;
  if (a->k < 1 || a->k > kBatchMax || a->sweeps < 1 || a->inner < 1) return PLSQR_ERR_ARG;
  if (a->retire_every < 0 || !(a->retire_err >= 0.0) || (a->retire_err > 0.0 && !a->x_ref))
    return PLSQR_ERR_ARG;
  // as in the mixed solver: a damped sweep regularises the correction, not
  // the solution, so damp > 0 allows one sweep only
  if (a->damp != 0.0 && (a->sweeps > 1 || a->x0)) {
    ctx_set_error(ctx, "damp > 0 needs sweeps = 1 and no starting solution");
    return PLSQR_ERR_ARG;
  }
  const int k = a->k, kw = width_for(k);
  if ((a->variant_rows >= 0 && !variant_ok(a->variant_rows, kw)) ||
      (a->variant_cols >= 0 && !variant_ok(a->variant_cols, kw)) ||
      a->variant_rows >= kNumVariants || a->variant_cols >= kNumVariants)
    return PLSQR_ERR_ARG;
  if (a->lambda)
    for (int j = 0; j < k; ++j)
      if (!(a->lambda[j] >= 0.0) || a->lambda[j] > 1e300) return PLSQR_ERR_ARG;
  const int S = a->sweeps, I = a->inner;
  const int64_t total = (int64_t)S * I;
  if (total > (int64_t)1 << 24) return PLSQR_ERR_ARG;
  int rc;
  for (int j = 0; j < k; ++j)
    if ((rc = magnitude_ok(a->b_k + (int64_t)j * ctx->m_k, ctx->m_k)) ||
        (a->x0 && (rc = magnitude_ok(a->x0 + (int64_t)j * ctx->n, ctx->n))) ||
        (a->x_ref && (rc = magnitude_ok(a->x_ref + (int64_t)j * ctx->n, ctx->n)))) {
      ctx_set_error(ctx, "right-hand side %d: b_k, x0 or x_ref holds NaN, Inf or magnitudes "
                         "outside [2^-500, 2^500]", j);
      return rc;
    }
  CK(cudaSetDevice(ctx->opts.device));
  if ((rc = batch_prepare(ctx, kw))) return rc;
  BatchState *B = ctx->batch;
  for (const int v : {a->variant_rows, a->variant_cols}) {
    bool ok = true;
    if (v >= 0 && (rc = variant_usable(ctx, v, kw, &ok))) return rc;
    if (!ok) {
      ctx_set_error(ctx, "product variant %d cannot run on this operator (the slab form needs "
                         "every kernel row and column in ascending order, the units form "
                         "at most 64 slabs of %d rows)", v, kBUnitSlab);
      return PLSQR_ERR_ARG;
    }
  }
  B->k = k;
  B->kw = kw;
  B->has_ref = a->x_ref != nullptr;
  const int64_t n = ctx->n, mk = ctx->m_k, m = mk + ctx->m_d;
  cudaStream_t s = ctx->stream;
  const int R = a->retire_every;
  if (R > 0 && !B->tmp) {
    const size_t big = std::max(std::max((size_t)m, (size_t)n), (size_t)1);
    if ((rc = dev_alloc(ctx, &B->tmp, big * B->kp))) return rc;
  }
  // inputs: right-hand sides, weights, reference solutions
  std::vector<double> lam(kBatchMax, 1.0);
  for (int j = 0; j < k; ++j) lam[(size_t)j] = a->lambda ? a->lambda[j] : 1.0;
  CK(cudaMemcpyAsync(B->LAM, lam.data(), sizeof(double) * kBatchMax, cudaMemcpyHostToDevice, s));
  const int gl = 8 * ctx->sm_count;
  if (mk > 0) {
    CK(cudaMemcpyAsync(B->stage, a->b_k, sizeof(double) * mk * k, cudaMemcpyHostToDevice, s));
    k_bgather<<<gl, 256, 0, s>>>(B->stage, mk, mk, kw, k, B->B);
  }
  if (a->x_ref) {
    CK(cudaMemcpyAsync(B->stage, a->x_ref, sizeof(double) * n * k, cudaMemcpyHostToDevice, s));
    k_bgather<<<gl, 256, 0, s>>>(B->stage, n, n, kw, k, B->XR);
  }
  CK(cudaGetLastError());
  // starting solutions; the warm-start test needs ||b_j|| and, for the
  // history, ||x0_j - xref_j|| / ||xref_j||
  std::vector<double> bnorm((size_t)k, 0.0), err0((size_t)k, 1.0);
  unsigned int warm = 0;
  if (a->x0) {
    CK(cudaMemcpyAsync(B->stage, a->x0, sizeof(double) * n * k, cudaMemcpyHostToDevice, s));
    k_bgather<<<gl, 256, 0, s>>>(B->stage, n, n, kw, k, B->X);
    CK(cudaGetLastError());
    for (int j = 0; j < k; ++j) {
      double sb = 0.0;
      for (int64_t r = 0; r < mk; ++r) sb += a->b_k[(int64_t)j * mk + r] * a->b_k[(int64_t)j * mk + r];
      bnorm[(size_t)j] = sqrt(sb);
      if (a->x_ref) {
        double d2 = 0.0, r2 = 0.0;
        for (int64_t c = 0; c < n; ++c) {
          const double xr = a->x_ref[(int64_t)j * n + c], d = a->x0[(int64_t)j * n + c] - xr;
          d2 += d * d;
          r2 += xr * xr;
        }
        err0[(size_t)j] = r2 > 0.0 ? sqrt(d2 / r2) : 0.0;
      }
    }
    warm = k >= 32 ? 0xffffffffu : ((1u << k) - 1u);
  } else {
    CK(cudaMemsetAsync(B->X, 0, sizeof(double) * n * kw, s));
  }
  // history: [k][total + 1]
  B->hist_stride = (int)(total + 1);
  if (B->hist_cap < (int64_t)k * (total + 1)) {
    if (B->hist) dev_free(ctx, B->hist);
    B->hist = nullptr;
    B->hist_cap = 0;
    if ((rc = dev_alloc(ctx, &B->hist, (size_t)k * (total + 1)))) return rc;
    B->hist_cap = (int64_t)k * (total + 1);
  }
  CK(cudaMemsetAsync(B->hist, 0, sizeof(plsqr_iter) * k * (total + 1), s));
  // product variants: of the narrower widths a retirement may pack into
  // (cached per operator shape, else timed here, before the timed solve),
  // then of the starting width
  std::map<int, std::pair<int, int>> width_var;
  if (R > 0)
    for (int kq = 4; kq < kw; kq *= 2) {
      B->kw = kq;
      B->k = std::min(k, kq);
      // the caller's variants where they suit the narrower block
      bool okr = false, okc = false;
      if ((rc = variant_usable(ctx, a->variant_rows, kq, &okr)) ||
          (rc = variant_usable(ctx, a->variant_cols, kq, &okc)))
        return rc;
      const int vr = okr ? a->variant_rows : -1;
      const int vc = okc ? a->variant_cols : -1;
      if ((rc = batch_choose(ctx, vr, vc))) return rc;
      width_var[kq] = std::make_pair(B->var_rows, B->var_cols);
    }
  B->kw = kw;
  B->k = k;
  if ((rc = batch_choose(ctx, a->variant_rows, a->variant_cols))) return rc;
  const int tuned = B->tuned;
  const double ms_rows = B->ms_rows, ms_cols = B->ms_cols;
  width_var[kw] = std::make_pair(B->var_rows, B->var_cols);
  if ((rc = ensure_graph(ctx, B))) return rc;
  // ka right-hand sides active in a block of width kwa; block column j holds
  // the caller's right-hand side orig[j]
  int ka = k, kwa = kw;
  ColMap orig;
  for (int j = 0; j < kBatchMax; ++j) orig.c[j] = j < k ? j : 0;
  std::vector<DevState> fin((size_t)k);
  std::vector<int> fin_itn((size_t)k, -1);
  std::vector<plsqr_iter> h0((size_t)k);
  std::vector<DevState> cur((size_t)k);
  memset(h0.data(), 0, sizeof(plsqr_iter) * k);
  int last_itn = 0;
  bool finished = false;
  CK(cudaEventRecord(ctx->ev0, s));
  for (int sw = 0; sw < S && !finished; ++sw) {
   for (int attempt = 0; attempt < 2; ++attempt) {
    std::vector<DevState> h((size_t)ka);
    memset(h.data(), 0, sizeof(DevState) * ka);
    for (int j = 0; j < ka; ++j) {
      DevState &d = h[(size_t)j];
      d.damp = a->damp;
      d.atol = a->atol;
      d.btol = a->btol;
      d.ctol = a->conlim > 0.0 ? 1.0 / a->conlim : 0.0;
      d.itnlim = (int32_t)std::min<int64_t>(total + 1, INT32_MAX);
      d.has_ref = B->has_ref;
      d.cs2 = -1.0;
      d.hist_base = sw * I;
      d.slot = orig.c[j];
      d.err = -1.0;
    }
    CK(cudaMemcpyAsync(B->st, h.data(), sizeof(DevState) * ka, cudaMemcpyHostToDevice, s));
    if (B->has_ref)
      k_bref_norm<<<B->gvec, kBatchThreads, 0, s>>>(B->XR, ctx->n, kwa, ka, B->st, B->cf, B->parts);
    // outer residual and the start-up of the correction solves
    k_bresidual<<<B->gres, kBatchThreads, 0, s>>>(ctx->K.csr(), ctx->D.csr(), kwa, ka, B->X, B->B,
                                                   B->U, B->LAM, B->st, B->cf, B->parts);
    k_bscale_u<<<B->gvec, kBatchThreads, 0, s>>>(B->U, B->Uf, mk, m, kwa, B->cf);
    CK(cudaMemsetAsync(B->V, 0, sizeof(double) * n * kwa, s));
    kVariants[B->var_cols].cols(ctx, *B, kScaleZero, s);
    k_bupdate<<<B->gvec, kBatchThreads, 0, s>>>(B->V, B->Vf, B->W, B->DX, B->X, nullptr, ctx->n,
                                                 kwa, ka, B->cf, B->st, B->parts_dk, B->parts_err,
                                                 1, nullptr, 1);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(cur.data(), B->st, sizeof(DevState) * ka, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (sw == 0 && attempt == 0 && a->x0) {
      // cold start where x0 does not lower the residual: ||[b; 0] - A x0|| >= ||b||
      unsigned int cold = 0;
      for (int j = 0; j < k; ++j)
        if (!(cur[(size_t)j].beta < bnorm[(size_t)j])) cold |= 1u << j;
      if (cold) {
        warm &= ~cold;
        for (int j = 0; j < k; ++j)
          if ((cold >> j) & 1u) err0[(size_t)j] = 1.0;
        k_bzero_cols<<<gl, 256, 0, s>>>(B->X, n, kw, cold);
        CK(cudaGetLastError());
        continue;  // the start-up again, from the new X
      }
    }
    break;
   }
    bool all_done = true;
    for (int j = 0; j < ka; ++j) {
      const DevState &c = cur[(size_t)j];
      all_done = all_done && c.done;
      if (sw == 0) {
        plsqr_iter &e = h0[(size_t)orig.c[j]];
        e.alpha = c.alpha;
        e.beta = c.beta;
        e.rnorm = c.beta;
        e.arnorm = c.arnorm;
        e.test1 = 1.0;
        e.test2 = c.beta > 0.0 ? c.alpha / c.beta : 0.0;
        e.err = B->has_ref ? err0[(size_t)orig.c[j]] : -1.0;
      }
    }
    if (all_done) break;  // A^T r_j = 0 for every j: X solves every problem
    for (int i = 0; i < I;) {
      const int step = R > 0 ? std::min(R, I - i) : I;
      for (int t = 0; t < step; ++t) CK(cudaGraphLaunch(B->graph, s));
      i += step;
      last_itn = sw * I + i;
      if (R <= 0 || i == I) continue;
      // retirement: finished right-hand sides keep x = X + DX and their state
      CK(cudaMemcpyAsync(cur.data(), B->st, sizeof(DevState) * ka, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      ColMap from;
      int kn = 0;
      for (int j = 0; j < ka; ++j) {
        const DevState &c = cur[(size_t)j];
        const bool stop = c.done || (a->retire_err > 0.0 ? c.err >= 0.0 && c.err <= a->retire_err
                                                         : sw == S - 1 && c.istop != 0);
        if (!stop) {
          from.c[kn++] = j;
          continue;
        }
        const int o = orig.c[j];
        fin[(size_t)o] = c;
        fin_itn[(size_t)o] = last_itn;
        k_bput<<<gl, 256, 0, s>>>(B->X, B->DX, n, kwa, j, B->stage + (int64_t)o * n);
      }
      CK(cudaGetLastError());
      if (kn == ka) continue;
      if (kn == 0) {
        finished = true;
        ka = 0;
        break;
      }
      // pack the kn that go on into the narrowest width that holds them
      const int kq = width_for(kn);
      struct Blk {
        void *p;
        int64_t rows;
        bool f32;
      };
      const Blk blocks[] = {{B->U, m, false},   {B->V, n, false},  {B->W, n, false},
                            {B->X, n, false},   {B->DX, n, false}, {B->B, mk, false},
                            {B->XR, B->has_ref ? n : 0, false},    {B->Uf, mk, true},
                            {B->Vf, n, true}};
      for (const Blk &b : blocks) {
        if (b.rows <= 0) continue;
        const size_t bytes = (size_t)b.rows * kq * (b.f32 ? sizeof(float) : sizeof(double));
        if (b.f32)
          k_bcompact<float><<<gl, 256, 0, s>>>((const float *)b.p, (float *)B->tmp, b.rows, kwa,
                                               kq, kn, from);
        else
          k_bcompact<double><<<gl, 256, 0, s>>>((const double *)b.p, B->tmp, b.rows, kwa, kq, kn,
                                                from);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(b.p, B->tmp, bytes, cudaMemcpyDeviceToDevice, s));
      }
      std::vector<DevState> packed((size_t)kn);
      std::vector<double> lam2(kBatchMax, 1.0);
      ColMap orig2 = orig;
      for (int j = 0; j < kn; ++j) {
        packed[(size_t)j] = cur[(size_t)from.c[j]];
        lam2[(size_t)j] = lam[(size_t)from.c[j]];
        orig2.c[j] = orig.c[from.c[j]];
      }
      orig = orig2;
      lam = lam2;
      CK(cudaMemcpyAsync(B->st, packed.data(), sizeof(DevState) * kn, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(B->LAM, lam.data(), sizeof(double) * kBatchMax, cudaMemcpyHostToDevice,
                         s));
      CK(cudaStreamSynchronize(s));  // the host vectors above are reused
      ka = kn;
      kwa = kq;
      B->k = ka;
      B->kw = kwa;
      B->var_rows = width_var.at(kwa).first;
      B->var_cols = width_var.at(kwa).second;
      if ((rc = ensure_graph(ctx, B))) return rc;
    }
    if (finished) break;
    k_badd<<<gl, 256, 0, s>>>(B->X, B->DX, n * kwa);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(ctx->ev1, s));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  if (ka > 0)
    CK(cudaMemcpyAsync(cur.data(), B->st, sizeof(DevState) * ka, cudaMemcpyDeviceToHost, s));
  if (hist) {
    CK(cudaMemcpyAsync(hist, B->hist, sizeof(plsqr_iter) * k * (total + 1), cudaMemcpyDeviceToHost,
                       s));
  }
  if (ka > 0) {
    k_bscatter<<<gl, 256, 0, s>>>(B->X, n, kwa, ka, orig, B->stage, n);
    CK(cudaGetLastError());
  }
  if (x) CK(cudaMemcpyAsync(x, B->stage, sizeof(double) * n * k, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int j = 0; j < ka; ++j) {
    fin[(size_t)orig.c[j]] = cur[(size_t)j];
    fin_itn[(size_t)orig.c[j]] = last_itn;
  }
  if (hist)
    for (int j = 0; j < k; ++j) hist[(int64_t)j * (total + 1)] = h0[(size_t)j];
  if (res) {
    for (int j = 0; j < k; ++j) {
      const DevState &c = fin[(size_t)j];
      plsqr_result &r = res[j];
      memset(&r, 0, sizeof(r));
      r.istop = c.istop;
      r.itn = fin_itn[(size_t)j];
      r.anorm = c.anorm;
      r.acond = c.acond;
      r.rnorm = c.rnorm;
      r.arnorm_out = c.test2;
      r.xnorm = c.xnorm;
      r.arnorm = c.arnorm;
      r.bnorm = c.bnorm;
      r.dxmax = c.dxmax;
      r.maxdx = c.maxdx;
      r.warm = (int32_t)((warm >> j) & 1u);
      r.seconds = ms * 1e-3;
      r.seconds_total = r.seconds;
    }
  }
  B->tuned = tuned;
  B->ms_rows = ms_rows;
  B->ms_cols = ms_cols;
  B->var_rows = width_var.at(kw).first;
  B->var_cols = width_var.at(kw).second;
  B->k = k;
  B->kw = kw;
  fill_info(B, info);
  if (info) info->warm = (int32_t)warm;
  return PLSQR_OK;
}

extern "C" int plsqr_batch_bench_aprod(plsqr_ctx *ctx, int32_t k, int mode, int32_t variant,
                                       int reps, double *ms_per_launch) {
  if (!ctx || !ms_per_launch || k < 1 || k > kBatchMax || (mode != 1 && mode != 2) || reps < 1)
    return PLSQR_ERR_ARG;
  const int kw = width_for(k);
  if (variant >= 0 && !variant_ok(variant, kw)) return PLSQR_ERR_ARG;
  if (variant >= kNumVariants) return PLSQR_ERR_ARG;
  CK(cudaSetDevice(ctx->opts.device));
  int rc;
  if ((rc = batch_prepare(ctx, kw))) return rc;
  BatchState *B = ctx->batch;
  B->k = k;
  B->kw = kw;
  if (variant < 0) {
    if ((rc = batch_choose(ctx, -1, -1))) return rc;
    variant = mode == 1 ? B->var_rows : B->var_cols;
  }
  bool ok = false;
  if ((rc = variant_usable(ctx, variant, kw, &ok))) return rc;
  if (!ok) return PLSQR_ERR_ARG;
  const Variant &V = kVariants[variant];
  return time_product(ctx, B, mode == 1 ? V.rows : V.cols, kScaleOne, reps, ms_per_launch);
}

// ---- damping weight ---------------------------------------------------------------
static __global__ void k_weighted(const double *__restrict__ src, int64_t n, double w,
                                  double *__restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = w == 1.0 ? src[i] : __dmul_rn(w, src[i]);
}

extern "C" int plsqr_set_damping_weight(plsqr_ctx *ctx, double lambda) {
  if (!ctx || !(lambda >= 0.0) || lambda > 1e300) return PLSQR_ERR_ARG;
  CK(cudaSetDevice(ctx->opts.device));
  int rc;
  if (!ctx->d_val0) {
    if ((rc = dev_alloc(ctx, &ctx->d_val0, (size_t)ctx->nnz_d)) ||
        (rc = dev_alloc(ctx, &ctx->dc_val0, (size_t)ctx->nnz_d)))
      return rc;
    CK(cudaMemcpyAsync(ctx->d_val0, ctx->D.val, sizeof(double) * ctx->nnz_d,
                       cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->dc_val0, ctx->DC.val, sizeof(double) * ctx->nnz_d,
                       cudaMemcpyDeviceToDevice, ctx->stream));
  }
  const int g = 4 * ctx->sm_count;
  k_weighted<<<g, 256, 0, ctx->stream>>>(ctx->d_val0, ctx->nnz_d, lambda, ctx->D.val);
  k_weighted<<<g, 256, 0, ctx->stream>>>(ctx->dc_val0, ctx->nnz_d, lambda, ctx->DC.val);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return PLSQR_OK;
}
