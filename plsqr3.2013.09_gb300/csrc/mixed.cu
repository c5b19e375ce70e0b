// Mixed-precision LSQR: iterative refinement with FP32 inner sweeps.
//
//   x = 0
//   repeat `sweeps` times:
//     r  = [b_k; 0] - A x                   FP64, kernel values hi + lo
//     dx = LSQR(A_hi, r), `inner` iterations FP32 vectors, FP64 scalars/norms
//     x += dx                               FP64
//
// The least-squares correction problem min ||A dx - r|| has the solution
// x* - x, so every sweep contracts the error by the factor the inner sweep
// reaches.  The inner iteration is the five-kernel iteration of the FP64
// solver with FP32 vectors and 8-byte kernel nonzeros (kernels_f32.cuh),
// captured once as a CUDA graph.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "kernels_f32.cuh"
#include "plsqr_internal.h"
#include "slab.cuh"

using namespace plsqr;

namespace {
constexpr int kThreads = 256;
}

struct MixedState {
  float *k_hi = nullptr, *k_lo = nullptr, *kc_hi = nullptr;
  // FP32 layouts of the high half of the split (6 bytes per nonzero) used by
  // the inner sweeps: the unit layout (default) or the slab layout
  bool slabs = false;  // either layout: slab partials added by the combine kernels
  bool units = false;
  DevSlab<float> s_rows, s_cols;
  DevUnitsT<float> u_rows, u_cols;
  // the unit products gather the FP32 pairs (mirror, mirror_lo) with
  // error-free products and sums (units.cuh; PLSQR_MIXED_HILO=0: the mirror
  // alone)
  bool hilo = false;
  float *uf_lo = nullptr, *vf_lo = nullptr;
  float *uf = nullptr, *vf = nullptr, *wf = nullptr, *dxf = nullptr;
  double *dx = nullptr;  // FP64 correction of the FP64-vector inner sweeps
  bool v64 = false;      // inner sweeps keep u, v, w, dx in FP64 (slab products in FP32)
  double *b = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_key = -1;
  plsqr_iter *graph_hist = nullptr;
};

#define CK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      ctx_set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call,              \
                    cudaGetErrorString(e_));                                     \
      return PLSQR_ERR_CUDA;                                                     \
    }                                                                            \
  } while (0)

void mixed_free(plsqr_ctx *ctx) {
  if (!ctx || !ctx->mixed) return;
  if (ctx->mixed->graph) cudaGraphExecDestroy(ctx->mixed->graph);
  delete ctx->mixed;  // device buffers are in ctx->allocs
  ctx->mixed = nullptr;
}

int mixed_prepare(plsqr_ctx *ctx) {
  if (ctx->mixed) return PLSQR_OK;
  ctx->mixed = new MixedState();
  MixedState *M = ctx->mixed;
  int rc;
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  if ((rc = dev_alloc(ctx, &M->k_hi, (size_t)ctx->nnz_k)) ||
      (rc = dev_alloc(ctx, &M->k_lo, (size_t)ctx->nnz_k)) ||
      (rc = dev_alloc(ctx, &M->kc_hi, (size_t)ctx->nnz_k)) ||
      (rc = dev_alloc(ctx, &M->uf, (size_t)m)) || (rc = dev_alloc(ctx, &M->vf, (size_t)ctx->n)) ||
      (rc = dev_alloc(ctx, &M->wf, (size_t)ctx->n)) ||
      (rc = dev_alloc(ctx, &M->dxf, (size_t)ctx->n)) || (rc = dev_alloc(ctx, &M->dx, (size_t)ctx->n)) ||
      (rc = dev_alloc(ctx, &M->b, (size_t)std::max(ctx->m_k, 1))))
    return rc;
  const int g = ctx->sm_count * 8;
  k_split_hilo<<<g, 256, 0, ctx->stream>>>(ctx->K.val, ctx->nnz_k, M->k_hi, M->k_lo);
  k_split_hilo<<<g, 256, 0, ctx->stream>>>(ctx->KC.val, ctx->nnz_k, M->kc_hi, nullptr);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->slab_ok) {
    // the unit layout on slabs of 49,152 FP32 values (192 KB, one 1,024-thread
    // block per SM) unless PLSQR_MIXED_UNITS=0; PLSQR_UNIT_SIZE_F sets the slab
    // hi + lo mirrors with error-free products and sums unless
    // PLSQR_MIXED_HILO=0: on the 96x96x32 problem 381 inner iterations to
    // 1e-6 (FP64: 376) at 2.62 ms against 422 at 2.48 ms with the plain FP32
    // mirror, whose rounding, and the products', the solver otherwise pays
    // for in iterations
    const char *eh = getenv("PLSQR_MIXED_HILO");
    const bool hilo = !(eh && atoi(eh) == 0);
    int uslab = hilo ? 24576 : 49152;  // 192 KB of FP32 pairs or of FP32 values
    if (const char *e = getenv("PLSQR_UNIT_SIZE_F"))
      if (atoi(e) >= 1024) uslab = atoi(e);
    bool units = units_fit<float>(ctx->n, uslab, hilo) && units_fit<float>(ctx->m_k, uslab, hilo);
    if (const char *e = getenv("PLSQR_MIXED_UNITS"))
      if (atoi(e) == 0) units = false;
    if (units) {
      if ((rc = build_units<float>(ctx, ctx->K, ctx->n, uslab, &M->u_rows, hilo)) ||
          (rc = build_units<float>(ctx, ctx->KC, ctx->m_k, uslab, &M->u_cols, hilo)))
        return rc;
      if (hilo) {
        if ((rc = dev_alloc(ctx, &M->uf_lo, (size_t)m)) ||
            (rc = dev_alloc(ctx, &M->vf_lo, (size_t)ctx->n)))
          return rc;
        CK(cudaMemsetAsync(M->uf_lo, 0, sizeof(float) * m, ctx->stream));
        CK(cudaMemsetAsync(M->vf_lo, 0, sizeof(float) * ctx->n, ctx->stream));
      }
      M->hilo = hilo;
      if ((rc = units_set_smem<float>(std::max(M->u_rows.smem, M->u_cols.smem)))) return rc;
      M->units = true;
    } else {
      int slab = 24576;  // 96 KB of FP32 per block: two blocks per SM
      if (const char *e = getenv("PLSQR_SLAB_SIZE_F"))
        if (atoi(e) >= 1024 && atoi(e) <= 57344) slab = atoi(e);
      // kernel rows: mostly consecutive columns, read by the lanes of a
      // group in step (transposed chunks); columns: random rows, as stored
      const int dyn = slab_dyn_blocks(ctx, true);
      if ((rc = build_slab<float>(ctx, ctx->K, ctx->n, slab, 16 * ctx->sm_count, &M->s_rows,
                                  ctx->slab_group_f, dyn)) ||
          (rc = build_slab<float>(ctx, ctx->KC, ctx->m_k, slab, 16 * ctx->sm_count, &M->s_cols,
                                  0, dyn)))
        return rc;
      if ((rc = slab_set_smem<float>(std::max(M->s_rows.smem, M->s_cols.smem)))) return rc;
    }
    M->slabs = true;
    const char *e = getenv("PLSQR_MIXED_F32VEC");
    M->v64 = !(e && atoi(e) == 1);
  }
  return PLSQR_OK;
}

// partial-sum counts of the inner products (slab combine grids or per-line grids)
static int pu_k(const plsqr_ctx *ctx) { return ctx->mixed->slabs ? ctx->gc1k : ctx->g1k * (kThreads / 32); }
static int pu_d(const plsqr_ctx *ctx) { return ctx->mixed->slabs ? ctx->gc1d : ctx->g1d; }
static int pv(const plsqr_ctx *ctx) { return ctx->mixed->slabs ? ctx->gc2 : ctx->g2; }

static CsrF rows_hilo(const plsqr_ctx *ctx) {
  return CsrF{ctx->K.ptr, ctx->K.idx, ctx->mixed->k_hi, ctx->mixed->k_lo, ctx->K.n_lines};
}
static CsrT<float> rows_f(const plsqr_ctx *ctx) {
  return CsrT<float>{ctx->K.ptr, ctx->K.idx, ctx->mixed->k_hi, ctx->K.n_lines};
}
static CsrT<float> cols_f(const plsqr_ctx *ctx) {
  return CsrT<float>{ctx->KC.ptr, ctx->KC.idx, ctx->mixed->kc_hi, ctx->KC.n_lines};
}
// The inner sweeps' products.  The FP32 kernel part into slab partials (K v_f
// per slab of v_f, K^T u_f per slab of u_f): on the unit layout (FP64
// partials: each line's slab sum kept to FP64, a rounding to FP32 there cost
// as many iterations as the FP32 mirror) or the slab layout (FP32
// partials); then the combine kernel with the damping part and the scaling,
// into the FP32 vectors (m1f, m2f) or the FP64 ones (m1v, m2v).  Without
// slabs: the per-line kernels instantiated for FP32.
template <typename TV>
static void combine_rows(plsqr_ctx *ctx, cudaStream_t s, const TV *v, TV *u, int mode) {
  MixedState *M = ctx->mixed;
  const int g = ctx->gc1k + ctx->gc1d;
  if (M->units) {
    units_spmv(M->u_rows, M->vf, s, M->hilo && M->v64 ? M->vf_lo : nullptr);
    k_combine_rows<double, TV, kThreads><<<g, kThreads, 0, s>>>(
        M->u_rows.partial, M->u_rows.n_slabs, ctx->m_k, ctx->D.csr(), v, u, ctx->gc1k, mode,
        ctx->st, ctx->parts_u);
  } else {
    slab_spmv(M->s_rows, ctx->slab_group_f, M->vf, s);
    k_combine_rows<float, TV, kThreads><<<g, kThreads, 0, s>>>(
        M->s_rows.partial, M->s_rows.n_slabs, ctx->m_k, ctx->D.csr(), v, u, ctx->gc1k, mode,
        ctx->st, ctx->parts_u);
  }
}
template <typename TV>
static void combine_cols(plsqr_ctx *ctx, cudaStream_t s, const TV *u, TV *v, int mode) {
  MixedState *M = ctx->mixed;
  if (M->units) {
    units_spmv(M->u_cols, M->uf, s, M->hilo && M->v64 ? M->uf_lo : nullptr);
    k_combine_cols<double, TV, kThreads><<<ctx->gc2, kThreads, 0, s>>>(
        M->u_cols.partial, M->u_cols.n_slabs, ctx->n, ctx->DC.csr(), u, ctx->m_k, v, mode, ctx->st,
        ctx->parts_v);
  } else {
    slab_spmv(M->s_cols, ctx->slab_group_f, M->uf, s);
    k_combine_cols<float, TV, kThreads><<<ctx->gc2, kThreads, 0, s>>>(
        M->s_cols.partial, M->s_cols.n_slabs, ctx->n, ctx->DC.csr(), u, ctx->m_k, v, mode, ctx->st,
        ctx->parts_v);
  }
}

static void m1f(plsqr_ctx *ctx, cudaStream_t s) {
  MixedState *M = ctx->mixed;
  if (M->slabs) {
    combine_rows<float>(ctx, s, M->vf, M->uf, kScaleNegAlpha);
    return;
  }
  k_aprod1<float, kThreads, 2><<<ctx->g1k + ctx->g1d, kThreads, 0, s>>>(
      rows_f(ctx), ctx->D.csr(), ctx->kpart, M->vf, M->uf, ctx->g1k, kScaleNegAlpha, ctx->st,
      ctx->parts_u);
}
static void m2f(plsqr_ctx *ctx, cudaStream_t s, int mode) {
  MixedState *M = ctx->mixed;
  if (M->slabs) {
    combine_cols<float>(ctx, s, M->uf, M->vf, mode);
    return;
  }
  k_aprod2<float, kThreads, 2><<<ctx->g2, kThreads, 0, s>>>(
      cols_f(ctx), ctx->DC.csr(), ctx->cpart, ctx->corder, M->uf, ctx->m_k, M->vf, mode, ctx->st,
      ctx->parts_v);
}

// FP64-vector inner sweeps: the products read the FP32 mirrors of v and u
// (written by the scaling kernels) and combine the partials into the FP64
// vectors.
static void m1v(plsqr_ctx *ctx, cudaStream_t s, int mode) {
  combine_rows<double>(ctx, s, ctx->v, ctx->u, mode);
}
static void m2v(plsqr_ctx *ctx, cudaStream_t s, int mode) {
  combine_cols<double>(ctx, s, ctx->u, ctx->v, mode);
}

static int enqueue_inner64(plsqr_ctx *ctx, cudaStream_t s) {
  MixedState *M = ctx->mixed;
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  const double *xref = ctx->has_ref ? ctx->xref : nullptr;
  m1v(ctx, s, kScaleNegAlpha);
  k_norm_u<double, kThreads><<<ctx->gvu, kThreads, 0, s>>>(ctx->u, m, ctx->parts_u, ctx->gc1k,
                                                           ctx->gc1d, ctx->st, 0, M->uf, M->uf_lo);
  m2v(ctx, s, kScaleNegBeta);
  k_update_x<kThreads><<<ctx->gvx, kThreads, 0, s>>>(
      ctx->v, ctx->w, M->dx, nullptr, xref, ctx->n, ctx->parts_v, ctx->gc2, ctx->st, ctx->parts_dk,
      xref ? ctx->parts_err : nullptr, ctx->hist, 0, M->vf, ctx->x, M->vf_lo);
  k_tail<kThreads><<<1, kThreads, 0, s>>>(ctx->st, ctx->parts_dk, xref ? ctx->parts_err : nullptr,
                                           ctx->gvx, ctx->x, ctx->hist);
  CK(cudaGetLastError());
  return PLSQR_OK;
}

static __global__ void k_add_vec(double *__restrict__ x, const double *__restrict__ dx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += dx[i];
}

static int enqueue_inner(plsqr_ctx *ctx, cudaStream_t s) {
  if (ctx->mixed->v64) return enqueue_inner64(ctx, s);
  MixedState *M = ctx->mixed;
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  const double *xref = ctx->has_ref ? ctx->xref : nullptr;
  m1f(ctx, s);
  k_norm_u<float, kThreads><<<ctx->gvu, kThreads, 0, s>>>(M->uf, m, ctx->parts_u, pu_k(ctx),
                                                          pu_d(ctx), ctx->st, 0);
  m2f(ctx, s, kScaleNegBeta);
  k_update_dx_f32<kThreads><<<ctx->gvx, kThreads, 0, s>>>(
      M->vf, M->wf, M->dxf, ctx->x, xref, ctx->n, ctx->parts_v, pv(ctx), ctx->st, ctx->parts_dk,
      xref ? ctx->parts_err : nullptr, 0);
  k_tail<kThreads><<<1, kThreads, 0, s>>>(ctx->st, ctx->parts_dk, xref ? ctx->parts_err : nullptr,
                                           ctx->gvx, ctx->x, ctx->hist);
  CK(cudaGetLastError());
  return PLSQR_OK;
}

static int ensure_inner_graph(plsqr_ctx *ctx) {
  MixedState *M = ctx->mixed;
  const int key = (ctx->has_ref ? 1 : 0) | (M->v64 ? 2 : 0);
  if (M->graph && M->graph_key == key && M->graph_hist == ctx->hist) return PLSQR_OK;
  if (M->graph) cudaGraphExecDestroy(M->graph);
  M->graph = nullptr;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_inner(ctx, ctx->stream);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CK(e);
  e = cudaGraphInstantiate(&M->graph, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  M->graph_key = key;
  M->graph_hist = ctx->hist;
  return PLSQR_OK;
}

int mixed_lsqr(plsqr_ctx *ctx, const plsqr_lsqr_args *args, const double *b_k, double *x,
               double *w, double *se, plsqr_iter *hist, plsqr_result *res) {
  (void)w;
  (void)se;
  if (args->sweeps < 1 || args->inner < 1 || args->want_se) return PLSQR_ERR_ARG;
  // A sweep solves for the correction dx with damp^2 ||dx||^2, not
  // damp^2 ||x + dx||^2, so damped refinement past the first sweep would
  // solve another problem: refuse it.
  if (args->damp != 0.0 && args->sweeps > 1) {
    ctx_set_error(ctx, "damp > 0 needs sweeps = 1 (refinement sweeps would regularise the "
                       "correction instead of the solution)");
    return PLSQR_ERR_ARG;
  }
  const double *x0 = args->x0;
  if (x0 && args->damp != 0.0) {
    ctx_set_error(ctx, "x0 needs damp = 0 (damping would regularise the correction)");
    return PLSQR_ERR_ARG;
  }
  int rc;
  if ((rc = mixed_prepare(ctx))) return rc;
  MixedState *M = ctx->mixed;
  const double *b = b_k;
  if (!b) {
    if ((int32_t)ctx->b_k.size() != ctx->m_k) return PLSQR_ERR_STATE;
    b = ctx->b_k.data();
  }
  if ((rc = magnitude_ok(b, ctx->m_k)) || (x0 && (rc = magnitude_ok(x0, ctx->n)))) {
    ctx_set_error(ctx, "b_k or x0 holds NaN, Inf or magnitudes outside [2^-500, 2^500]");
    return rc;
  }
  CK(cudaSetDevice(ctx->opts.device));
  const int S = args->sweeps, I = args->inner;
  const int total = S * I;
  if (ctx->hist_cap < total + 1) {
    if (ctx->hist) dev_free(ctx, ctx->hist);
    ctx->hist = nullptr;
    if ((rc = dev_alloc(ctx, &ctx->hist, (size_t)total + 1))) return rc;
    ctx->hist_cap = total + 1;
  }
  if (ctx->m_k > 0)
    CK(cudaMemcpyAsync(M->b, b, sizeof(double) * ctx->m_k, cudaMemcpyHostToDevice, ctx->stream));
  // ||[b; 0]||, the residual norm of the cold start, for the warm-start test
  double bnorm = 0.0;
  if (x0) {
    for (int32_t i = 0; i < ctx->m_k; ++i) bnorm += b[i] * b[i];
    bnorm = sqrt(bnorm);
    CK(cudaMemcpyAsync(ctx->x, x0, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->stream));
  } else {
    CK(cudaMemsetAsync(ctx->x, 0, sizeof(double) * ctx->n, ctx->stream));
  }
  CK(cudaMemsetAsync(ctx->hist, 0, sizeof(plsqr_iter) * (total + 1), ctx->stream));
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  std::vector<plsqr_iter> hh((size_t)total + 1);
  DevState cur;
  memset(&cur, 0, sizeof(cur));
  int done_sweeps = 0, last_itn = 0;
  if ((rc = ensure_inner_graph(ctx))) return rc;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int s = 0; s < S; ++s) {
    DevState h;
    memset(&h, 0, sizeof(h));
    h.damp = args->damp;
    h.atol = args->atol;
    h.btol = args->btol;
    h.ctol = args->conlim > 0.0 ? 1.0 / args->conlim : 0.0;
    h.itnlim = args->itnlim;
    h.has_ref = ctx->has_ref;
    h.cs2 = -1.0;
    h.hist_base = s * I;
    CK(cudaMemcpyAsync(ctx->st, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->has_ref) k_ref_norm<kThreads><<<1, kThreads, 0, ctx->stream>>>(ctx->xref, ctx->n, ctx->st);
    // outer residual and the start-up of the inner solve
    k_residual<kThreads><<<ctx->g1k + ctx->g1d, kThreads, 0, ctx->stream>>>(
        rows_hilo(ctx), ctx->D.csr(), ctx->kpart, ctx->x, M->b, ctx->u, ctx->g1k, ctx->parts_u);
    if (M->v64) {
      // FP64-vector inner solve: scaled r and its FP32 mirror, v = A^T u
      k_norm_u<double, kThreads><<<ctx->gvu, kThreads, 0, ctx->stream>>>(
          ctx->u, m, ctx->parts_u, ctx->g1k, ctx->g1d, ctx->st, 1, M->uf, M->uf_lo);
      CK(cudaMemsetAsync(ctx->v, 0, sizeof(double) * ctx->n, ctx->stream));
      m2v(ctx, ctx->stream, kScaleZero);
      k_update_x<kThreads><<<ctx->gvx, kThreads, 0, ctx->stream>>>(
          ctx->v, ctx->w, M->dx, nullptr, nullptr, ctx->n, ctx->parts_v, ctx->gc2, ctx->st,
          ctx->parts_dk, nullptr, nullptr, 1, M->vf, nullptr, M->vf_lo);
    } else {
      k_norm_u<double, kThreads><<<ctx->gvu, kThreads, 0, ctx->stream>>>(
          ctx->u, m, ctx->parts_u, ctx->g1k, ctx->g1d, ctx->st, 1);
      k_to_f32<<<ctx->gvu, kThreads, 0, ctx->stream>>>(ctx->u, m, M->uf);
      m2f(ctx, ctx->stream, kScaleZero);
      k_update_dx_f32<kThreads><<<ctx->gvx, kThreads, 0, ctx->stream>>>(
          M->vf, M->wf, M->dxf, ctx->x, nullptr, ctx->n, ctx->parts_v, pv(ctx), ctx->st,
          ctx->parts_dk, nullptr, 1);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&cur, ctx->st, sizeof(cur), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (s == 0 && x0 && !(cur.beta < bnorm)) {
      // x0 does not lower the residual: start again from x = 0
      x0 = nullptr;
      CK(cudaMemsetAsync(ctx->x, 0, sizeof(double) * ctx->n, ctx->stream));
      s = -1;
      continue;
    }
    if (s == 0) {
      plsqr_iter &h0 = hh[0];
      h0.alpha = cur.alpha;
      h0.beta = cur.beta;
      h0.rnorm = cur.beta;
      h0.arnorm = cur.arnorm;
      h0.test1 = 1.0;
      h0.test2 = cur.beta > 0.0 ? cur.alpha / cur.beta : 0.0;
      h0.err = ctx->has_ref ? 1.0 : -1.0;
      if (ctx->has_ref && x0) {  // the start is x0: its distance to the reference
        std::vector<double> xr((size_t)ctx->n);
        CK(cudaMemcpy(xr.data(), ctx->xref, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost));
        double d = 0.0, r2 = 0.0;
        for (int32_t i = 0; i < ctx->n; ++i) {
          d += (x0[i] - xr[(size_t)i]) * (x0[i] - xr[(size_t)i]);
          r2 += xr[(size_t)i] * xr[(size_t)i];
        }
        h0.err = r2 > 0.0 ? sqrt(d / r2) : sqrt(d);
      }
    }
    if (cur.done) break;  // A^T r = 0: x is a least-squares solution
    for (int i = 0; i < I; ++i) CK(cudaGraphLaunch(M->graph, ctx->stream));
    if (M->v64)
      k_add_vec<<<ctx->gvx, kThreads, 0, ctx->stream>>>(ctx->x, M->dx, ctx->n);
    else
      k_add_dx<<<ctx->gvx, kThreads, 0, ctx->stream>>>(ctx->x, M->dxf, ctx->n);
    CK(cudaGetLastError());
    done_sweeps = s + 1;
    last_itn = (s + 1) * I;
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  CK(cudaMemcpyAsync(&cur, ctx->st, sizeof(cur), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(hh.data() + 1, ctx->hist + 1, sizeof(plsqr_iter) * total,
                     cudaMemcpyDeviceToHost, ctx->stream));
  if (x) CK(cudaMemcpyAsync(x, ctx->x, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->solved = true;
  (void)done_sweeps;
  plsqr_result r;
  memset(&r, 0, sizeof(r));
  r.istop = cur.istop;
  r.itn = last_itn;
  r.anorm = cur.anorm;
  r.acond = cur.acond;
  r.rnorm = cur.rnorm;
  r.arnorm_out = cur.test2;
  r.xnorm = cur.xnorm;
  r.arnorm = cur.arnorm;
  r.bnorm = cur.bnorm;
  r.dxmax = cur.dxmax;
  r.maxdx = cur.maxdx;
  r.warm = x0 ? 1 : 0;
  r.seconds = ms * 1e-3;
  r.seconds_total = r.seconds;
  if (res) *res = r;
  if (hist) memcpy(hist, hh.data(), sizeof(plsqr_iter) * (total + 1));
  return PLSQR_OK;
}

int mixed_bench_aprod(plsqr_ctx *ctx, int mode, int reps, double *ms_per_launch) {
  int rc;
  if ((rc = mixed_prepare(ctx))) return rc;
  CK(cudaSetDevice(ctx->opts.device));
  const bool v64 = ctx->mixed->v64;
  auto launch = [&]() {
    if (v64 && mode == 1)
      m1v(ctx, ctx->stream, kScaleOne);
    else if (v64)
      m2v(ctx, ctx->stream, kScaleZero);
    else if (mode == 1)
      m1f(ctx, ctx->stream);
    else
      m2f(ctx, ctx->stream, kScaleZero);
  };
  // a state with beta > 0 and alpha = 0 so that both kernels run fully
  DevState h;
  memset(&h, 0, sizeof(h));
  h.s_beta_pos = 1;
  h.beta = 1.0;
  CK(cudaMemcpy(ctx->st, &h, sizeof(h), cudaMemcpyHostToDevice));
  launch();
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int i = 0; i < reps; ++i) launch();
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *ms_per_launch = (double)ms / reps;
  return PLSQR_OK;
}

int mixed_bench_iteration(plsqr_ctx *ctx, int reps, double *ms_per_iteration) {
  if (!ctx->solved || !ctx->mixed) return PLSQR_ERR_STATE;
  CK(cudaSetDevice(ctx->opts.device));
  int rc;
  if (ctx->hist_cap < reps + 1) {
    dev_free(ctx, ctx->hist);
    ctx->hist = nullptr;
    ctx->hist_cap = 0;
    if ((rc = dev_alloc(ctx, &ctx->hist, (size_t)reps + 1))) return rc;
    ctx->hist_cap = reps + 1;
  }
  if ((rc = ensure_inner_graph(ctx))) return rc;
  DevState h;
  CK(cudaMemcpy(&h, ctx->st, sizeof(h), cudaMemcpyDeviceToHost));
  h.itn = 0;
  h.hist_base = 0;
  CK(cudaMemcpy(ctx->st, &h, sizeof(h), cudaMemcpyHostToDevice));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int i = 0; i < reps; ++i) CK(cudaGraphLaunch(ctx->mixed->graph, ctx->stream));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *ms_per_iteration = (double)ms / reps;
  return PLSQR_OK;
}
