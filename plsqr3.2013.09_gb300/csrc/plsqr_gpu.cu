// GB300 PLSQR3: device context, the aprod operator and the LSQR driver
// behind the C ABI of include/plsqr_gpu.h.
//
// One context holds the operator in four layouts (kernel and damping matrix,
// by row and by column; the kernel rows are built on the device from the
// by-column input), the LSQR vectors u = [y_k; y_d], v, w, x (and se), the
// scalar state and the per-iteration history, all in device memory.  One LSQR
// iteration is five kernels (kernels_fp64.cuh) captured once as a CUDA graph
// and replayed; the host only enqueues graph launches and reads results back
// at the end.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "kernels_exact.cuh"
#include "kernels_fp64.cuh"
#include "plsqr_internal.h"
#include "slab.cuh"
#include "transpose.cuh"
#include "units.cuh"

using namespace plsqr;

namespace {

constexpr int kThreads = 256;

// The regions of one iteration for the timing report and the NVTX ranges,
// named after the reference's GPTL timers (source/lsqr.c:500-642,
// aprod_impl.c:69-497); each lists the reference timers whose work it holds
// (the products fuse the reference's scaling passes into their epilogues).
constexpr int kRegions = 5;
const char *const kRegionName[kRegions] = {"spmv", "norm1", "spmvT", "update_x", "krylov_p1"};
const char *const kRegionCovers[kRegions] = {
    "scale1 (u *= -alpha), spmv_ker, spmv_damp",
    "norm1 (beta), scale2 (u *= 1/beta)",
    "scale1 (v *= -beta), spmvT_ker, spmvT_damp",
    "norm1 (alpha), scale3 (v *= 1/alpha), krylov_p1 (rotation, x and w update)",
    "krylov_p1 (dknorm, scalar recurrence, history record)"};

const char *const kErrText[] = {
    "success",
    "invalid argument or size",
    "file cannot be opened, read or written",
    "file or matrix content is inconsistent",
    "host allocation failed",
    "CUDA runtime error",
    "no usable CUDA device",
    "call out of sequence",
    "a bounded device wait gave up",
    "internal consistency check failed",
    "NaN, Inf or out-of-range magnitude in an input (|value| above 2^500, or a vector all below "
    "2^-500)",
};

}  // namespace

#define CK(call)                                                               \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ctx_set_error(ctx, "%s:%d %s: %s", __FILE__, __LINE__, #call,            \
                    cudaGetErrorString(e_));                                   \
      return PLSQR_ERR_CUDA;                                                   \
    }                                                                          \
  } while (0)

void ctx_set_error(plsqr_ctx *ctx, const char *fmt, ...) {
  if (!ctx) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(ctx->last_error, sizeof(ctx->last_error), fmt, ap);
  va_end(ap);
}

int ctx_dev_alloc_bytes(plsqr_ctx *ctx, void **p, size_t bytes) {
  *p = nullptr;
  CK(cudaMalloc(p, bytes));
  ctx->allocs.emplace_back(*p, bytes);
  ctx->device_bytes += (int64_t)bytes;
  return PLSQR_OK;
}

void ctx_dev_free(plsqr_ctx *ctx, void *p) {
  if (!p) return;
  for (size_t i = 0; i < ctx->allocs.size(); ++i)
    if (ctx->allocs[i].first == p) {
      ctx->device_bytes -= (int64_t)ctx->allocs[i].second;
      ctx->allocs.erase(ctx->allocs.begin() + (long)i);
      break;
    }
  cudaFree(p);
}

// ---------------------------------------------------------------------------
// host-side validation of a compressed sparse matrix (no device fault can
// come from a bad index: every index is checked before upload)
// The norms are plain FP64 sums of squares (the reference's cblas_dnrm2,
// source/mycblas.c:182-222, rescales as it goes): a vector whose largest
// magnitude is above 2^500, or nonzero but below 2^-500, would overflow or
// underflow them, and is refused, as are NaN and Inf.  Matrix values
// (allow_small = 1) are refused only above 2^500: the products of small
// values underflow in the reference's sums alike.
int magnitude_ok(const double *p, int64_t n, int allow_small) {
  double mx = 0.0;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(max : mx) reduction(| : bad)
  for (int64_t i = 0; i < n; ++i) {
    const double a = fabs(p[i]);
    if (!(a <= 1.7976931348623157e308)) bad = 1;  // NaN or Inf
    else if (a > mx) mx = a;
  }
  if (bad || mx > 0x1p500 || (!allow_small && mx > 0.0 && mx < 0x1p-500)) return PLSQR_ERR_NUMERIC;
  return PLSQR_OK;
}

static int validate_sparse(const plsqr_sparse *a, int32_t rows, int32_t cols, int by_col,
                           std::vector<int64_t> &ptr64) {
  if (!a || (!a->ptr32 && !a->ptr64) || (a->ptr32 && a->ptr64)) return PLSQR_ERR_ARG;
  if (a->num_row != rows || a->num_col != cols || a->nnz < 0) return PLSQR_ERR_ARG;
  const int32_t n_lines = by_col ? cols : rows, n_idx = by_col ? rows : cols;
  ptr64.resize((size_t)n_lines + 1);
  for (int32_t i = 0; i <= n_lines; ++i) ptr64[i] = a->ptr32 ? (int64_t)a->ptr32[i] : a->ptr64[i];
  if (ptr64[0] != 0 || ptr64[n_lines] != a->nnz) return PLSQR_ERR_FORMAT;
  for (int32_t i = 0; i < n_lines; ++i)
    if (ptr64[i + 1] < ptr64[i]) return PLSQR_ERR_FORMAT;
  if (a->nnz > 0 && (!a->idx || !a->val)) return PLSQR_ERR_ARG;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t e = 0; e < a->nnz; ++e)
    if (a->idx[e] < 0 || a->idx[e] >= n_idx) bad = 1;
  if (bad) return PLSQR_ERR_FORMAT;
  return magnitude_ok(a->val, a->nnz, 1);
}

static int upload_lines(plsqr_ctx *ctx, const plsqr_sparse *a, const std::vector<int64_t> &ptr,
                        DevLines *out, int32_t n_lines) {
  int rc;
  if ((rc = dev_alloc(ctx, &out->ptr, (size_t)n_lines + 1))) return rc;
  if ((rc = dev_alloc(ctx, &out->idx, (size_t)a->nnz))) return rc;
  if ((rc = dev_alloc(ctx, &out->val, (size_t)a->nnz))) return rc;
  CK(cudaMemcpy(out->ptr, ptr.data(), ((size_t)n_lines + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
  if (a->nnz > 0) {
    CK(cudaMemcpy(out->idx, a->idx, (size_t)a->nnz * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(out->val, a->val, (size_t)a->nnz * sizeof(double), cudaMemcpyHostToDevice));
  }
  out->n_lines = n_lines;
  out->nnz = a->nnz;
  return PLSQR_OK;
}

// K by row from K by column, on the device (transpose.cuh)
static int build_kernel_rows(plsqr_ctx *ctx) {
  const int m = ctx->m_k, n = ctx->n;
  int rc;
  if ((rc = dev_alloc(ctx, &ctx->K.ptr, (size_t)m + 1))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->K.idx, (size_t)ctx->nnz_k))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->K.val, (size_t)ctx->nnz_k))) return rc;
  ctx->K.n_lines = m;
  ctx->K.nnz = ctx->nnz_k;
  if (m == 0) {
    CK(cudaMemset(ctx->K.ptr, 0, sizeof(int64_t)));
    return PLSQR_OK;
  }
  // chunk count: enough blocks to fill the GPU, bounded by 2 GiB of cursors
  int64_t nb = std::min<int64_t>((int64_t)ctx->sm_count * 4, std::max(n, 1));
  nb = std::min<int64_t>(nb, std::max<int64_t>(1, (int64_t)(2LL << 30) / (12LL * m)));
  int32_t *cnt = nullptr;
  int64_t *cur = nullptr, *rowcnt = nullptr;
  if ((rc = dev_alloc(ctx, &cnt, (size_t)(nb * m)))) return rc;
  if ((rc = dev_alloc(ctx, &cur, (size_t)(nb * m)))) return rc;
  if ((rc = dev_alloc(ctx, &rowcnt, (size_t)m))) return rc;
  CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * nb * m, ctx->stream));
  k_tr_count<<<(int)nb, 256, 0, ctx->stream>>>(ctx->KC.ptr, ctx->KC.idx, n, (int)nb, m, cnt);
  k_tr_rowtot<<<std::max(1, std::min(4096, (m + 255) / 256)), 256, 0, ctx->stream>>>(cnt, (int)nb, m, rowcnt);
  k_scan_one_block<<<1, 1024, 0, ctx->stream>>>(rowcnt, m, ctx->K.ptr);
  k_tr_cursor<<<std::max(1, std::min(4096, (m + 255) / 256)), 256, 0, ctx->stream>>>(cnt, (int)nb, m, ctx->K.ptr, cur);
  k_tr_scatter<<<(int)nb, 256, 0, ctx->stream>>>(ctx->KC.ptr, ctx->KC.idx, ctx->KC.val, n, (int)nb, m,
                                                (unsigned long long *)cur, ctx->K.idx, ctx->K.val);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  int64_t total = -1;
  CK(cudaMemcpy(&total, ctx->K.ptr + m, sizeof(int64_t), cudaMemcpyDeviceToHost));
  dev_free(ctx, cnt);
  dev_free(ctx, cur);
  dev_free(ctx, rowcnt);
  return total == ctx->nnz_k ? PLSQR_OK : PLSQR_ERR_INTERNAL;
}

// Contiguous line ranges [part[w], part[w+1]) with about nnz/parts nonzeros
// each (a line is never split): the static, balanced warp-to-line map of the
// product kernels.
static void balanced_partition(const int64_t *ptr, int32_t n_lines, int parts,
                               std::vector<int32_t> &out) {
  out.assign((size_t)parts + 1, 0);
  const int64_t nnz = ptr[n_lines];
  for (int w = 1; w < parts; ++w) {
    const int64_t target = (int64_t)((long double)nnz * w / parts);
    const int64_t *it = std::lower_bound(ptr, ptr + n_lines + 1, target);
    int32_t r = (int32_t)(it - ptr);
    if (r > n_lines) r = n_lines;
    out[(size_t)w] = std::max(r, out[(size_t)w - 1]);
  }
  out[(size_t)parts] = n_lines;
}

template <int U>
static void launch_m1(plsqr_ctx *ctx, cudaStream_t s, int mode, double *parts) {
  k_aprod1<double, kThreads, U><<<ctx->g1k + ctx->g1d, kThreads, 0, s>>>(
      ctx->K.csr(), ctx->D.csr(), ctx->kpart, ctx->v, ctx->u, ctx->g1k, mode, ctx->st, parts);
}
template <int U>
static void launch_m2(plsqr_ctx *ctx, cudaStream_t s, int mode, double *parts) {
  k_aprod2<double, kThreads, U><<<ctx->g2, kThreads, 0, s>>>(ctx->KC.csr(), ctx->DC.csr(), ctx->cpart,
                                                      ctx->corder, ctx->u, ctx->m_k, ctx->v, mode,
                                                      ctx->st, parts);
}
// The products.  Slab path: slab SpMV into per-slab partials, then the
// combine kernel (scale, damping part, sums of squares).  Otherwise the
// per-line kernels.  Either way `parts` receives pu_k + pu_d (mode 1) or pv
// (mode 2) per-block sums of squares for the norm kernels.
template <typename T>
void slab_spmv(const DevSlab<T> &S, int group, const T *x, cudaStream_t s) {
  const SlabCsr<T> A{S.ptr, S.order, S.idx, S.val, S.n_lines, S.n_slabs, S.slab, S.n_idx};
  if (S.next) {  // persistent form: line counters zeroed, then one block per SM slot
    cudaMemsetAsync(S.next, 0, sizeof(int) * S.n_slabs, s);
    const int g = S.dyn_blocks;
    if (group == 4)
      k_slab_spmv_dyn<T, 1024, 4><<<g, 1024, S.smem, s>>>(A, S.next, S.chunk, x, S.partial);
    else if (group == 8)
      k_slab_spmv_dyn<T, 1024, 8><<<g, 1024, S.smem, s>>>(A, S.next, S.chunk, x, S.partial);
    else if (group == 32)
      k_slab_spmv_dyn<T, 1024, 32><<<g, 1024, S.smem, s>>>(A, S.next, S.chunk, x, S.partial);
    else
      k_slab_spmv_dyn<T, 1024, 16><<<g, 1024, S.smem, s>>>(A, S.next, S.chunk, x, S.partial);
    return;
  }
  const int grid = S.n_slabs * S.bps;
  if (group == 4)
    k_slab_spmv<T, 1024, 4><<<grid, 1024, S.smem, s>>>(A, S.lpart, S.bps, x, S.partial);
  else if (group == 8)
    k_slab_spmv<T, 1024, 8><<<grid, 1024, S.smem, s>>>(A, S.lpart, S.bps, x, S.partial);
  else if (group == 32)
    k_slab_spmv<T, 1024, 32><<<grid, 1024, S.smem, s>>>(A, S.lpart, S.bps, x, S.partial);
  else
    k_slab_spmv<T, 1024, 16><<<grid, 1024, S.smem, s>>>(A, S.lpart, S.bps, x, S.partial);
}
template void slab_spmv<double>(const DevSlab<double> &, int, const double *, cudaStream_t);
template void slab_spmv<float>(const DevSlab<float> &, int, const float *, cudaStream_t);

template <typename T>
int slab_set_smem(size_t smem) {
  const int b = (int)std::max<size_t>(smem, 1);
  if (cudaFuncSetAttribute(k_slab_spmv<T, 1024, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv<T, 1024, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv<T, 1024, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv<T, 1024, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv_dyn<T, 1024, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv_dyn<T, 1024, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv_dyn<T, 1024, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ||
      cudaFuncSetAttribute(k_slab_spmv_dyn<T, 1024, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, b))
    return PLSQR_ERR_CUDA;
  return PLSQR_OK;
}
template int slab_set_smem<double>(size_t);
template int slab_set_smem<float>(size_t);

template <typename T>
void units_spmv(const DevUnitsT<T> &U, const T *x, cudaStream_t s, const T *x_lo) {
  const UnitsArgs<T> A{U.idx,     U.val,     U.slot0,  U.q,     U.c,       U.line,       U.unit_begin,
                       U.n_lines, U.n_slabs, U.slab,   U.n_idx, U.pf_dist, U.pf_pieces, U.slots};
  cudaMemsetAsync(U.next, 0, sizeof(int) * U.n_slabs, s);
  if constexpr (sizeof(T) == 4) {
    if (x_lo && U.hilo) {
      if (U.threads == 512)
        k_slab_units<T, 512, true><<<U.blocks, 512, U.smem, s>>>(A, U.next, x, x_lo, U.partial);
      else
        k_slab_units<T, 1024, true><<<U.blocks, 1024, U.smem, s>>>(A, U.next, x, x_lo, U.partial);
      return;
    }
  }
  if constexpr (sizeof(T) == 8) {
    if (U.chains == 4) {
      if (U.threads == 512)
        k_slab_units<T, 512, false, 4><<<U.blocks, 512, U.smem, s>>>(A, U.next, x, nullptr, U.partial);
      else
        k_slab_units<T, 1024, false, 4><<<U.blocks, 1024, U.smem, s>>>(A, U.next, x, nullptr,
                                                                       U.partial);
      return;
    }
  }
  if (U.threads == 512)
    k_slab_units<T, 512><<<U.blocks, 512, U.smem, s>>>(A, U.next, x, nullptr, U.partial);
  else
    k_slab_units<T, 1024><<<U.blocks, 1024, U.smem, s>>>(A, U.next, x, nullptr, U.partial);
}
template void units_spmv<double>(const DevUnitsT<double> &, const double *, cudaStream_t,
                                 const double *);
template void units_spmv<float>(const DevUnitsT<float> &, const float *, cudaStream_t,
                                const float *);

template <typename T>
int units_set_smem(size_t smem) {
  const int bytes = (int)std::max<size_t>(smem, 1);
  const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  bool bad = cudaFuncSetAttribute(k_slab_units<T, 1024>, attr, bytes) != cudaSuccess ||
             cudaFuncSetAttribute(k_slab_units<T, 512>, attr, bytes) != cudaSuccess;
  if constexpr (sizeof(T) == 4)
    bad = bad || cudaFuncSetAttribute(k_slab_units<T, 1024, true>, attr, bytes) != cudaSuccess ||
          cudaFuncSetAttribute(k_slab_units<T, 512, true>, attr, bytes) != cudaSuccess;
  else
    bad = bad || cudaFuncSetAttribute(k_slab_units<T, 1024, false, 4>, attr, bytes) != cudaSuccess ||
          cudaFuncSetAttribute(k_slab_units<T, 512, false, 4>, attr, bytes) != cudaSuccess;
  return bad ? PLSQR_ERR_CUDA : PLSQR_OK;
}
template int units_set_smem<double>(size_t);
template int units_set_smem<float>(size_t);

static void m1(plsqr_ctx *ctx, cudaStream_t s, int mode, double *parts) {
  if (ctx->exact) {  // the reference's order (kernels_exact.cuh); no partial sums
    k_ref_rows<kThreads><<<ctx->ex_gk + ctx->ex_gd, kThreads, 0, s>>>(
        ctx->K.csr(), ctx->D.csr(), ctx->v, ctx->u, ctx->ex_gk, mode, ctx->st);
    return;
  }
  if (ctx->use_units_rows) {
    const DevUnits &U = ctx->u_rows;
    units_spmv(U, ctx->v, s);
    k_combine_rows<double, double, kThreads><<<ctx->gc1k + ctx->gc1d, kThreads, 0, s>>>(
        U.partial, U.n_slabs, ctx->m_k, ctx->D.csr(), ctx->v, ctx->u, ctx->gc1k, mode, ctx->st, parts);
    return;
  }
  if (ctx->use_slabs_rows) {
    const DevSlab<double> &S = ctx->s_rows;
    slab_spmv(S, ctx->slab_group, ctx->v, s);
    k_combine_rows<double, double, kThreads><<<ctx->gc1k + ctx->gc1d, kThreads, 0, s>>>(
        S.partial, S.n_slabs, ctx->m_k, ctx->D.csr(), ctx->v, ctx->u, ctx->gc1k, mode, ctx->st, parts);
    return;
  }
  switch (ctx->unroll) {
    case 1: launch_m1<1>(ctx, s, mode, parts); break;
    case 4: launch_m1<4>(ctx, s, mode, parts); break;
    default: launch_m1<2>(ctx, s, mode, parts);
  }
}
static void m2(plsqr_ctx *ctx, cudaStream_t s, int mode, double *parts) {
  if (ctx->exact) {
    k_ref_cols<kThreads><<<ctx->ex_gc, kThreads, 0, s>>>(ctx->KC.csr(), ctx->DC.csr(), ctx->u,
                                                          ctx->m_k, ctx->v, mode, ctx->st);
    return;
  }
  if (ctx->use_units) {
    const DevUnits &U = ctx->u_cols;
    units_spmv(U, ctx->u, s);
    k_combine_cols<double, double, kThreads><<<ctx->gc2, kThreads, 0, s>>>(
        U.partial, U.n_slabs, ctx->n, ctx->DC.csr(), ctx->u, ctx->m_k, ctx->v, mode, ctx->st, parts);
    return;
  }
  if (ctx->use_slabs) {
    const DevSlab<double> &S = ctx->s_cols;
    slab_spmv(S, ctx->slab_group, ctx->u, s);
    k_combine_cols<double, double, kThreads><<<ctx->gc2, kThreads, 0, s>>>(
        S.partial, S.n_slabs, ctx->n, ctx->DC.csr(), ctx->u, ctx->m_k, ctx->v, mode, ctx->st, parts);
    return;
  }
  switch (ctx->unroll) {
    case 1: launch_m2<1>(ctx, s, mode, parts); break;
    case 4: launch_m2<4>(ctx, s, mode, parts); break;
    default: launch_m2<2>(ctx, s, mode, parts);
  }
}
// The slab kernel stages up to 192 KB of shared memory; the limit is a
// per-module attribute, so it is set here, where the kernel is launched.
static int slab_attrs(plsqr_ctx *ctx) {
  if (!ctx->use_slabs && !ctx->use_slabs_rows) return PLSQR_OK;
  int rc = slab_set_smem<double>(std::max(ctx->s_rows.smem, ctx->s_cols.smem));
  if (!rc && (ctx->use_units || ctx->use_units_rows))
    rc = units_set_smem<double>(std::max(ctx->u_cols.smem, ctx->u_rows.smem));
  if (rc) ctx_set_error(ctx, "cudaFuncSetAttribute failed for the slab kernels");
  return rc;
}

// ---- the reference's order of operations (PLSQR_ORDER_REFERENCE) ----------
// Scratch of the ordered norms and of the dknorm terms, and the grids of the
// one-thread-per-line products.
static int exact_prepare(plsqr_ctx *ctx) {
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  auto chunks = [](int64_t n) { return (int)((n + kNrmChunk - 1) / kNrmChunk); };
  ctx->ex_nb_k = chunks(ctx->m_k);
  ctx->ex_nb_d = chunks(ctx->m_d);
  ctx->ex_nb_v = chunks(ctx->n);
  const int g = ctx->sm_count * 8;
  ctx->ex_gk = std::max(1, std::min(g, (ctx->m_k + kThreads - 1) / kThreads));
  ctx->ex_gd = std::max(1, std::min(g, (ctx->m_d + kThreads - 1) / kThreads));
  ctx->ex_gc = std::max(1, std::min(g, (ctx->n + kThreads - 1) / kThreads));
  int rc;
  if ((rc = dev_alloc(ctx, &ctx->ex_terms, (size_t)std::max<int64_t>(m, ctx->n))) ||
      (rc = dev_alloc(ctx, &ctx->ex_bmax,
                      (size_t)std::max(ctx->ex_nb_k + ctx->ex_nb_d, ctx->ex_nb_v))))
    return rc;
  return PLSQR_OK;
}

// beta = ||[y_k; y_d]|| (two segments) or alpha = ||v|| (one)
static NrmArgs exact_nrm_u(const plsqr_ctx *ctx) {
  NrmArgs a{};
  a.nseg = 2;
  a.bmax = ctx->ex_bmax;
  a.seg[0] = NrmSeg{ctx->u, ctx->m_k, ctx->ex_terms, 0, ctx->ex_nb_k};
  a.seg[1] = NrmSeg{ctx->u + ctx->m_k, ctx->m_d, ctx->ex_terms + ctx->m_k, ctx->ex_nb_k,
                    ctx->ex_nb_d};
  return a;
}
static NrmArgs exact_nrm_v(const plsqr_ctx *ctx) {
  NrmArgs a{};
  a.nseg = 1;
  a.bmax = ctx->ex_bmax;
  a.seg[0] = NrmSeg{ctx->v, ctx->n, ctx->ex_terms, 0, ctx->ex_nb_v};
  a.seg[1] = NrmSeg{nullptr, 0, nullptr, ctx->ex_nb_v, 0};
  return a;
}
static void exact_norm(const plsqr_ctx *ctx, const NrmArgs &a, int kind, cudaStream_t s) {
  const int blocks = a.seg[0].nb + (a.nseg > 1 ? a.seg[1].nb : 0);
  if (blocks > 0) {
    k_nrm_max<<<blocks, kNrmThreads, 0, s>>>(a, kind, ctx->st);
    k_nrm_terms<<<blocks, kNrmThreads, 0, s>>>(a, kind, ctx->st);
  }
  k_nrm_chain<<<1, 64, 0, s>>>(a, kind, ctx->st);
}

// partial-sum counts the norm kernels read
int ctx_pu_k(const plsqr_ctx *ctx) {
  return ctx->use_slabs_rows ? ctx->gc1k : ctx->g1k * (kThreads / 32);  // k_aprod1: per warp
}
int ctx_pu_d(const plsqr_ctx *ctx) { return ctx->use_slabs_rows ? ctx->gc1d : ctx->g1d; }
int ctx_pv(const plsqr_ctx *ctx) { return ctx->use_slabs ? ctx->gc2 : ctx->g2; }

// Spread the low 10 bits of v to every third bit.
static uint32_t part1by2(uint32_t v) {
  v &= 0x3ff;
  v = (v | (v << 16)) & 0x030000ff;
  v = (v | (v << 8)) & 0x0300f00f;
  v = (v | (v << 4)) & 0x030c30c3;
  v = (v | (v << 2)) & 0x09249249;
  return v;
}

// Visit order of the columns for the A^T y product: 3-D Morton order of the
// cells when the grid is known, the natural order otherwise.
static void column_order(const plsqr_ctx *ctx, std::vector<int32_t> &order) {
  const int n = ctx->n;
  order.resize((size_t)n);
  for (int c = 0; c < n; ++c) order[(size_t)c] = c;
  const int nx = ctx->opts.grid[0], ny = ctx->opts.grid[1], nz = ctx->opts.grid[2];
  if (nx <= 0 || ny <= 0 || nz <= 0 || (int64_t)nx * ny * nz != n || nx > 1024 || ny > 1024 ||
      nz > 1024)
    return;
  std::vector<uint32_t> key((size_t)n);
  for (int c = 0; c < n; ++c) {
    const uint32_t ix = c % nx, iy = (c / nx) % ny, iz = c / (nx * ny);
    key[(size_t)c] = part1by2(ix) | (part1by2(iy) << 1) | (part1by2(iz) << 2);
  }
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return key[(size_t)a] < key[(size_t)b]; });
}

static int plan_launch(plsqr_ctx *ctx, const std::vector<int64_t> &kc_ptr) {
  const int sm = ctx->sm_count;
  const int wpb = kThreads / 32;
  int occ1 = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, k_aprod1<double, kThreads, 2>, kThreads, 0));
  occ1 = std::max(1, std::min(occ1, ctx->blocks_per_sm));
  // every reduction kernel writes at most kMaxParts partials
  const int half = kMaxParts / 2;
  // mode 1: one resident wave of warps over kernel rows (one partial per
  // warp), threads over damping rows (one partial per block)
  ctx->g1k = std::max(1, std::min({sm * occ1, (ctx->m_k + wpb - 1) / wpb, half / wpb}));
  ctx->g1d = std::max(1, std::min({sm, (ctx->m_d + kThreads - 1) / kThreads, half}));
  // mode 2: many small blocks of neighbouring columns (several waves)
  int m2b = ctx->m2_blocks_per_sm;
  if (const char *e = getenv("PLSQR_M2_BLOCKS_PER_SM"))
    if (atoi(e) > 0) m2b = atoi(e);
  ctx->g2 = std::max(1, std::min({sm * m2b, (ctx->n + wpb - 1) / wpb, kMaxParts}));
  // vector kernels
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  ctx->gvu = (int)std::max<int64_t>(1, std::min<int64_t>(sm * 4, (m + kThreads - 1) / kThreads));
  ctx->gvx = std::max(1, std::min(sm * 4, (ctx->n + kThreads - 1) / kThreads));
  ctx->gsk = std::max(1, std::min(sm, (ctx->m_k + kThreads - 1) / kThreads));
  ctx->gsd = std::max(1, std::min(sm, (ctx->m_d + kThreads - 1) / kThreads));
  // balanced warp ranges over kernel rows (pointer array copied back from
  // the device transpose) and over columns
  std::vector<int64_t> krp((size_t)ctx->m_k + 1);
  CK(cudaMemcpy(krp.data(), ctx->K.ptr, krp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost));
  std::vector<int32_t> kp, cp;
  balanced_partition(krp.data(), ctx->m_k, ctx->g1k * wpb, kp);
  std::vector<int32_t> order;
  column_order(ctx, order);
  const char *no = getenv("PLSQR_NATURAL_ORDER");
  if (no && atoi(no) > 0)
    for (int c = 0; c < ctx->n; ++c) order[(size_t)c] = c;
  std::vector<int64_t> optr((size_t)ctx->n + 1);  // nonzero prefix in visit order
  optr[0] = 0;
  for (int k = 0; k < ctx->n; ++k) {
    const int c = order[(size_t)k];
    optr[(size_t)k + 1] = optr[(size_t)k] + (kc_ptr[(size_t)c + 1] - kc_ptr[(size_t)c]);
  }
  balanced_partition(optr.data(), ctx->n, ctx->g2, cp);  // per block
  int rc;
  if ((rc = dev_alloc(ctx, &ctx->kpart, kp.size())) || (rc = dev_alloc(ctx, &ctx->cpart, cp.size())) ||
      (rc = dev_alloc(ctx, &ctx->corder, order.size())))
    return rc;
  CK(cudaMemcpy(ctx->corder, order.data(), order.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->kpart, kp.data(), kp.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->cpart, cp.data(), cp.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  return PLSQR_OK;
}

static void free_graph(plsqr_ctx *ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  ctx->graph_exec = nullptr;
}

static int ctx_init_common(plsqr_ctx *ctx) {
  CK(cudaSetDevice(ctx->opts.device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  CK(cudaEventCreate(&ctx->ev_start));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, ctx->opts.device));
  ctx->sm_count = prop.multiProcessorCount;
  if (ctx->blocks_per_sm <= 0) ctx->blocks_per_sm = 8;
  const char *env = getenv("PLSQR_BLOCKS_PER_SM");
  if (env && atoi(env) > 0) ctx->blocks_per_sm = atoi(env);
  ctx->m2_blocks_per_sm = 48;
  ctx->slab_group = 8;
  env = getenv("PLSQR_SLAB_GROUP");
  if (env && (atoi(env) == 4 || atoi(env) == 8 || atoi(env) == 16 || atoi(env) == 32))
    ctx->slab_group = atoi(env);
  ctx->slab_group_f = 16;
  env = getenv("PLSQR_SLAB_GROUP_F");
  if (env && (atoi(env) == 4 || atoi(env) == 8 || atoi(env) == 16 || atoi(env) == 32))
    ctx->slab_group_f = atoi(env);
  ctx->unroll = 2;
  env = getenv("PLSQR_UNROLL");
  if (env && (atoi(env) == 1 || atoi(env) == 2 || atoi(env) == 4)) ctx->unroll = atoi(env);
  return PLSQR_OK;
}

static int ctx_alloc_vectors(plsqr_ctx *ctx) {
  int rc;
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  if ((rc = dev_alloc(ctx, &ctx->u, (size_t)m))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->v, (size_t)ctx->n))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->w, (size_t)ctx->n))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->x, (size_t)ctx->n))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->parts_u, kMaxParts))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->parts_v, kMaxParts))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->parts_dk, kMaxParts))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->parts_err, kMaxParts))) return rc;
  if ((rc = dev_alloc(ctx, &ctx->st, 1))) return rc;
  CK(cudaMemset(ctx->u, 0, sizeof(double) * std::max<int64_t>(m, 1)));
  CK(cudaMemset(ctx->v, 0, sizeof(double) * std::max(ctx->n, 1)));
  CK(cudaMemset(ctx->w, 0, sizeof(double) * std::max(ctx->n, 1)));
  CK(cudaMemset(ctx->x, 0, sizeof(double) * std::max(ctx->n, 1)));
  CK(cudaMemset(ctx->st, 0, sizeof(DevState)));
  return PLSQR_OK;
}

static double algorithmic_bytes(const plsqr_ctx *ctx, int mode) {
  // bytes a perfect kernel moves: matrix entries (int32 index + FP64 value),
  // pointer arrays, the vector it updates read and written once, the gathered
  // vector read once (it stays in L2)
  const double mk = ctx->m_k, md = ctx->m_d, n = ctx->n;
  if (mode == 1)
    return 12.0 * ((double)ctx->nnz_k + (double)ctx->nnz_d) + 8.0 * (mk + 1 + md + 1) +
           16.0 * (mk + md) + 8.0 * n;
  return 12.0 * ((double)ctx->nnz_k + (double)ctx->nnz_d) + 16.0 * (n + 1) + 16.0 * n +
         8.0 * (mk + md);
}

extern "C" {

const char *plsqr_strerror(int code) {
  const int i = -code;
  if (i < 0 || i >= (int)(sizeof(kErrText) / sizeof(kErrText[0]))) return "unknown error";
  return kErrText[i];
}

int plsqr_abi_version(void) { return PLSQR_GPU_ABI_VERSION; }

int plsqr_check_flags(int32_t *checked, uint32_t *flags, int32_t reset) {
  if (!checked || !flags) return PLSQR_ERR_ARG;
#ifdef PLSQR_CHECK
  *checked = 1;
#else
  *checked = 0;
#endif
  // the unit kernels run in this translation unit, their fill and reorder in
  // slab.cu, the batched solver's k-wide unit kernels in batched.cu
  const unsigned a = plsqr::check_word(reset != 0), b = slab_check_word(reset != 0),
                 c = batched_check_word(reset != 0);
  if (a == ~0u || b == ~0u || c == ~0u) return PLSQR_ERR_CUDA;
  *flags = a | b | c;
  return PLSQR_OK;
}

void plsqr_default_opts(plsqr_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->device = 0;
  o->precision = PLSQR_PREC_FP64;
  o->use_graph = 1;
  o->verbose = 0;
}

void plsqr_default_lsqr_args(plsqr_lsqr_args *a) {
  if (!a) return;
  memset(a, 0, sizeof(*a));
  a->damp = 0.0;  // source/lsqr.c:47-51
  a->atol = 1e-10;
  a->btol = 1e-10;
  a->conlim = 100;
  a->itnlim = 1000;
  a->lsqr_iteration = 100;
  a->sweeps = 4;
  a->inner = 50;
}

int plsqr_device_count(int32_t *count) {
  if (!count) return PLSQR_ERR_ARG;
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c = 0;
  }
  *count = c;
  return PLSQR_OK;
}

void plsqr_ctx_destroy(plsqr_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->opts.device);
  free_graph(ctx);
  mixed_free(ctx);
  batch_free(ctx);
  for (auto &a : ctx->allocs) cudaFree(a.first);
  ctx->allocs.clear();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

// opts.lean: the index and value arrays of K by row (by column) go once the
// unit layout of the rows (columns) serves the FP64 product; the pointer
// arrays stay (small, and read by the launch planning).
static void release_kernel_lines(plsqr_ctx *ctx) {
  if (ctx->use_units_rows) {
    dev_free(ctx, ctx->K.idx);
    dev_free(ctx, ctx->K.val);
    ctx->K.idx = nullptr;
    ctx->K.val = nullptr;
    ctx->lines_released = true;
  }
  if (ctx->use_units) {
    dev_free(ctx, ctx->KC.idx);
    dev_free(ctx, ctx->KC.val);
    ctx->KC.idx = nullptr;
    ctx->KC.val = nullptr;
    ctx->lines_released = true;
  }
}

int plsqr_ctx_create(const plsqr_sparse *k_csc, const plsqr_sparse *d_csr,
                     const plsqr_sparse *d_csc, const plsqr_opts *opts, plsqr_ctx **out) {
  if (!out || !k_csc || !d_csr || !d_csc) return PLSQR_ERR_ARG;
  *out = nullptr;
  const int32_t m_k = k_csc->num_row, n = k_csc->num_col, m_d = d_csr->num_row;
  if (m_k < 0 || n < 1 || m_d < 0 || (int64_t)m_k + m_d < 1) return PLSQR_ERR_ARG;
  std::vector<int64_t> kp, dp, dcp;
  int rc;
  if ((rc = validate_sparse(k_csc, m_k, n, 1, kp))) return rc;
  if ((rc = validate_sparse(d_csr, m_d, n, 0, dp))) return rc;
  if ((rc = validate_sparse(d_csc, m_d, n, 1, dcp))) return rc;
  if (d_csc->nnz != d_csr->nnz) return PLSQR_ERR_FORMAT;
  int32_t ndev = 0;
  plsqr_device_count(&ndev);
  plsqr_opts o;
  plsqr_default_opts(&o);
  if (opts) o = *opts;
  if (ndev < 1 || o.device < 0 || o.device >= ndev) return PLSQR_ERR_NODEV;
  if (o.order != PLSQR_ORDER_FAST && o.order != PLSQR_ORDER_REFERENCE) return PLSQR_ERR_ARG;
  if (o.order == PLSQR_ORDER_REFERENCE && o.precision != PLSQR_PREC_FP64) return PLSQR_ERR_ARG;
  if (o.lean && (o.order != PLSQR_ORDER_FAST || o.precision != PLSQR_PREC_FP64)) return PLSQR_ERR_ARG;

  plsqr_ctx *ctx = new plsqr_ctx();
  ctx->opts = o;
  ctx->m_k = m_k;
  ctx->m_d = m_d;
  ctx->n = n;
  ctx->nnz_k = k_csc->nnz;
  ctx->nnz_d = d_csr->nnz;
  ctx->exact = o.order == PLSQR_ORDER_REFERENCE;
  if ((rc = ctx_init_common(ctx)) || (rc = upload_lines(ctx, k_csc, kp, &ctx->KC, n)) ||
      (rc = upload_lines(ctx, d_csr, dp, &ctx->D, m_d)) ||
      (rc = upload_lines(ctx, d_csc, dcp, &ctx->DC, n)) || (rc = build_kernel_rows(ctx)) ||
      (rc = ctx_alloc_vectors(ctx)) || (rc = plan_launch(ctx, kp)) ||
      (rc = ctx->exact ? exact_prepare(ctx) : slab_plan(ctx)) || (rc = slab_attrs(ctx))) {
    plsqr_ctx_destroy(ctx);
    return rc;
  }
  if (o.precision == PLSQR_PREC_MIXED && (rc = mixed_prepare(ctx))) {
    plsqr_ctx_destroy(ctx);
    return rc;
  }
  if (o.lean) release_kernel_lines(ctx);
  *out = ctx;
  return PLSQR_OK;
}

int plsqr_ctx_info(const plsqr_ctx *ctx, plsqr_info *info) {
  if (!ctx || !info) return PLSQR_ERR_ARG;
  memset(info, 0, sizeof(*info));
  info->m_k = ctx->m_k;
  info->m_d = ctx->m_d;
  info->n = ctx->n;
  info->nnz_k = ctx->nnz_k;
  info->nnz_d = ctx->nnz_d;
  info->device_bytes = ctx->device_bytes;
  info->sm_count = ctx->sm_count;
  info->hbm_bytes_aprod1 = algorithmic_bytes(ctx, 1);
  info->hbm_bytes_aprod2 = algorithmic_bytes(ctx, 2);
  // one iteration: both products plus the vector kernels (u scaled in place,
  // v scaled and x, w updated: 8 bytes read + written per element)
  const double m = (double)ctx->m_k + ctx->m_d, n = ctx->n;
  info->hbm_bytes_iteration = info->hbm_bytes_aprod1 + info->hbm_bytes_aprod2 + 16.0 * m +
                              8.0 * (2.0 * n + 4.0 * n);
  return PLSQR_OK;
}

const char *plsqr_ctx_last_error(const plsqr_ctx *ctx) { return ctx ? ctx->last_error : ""; }

static int check_finite(const double *p, int64_t n) {
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t i = 0; i < n; ++i)
    if (!isfinite(p[i])) bad = 1;
  return bad ? PLSQR_ERR_NUMERIC : PLSQR_OK;
}

int plsqr_set_u(plsqr_ctx *ctx, const double *y_k, const double *y_d) {
  if (!ctx || (!y_k && ctx->m_k > 0)) return PLSQR_ERR_ARG;
  int rc;
  if ((rc = check_finite(y_k, ctx->m_k))) return rc;
  if (y_d && (rc = check_finite(y_d, ctx->m_d))) return rc;
  CK(cudaSetDevice(ctx->opts.device));
  if (ctx->m_k > 0)
    CK(cudaMemcpyAsync(ctx->u, y_k, sizeof(double) * ctx->m_k, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->m_d > 0) {
    if (y_d)
      CK(cudaMemcpyAsync(ctx->u + ctx->m_k, y_d, sizeof(double) * ctx->m_d, cudaMemcpyHostToDevice,
                         ctx->stream));
    else
      CK(cudaMemsetAsync(ctx->u + ctx->m_k, 0, sizeof(double) * ctx->m_d, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return PLSQR_OK;
}

int plsqr_get_u(plsqr_ctx *ctx, double *y_k, double *y_d) {
  if (!ctx) return PLSQR_ERR_ARG;
  CK(cudaSetDevice(ctx->opts.device));
  if (y_k && ctx->m_k > 0)
    CK(cudaMemcpyAsync(y_k, ctx->u, sizeof(double) * ctx->m_k, cudaMemcpyDeviceToHost, ctx->stream));
  if (y_d && ctx->m_d > 0)
    CK(cudaMemcpyAsync(y_d, ctx->u + ctx->m_k, sizeof(double) * ctx->m_d, cudaMemcpyDeviceToHost,
                       ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PLSQR_OK;
}

int plsqr_set_v(plsqr_ctx *ctx, const double *v) {
  if (!ctx || !v) return PLSQR_ERR_ARG;
  int rc;
  if ((rc = check_finite(v, ctx->n))) return rc;
  CK(cudaSetDevice(ctx->opts.device));
  CK(cudaMemcpyAsync(ctx->v, v, sizeof(double) * ctx->n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PLSQR_OK;
}

int plsqr_get_v(plsqr_ctx *ctx, double *v) {
  if (!ctx || !v) return PLSQR_ERR_ARG;
  CK(cudaSetDevice(ctx->opts.device));
  CK(cudaMemcpyAsync(v, ctx->v, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return PLSQR_OK;
}

int plsqr_get_b(plsqr_ctx *ctx, double *b_k) {
  if (!ctx || !b_k) return PLSQR_ERR_ARG;
  if ((int32_t)ctx->b_k.size() != ctx->m_k) return PLSQR_ERR_STATE;
  memcpy(b_k, ctx->b_k.data(), sizeof(double) * ctx->m_k);
  return PLSQR_OK;
}

// Enqueue one product on the context's stream.
static int launch_aprod(plsqr_ctx *ctx, int mode, int scale_mode, bool with_parts) {
  if (mode == 1)
    m1(ctx, ctx->stream, scale_mode, with_parts ? ctx->parts_u : nullptr);
  else
    m2(ctx, ctx->stream, scale_mode, with_parts ? ctx->parts_v : nullptr);
  CK(cudaGetLastError());
  return PLSQR_OK;
}

int plsqr_aprod(plsqr_ctx *ctx, int mode, int iteration, int is_final) {
  (void)iteration;
  (void)is_final;
  if (!ctx || (mode != 1 && mode != 2)) return PLSQR_ERR_ARG;
  CK(cudaSetDevice(ctx->opts.device));
  int rc = launch_aprod(ctx, mode, kScaleOne, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return PLSQR_OK;
}

int plsqr_aprod_host(plsqr_ctx *ctx, int mode, double *y_k, double *y_d, double *x,
                     int iteration, int is_final) {
  if (!ctx || (mode != 1 && mode != 2) || !x || (!y_k && ctx->m_k > 0) ||
      (!y_d && ctx->m_d > 0))
    return PLSQR_ERR_ARG;
  int rc;
  if ((rc = plsqr_set_u(ctx, y_k, y_d)) || (rc = plsqr_set_v(ctx, x)) ||
      (rc = plsqr_aprod(ctx, mode, iteration, is_final)))
    return rc;
  return mode == 1 ? plsqr_get_u(ctx, y_k, y_d) : plsqr_get_v(ctx, x);
}

int plsqr_set_reference_x(plsqr_ctx *ctx, const double *x_ref) {
  if (!ctx) return PLSQR_ERR_ARG;
  CK(cudaSetDevice(ctx->opts.device));
  if (!x_ref) {
    ctx->has_ref = false;
    return PLSQR_OK;
  }
  int rc;
  if ((rc = check_finite(x_ref, ctx->n))) return rc;
  if (!ctx->xref && (rc = dev_alloc(ctx, &ctx->xref, (size_t)ctx->n))) return rc;
  CK(cudaMemcpy(ctx->xref, x_ref, sizeof(double) * ctx->n, cudaMemcpyHostToDevice));
  ctx->has_ref = true;
  return PLSQR_OK;
}

// One LSQR iteration (source/lsqr.c:487-775) as five regions named after
// the reference's GPTL timers.  Each region is a marker pair: with `ev` (the
// timed solve) an event is recorded before the first region and after every
// region, and the host enqueue is bracketed by an NVTX range of the region's
// name; graph capture and the plain solve pass no events.
struct Regions {
  plsqr_ctx *ctx;
  cudaStream_t s;
  const cudaEvent_t *ev;
  int k = 0;
  void begin() {
    if (ev) {
      cudaEventRecord(ev[0], s);
      nvtxRangePushA(kRegionName[0]);
    }
  }
  void next() {  // end of region k, start of region k + 1
    if (!ev) return;
    nvtxRangePop();
    cudaEventRecord(ev[++k], s);
    if (k < kRegions) nvtxRangePushA(kRegionName[k]);
  }
};

// The reference's order (kernels_exact.cuh): u = -alpha u + A v, beta,
// u /= beta, v = -beta v + A^T u, alpha, then the rotation, the x/w update
// and the ordered dknorm sum.
static int enqueue_iteration_exact(plsqr_ctx *ctx, cudaStream_t s, const cudaEvent_t *ev) {
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  double *se = ctx->want_se ? ctx->se : nullptr;
  const double *xref = ctx->has_ref ? ctx->xref : nullptr;
  Regions r{ctx, s, ev};
  r.begin();
  m1(ctx, s, kScaleNegAlpha, nullptr);
  r.next();
  exact_norm(ctx, exact_nrm_u(ctx), kNrmBeta, s);
  k_ref_scale_u<kThreads><<<ctx->gvu, kThreads, 0, s>>>(ctx->u, m, ctx->st);
  r.next();
  m2(ctx, s, kScaleNegBeta, nullptr);
  r.next();
  exact_norm(ctx, exact_nrm_v(ctx), kNrmAlpha, s);
  k_ref_update<kThreads><<<ctx->gvx, kThreads, 0, s>>>(
      ctx->v, ctx->w, ctx->x, se, xref, ctx->n, ctx->st, ctx->ex_terms,
      xref ? ctx->parts_err : nullptr, ctx->hist, 0);
  r.next();
  k_ref_tail<<<1, 32, 0, s>>>(ctx->st, ctx->ex_terms, ctx->n, xref ? ctx->parts_err : nullptr,
                              ctx->gvx, ctx->x, ctx->hist);
  r.next();
  CK(cudaGetLastError());
  return PLSQR_OK;
}

// Enqueue one LSQR iteration: five kernels.
static int enqueue_iteration(plsqr_ctx *ctx, cudaStream_t s, const cudaEvent_t *ev = nullptr) {
  if (ctx->exact) return enqueue_iteration_exact(ctx, s, ev);
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  double *se = ctx->want_se ? ctx->se : nullptr;
  const double *xref = ctx->has_ref ? ctx->xref : nullptr;
  Regions r{ctx, s, ev};
  r.begin();
  m1(ctx, s, kScaleNegAlpha, ctx->parts_u);
  r.next();
  k_norm_u<double, kThreads><<<ctx->gvu, kThreads, 0, s>>>(ctx->u, m, ctx->parts_u, ctx_pu_k(ctx),
                                                             ctx_pu_d(ctx), ctx->st, 0);
  r.next();
  m2(ctx, s, kScaleNegBeta, ctx->parts_v);
  r.next();
  k_update_x<kThreads><<<ctx->gvx, kThreads, 0, s>>>(
      ctx->v, ctx->w, ctx->x, se, xref, ctx->n, ctx->parts_v, ctx_pv(ctx), ctx->st, ctx->parts_dk,
      xref ? ctx->parts_err : nullptr, ctx->hist, 0);
  r.next();
  k_tail<kThreads><<<1, kThreads, 0, s>>>(ctx->st, ctx->parts_dk, xref ? ctx->parts_err : nullptr,
                                           ctx->gvx, ctx->x, ctx->hist);
  r.next();
  CK(cudaGetLastError());
  return PLSQR_OK;
}

static int ensure_graph(plsqr_ctx *ctx) {
  const int key = (ctx->want_se ? 1 : 0) | (ctx->has_ref ? 2 : 0);
  if (ctx->graph_exec && ctx->graph_key == key && ctx->graph_hist == ctx->hist) return PLSQR_OK;
  free_graph(ctx);
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_iteration(ctx, ctx->stream);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CK(e);
  e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  ctx->graph_key = key;
  ctx->graph_hist = ctx->hist;
  return PLSQR_OK;
}

int plsqr_lsqr(plsqr_ctx *ctx, const plsqr_lsqr_args *args, const double *b_k, double *x,
               double *w, double *se, plsqr_iter *hist, plsqr_result *res) {
  if (!ctx || !args || args->lsqr_iteration < 0) return PLSQR_ERR_ARG;
  if (ctx->opts.precision == PLSQR_PREC_MIXED)
    return mixed_lsqr(ctx, args, b_k, x, w, se, hist, res);
  if (args->x0) {
    ctx_set_error(ctx, "x0 needs a mixed-precision context (the FP64 path starts from 0, as "
                       "source/lsqr.c:311-312 does)");
    return PLSQR_ERR_ARG;
  }
  const double *b = b_k;
  if (!b) {
    if ((int32_t)ctx->b_k.size() != ctx->m_k) return PLSQR_ERR_STATE;
    b = ctx->b_k.data();
  }
  int rc;
  if ((rc = magnitude_ok(b, ctx->m_k))) {
    ctx_set_error(ctx, "b_k holds NaN, Inf or magnitudes outside [2^-500, 2^500]; scale it by a "
                       "power of two");
    return rc;
  }
  CK(cudaSetDevice(ctx->opts.device));
  const int itn = args->lsqr_iteration;
  if (ctx->hist_cap < itn + 1) {
    if (ctx->hist) dev_free(ctx, ctx->hist);
    ctx->hist = nullptr;
    if ((rc = dev_alloc(ctx, &ctx->hist, (size_t)itn + 1))) return rc;
    ctx->hist_cap = itn + 1;
  }
  ctx->want_se = args->want_se != 0;
  if (ctx->want_se && !ctx->se && (rc = dev_alloc(ctx, &ctx->se, (size_t)ctx->n))) return rc;

  // lsqr.c:278-295 and the u = b, v = 0 set-up (plsqr3.c:580-603, lsqr.c:311-312)
  if ((rc = plsqr_set_u(ctx, b, nullptr))) return rc;
  CK(cudaMemsetAsync(ctx->v, 0, sizeof(double) * ctx->n, ctx->stream));
  CK(cudaMemsetAsync(ctx->hist, 0, sizeof(plsqr_iter) * (itn + 1), ctx->stream));
  DevState h;
  memset(&h, 0, sizeof(h));
  h.damp = args->damp;
  h.atol = args->atol;
  h.btol = args->btol;
  h.ctol = args->conlim > 0.0 ? 1.0 / args->conlim : 0.0;
  h.itnlim = args->itnlim;
  h.want_se = ctx->want_se;
  h.has_ref = ctx->has_ref;
  h.cs2 = -1.0;
  CK(cudaMemcpyAsync(ctx->st, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->has_ref) k_ref_norm<kThreads><<<1, kThreads, 0, ctx->stream>>>(ctx->xref, ctx->n, ctx->st);

  // start-up: beta u = b, alpha v = A^T u (lsqr.c:343-445)
  nvtxRangePushA("norm0+spmvT_init");
  CK(cudaEventRecord(ctx->ev_start, ctx->stream));
  const int64_t m = (int64_t)ctx->m_k + ctx->m_d;
  if (ctx->exact) {
    exact_norm(ctx, exact_nrm_u(ctx), kNrmBetaStart, ctx->stream);
    k_ref_scale_u<kThreads><<<ctx->gvu, kThreads, 0, ctx->stream>>>(ctx->u, m, ctx->st);
    if ((rc = launch_aprod(ctx, 2, kScaleZero, false))) return rc;
    exact_norm(ctx, exact_nrm_v(ctx), kNrmAlpha, ctx->stream);
    k_ref_update<kThreads><<<ctx->gvx, kThreads, 0, ctx->stream>>>(
        ctx->v, ctx->w, ctx->x, ctx->want_se ? ctx->se : nullptr, nullptr, ctx->n, ctx->st,
        ctx->ex_terms, nullptr, ctx->hist, 1);
  } else {
    k_sumsq_u<kThreads><<<ctx->gsk + ctx->gsd, kThreads, 0, ctx->stream>>>(
        ctx->u, ctx->m_k, ctx->m_d, ctx->gsk, ctx->parts_u);
    k_norm_u<double, kThreads><<<ctx->gvu, kThreads, 0, ctx->stream>>>(
        ctx->u, m, ctx->parts_u, ctx->gsk, ctx->gsd, ctx->st, 1);
    if ((rc = launch_aprod(ctx, 2, kScaleZero, true))) return rc;
    k_update_x<kThreads><<<ctx->gvx, kThreads, 0, ctx->stream>>>(
        ctx->v, ctx->w, ctx->x, ctx->want_se ? ctx->se : nullptr, nullptr, ctx->n, ctx->parts_v,
        ctx_pv(ctx), ctx->st, ctx->parts_dk, nullptr, ctx->hist, 1);
  }
  CK(cudaGetLastError());
  DevState cur;
  CK(cudaMemcpyAsync(&cur, ctx->st, sizeof(cur), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  nvtxRangePop();

  int done_itn = 0;
  float ms = 0.f, ms_total = 0.f;
  // timed solve: events around every region of every iteration, no graph
  const bool timed = ctx->timing;
  std::vector<cudaEvent_t> evs;
  struct EventPool {
    std::vector<cudaEvent_t> &e;
    ~EventPool() {
      for (cudaEvent_t x : e) cudaEventDestroy(x);
    }
  } pool{evs};
  if (timed) {
    ctx->t_iters = 0;
    evs.assign((size_t)itn * (kRegions + 1), nullptr);
    for (auto &e : evs) CK(cudaEventCreate(&e));
  }
  if (!cur.done && itn > 0) {
    const bool graph = ctx->opts.use_graph != 0 && !timed;
    if (graph && (rc = ensure_graph(ctx))) return rc;
    nvtxRangePushA("LSQR_MAIN_ITERATION");
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    const int chunk = args->stop_on_istop ? 10 : itn;
    while (done_itn < itn) {
      const int k = std::min(chunk, itn - done_itn);
      for (int i = 0; i < k; ++i) {
        if (graph)
          CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
        else if ((rc = enqueue_iteration(
                      ctx, ctx->stream,
                      timed ? evs.data() + (size_t)(done_itn + i) * (kRegions + 1) : nullptr)))
          return rc;
      }
      done_itn += k;
      if (args->stop_on_istop && done_itn < itn) {
        CK(cudaMemcpyAsync(&cur, ctx->st, sizeof(cur), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (cur.istop != 0) break;
      }
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaEventSynchronize(ctx->ev1));
    nvtxRangePop();
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    CK(cudaEventElapsedTime(&ms_total, ctx->ev_start, ctx->ev1));
  }
  if (timed) {
    ctx->t_ms.assign((size_t)done_itn * kRegions, 0.f);
    for (int i = 0; i < done_itn; ++i)
      for (int r = 0; r < kRegions; ++r)
        CK(cudaEventElapsedTime(&ctx->t_ms[(size_t)i * kRegions + r],
                                evs[(size_t)i * (kRegions + 1) + r],
                                evs[(size_t)i * (kRegions + 1) + r + 1]));
    ctx->t_iters = done_itn;
    ctx->t_loop_ms = ms;
    ctx->t_startup_ms = ms_total - ms;
  }
  if (ctx->want_se && done_itn > 0)
    k_finish_se<<<ctx->gvx, kThreads, 0, ctx->stream>>>(ctx->se, ctx->n, ctx->st, ctx->m_k + ctx->m_d);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&cur, ctx->st, sizeof(cur), cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<plsqr_iter> hh((size_t)itn + 1);
  CK(cudaMemcpyAsync(hh.data(), ctx->hist, sizeof(plsqr_iter) * (itn + 1), cudaMemcpyDeviceToHost,
                     ctx->stream));
  if (x) CK(cudaMemcpyAsync(x, ctx->x, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  if (w) CK(cudaMemcpyAsync(w, ctx->w, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  if (se && ctx->want_se)
    CK(cudaMemcpyAsync(se, ctx->se, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->solved = true;

  plsqr_result r;
  memset(&r, 0, sizeof(r));
  r.istop = (args->damp > 0.0 && cur.istop == 2) ? 3 : cur.istop;  // lsqr.c:895-896
  r.itn = cur.itn;
  r.anorm = cur.anorm;
  r.acond = cur.acond;
  r.rnorm = cur.rnorm;
  r.arnorm_out = cur.test2;
  r.xnorm = cur.xnorm;
  r.arnorm = cur.arnorm;
  r.bnorm = cur.bnorm;
  r.dxmax = cur.dxmax;
  r.maxdx = cur.maxdx;
  r.seconds = ms * 1e-3;
  r.seconds_total = ms_total * 1e-3;
  if (res) *res = r;
  if (hist) memcpy(hist, hh.data(), sizeof(plsqr_iter) * (itn + 1));
  if (ctx->opts.verbose) print_iterations(hh.data(), r.itn, r.seconds);
  if (args->result_txt) {
    if ((rc = write_result_txt(args->result_txt, ctx->m_k + ctx->m_d, ctx->n, args, hh.data(),
                               cur.done ? -1 : r.itn, &r)))
      return rc;
  }
  return PLSQR_OK;
}

int plsqr_bench_aprod(plsqr_ctx *ctx, int mode, int reps, double *ms_per_launch) {
  if (!ctx || (mode != 1 && mode != 2) || reps < 1 || !ms_per_launch) return PLSQR_ERR_ARG;
  if (ctx->opts.precision == PLSQR_PREC_MIXED) return mixed_bench_aprod(ctx, mode, reps, ms_per_launch);
  CK(cudaSetDevice(ctx->opts.device));
  int rc;
  if ((rc = launch_aprod(ctx, mode, kScaleOne, false))) return rc;  // warm-up
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int i = 0; i < reps; ++i)
    if ((rc = launch_aprod(ctx, mode, kScaleOne, false))) return rc;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *ms_per_launch = (double)ms / reps;
  return PLSQR_OK;
}

int plsqr_bench_iteration(plsqr_ctx *ctx, int reps, double *ms_per_iteration) {
  if (!ctx || reps < 1 || !ms_per_iteration) return PLSQR_ERR_ARG;
  if (ctx->opts.precision == PLSQR_PREC_MIXED) return mixed_bench_iteration(ctx, reps, ms_per_iteration);
  if (!ctx->solved) return PLSQR_ERR_STATE;
  CK(cudaSetDevice(ctx->opts.device));
  int rc;
  if (ctx->hist_cap < reps + 1) {  // every replay writes one history record
    dev_free(ctx, ctx->hist);
    ctx->hist = nullptr;
    ctx->hist_cap = 0;
    if ((rc = dev_alloc(ctx, &ctx->hist, (size_t)reps + 1))) return rc;
    ctx->hist_cap = reps + 1;
  }
  if ((rc = ensure_graph(ctx))) return rc;
  // continue from the state of the last solve, history from index 1
  DevState h;
  CK(cudaMemcpy(&h, ctx->st, sizeof(h), cudaMemcpyDeviceToHost));
  h.itn = 0;
  h.hist_base = 0;
  CK(cudaMemcpy(ctx->st, &h, sizeof(h), cudaMemcpyHostToDevice));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int i = 0; i < reps; ++i) CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *ms_per_iteration = (double)ms / reps;
  return PLSQR_OK;
}

int plsqr_set_timing(plsqr_ctx *ctx, int on) {
  if (!ctx) return PLSQR_ERR_ARG;
  ctx->timing = on != 0;
  return PLSQR_OK;
}

int plsqr_write_timing(const plsqr_ctx *ctx, const char *path) {
  if (!ctx || !path) return PLSQR_ERR_ARG;
  if (ctx->t_iters <= 0) return PLSQR_ERR_STATE;
  FILE *f = fopen(path, "w");
  if (!f) return PLSQR_ERR_IO;
  const int n = ctx->t_iters;
  fprintf(f, "{\n \"timer\": \"CUDA events on the context's stream around each region\",\n");
  fprintf(f, " \"order\": \"%s\",\n \"iterations\": %d,\n", ctx->exact ? "reference" : "fast", n);
  fprintf(f, " \"LSQR_MAIN_ITERATION\": {\"seconds\": %.9g},\n", 1e-3 * ctx->t_loop_ms);
  fprintf(f, " \"startup_seconds\": %.9g,\n \"regions\": [\n", 1e-3 * ctx->t_startup_ms);
  for (int r = 0; r < kRegions; ++r) {
    double sum = 0.0, mn = 1e300, mx = 0.0;
    for (int i = 0; i < n; ++i) {
      const double t = ctx->t_ms[(size_t)i * kRegions + r];
      sum += t;
      mn = std::min(mn, t);
      mx = std::max(mx, t);
    }
    fprintf(f,
            "  {\"name\": \"%s\", \"covers\": \"%s\", \"seconds\": %.9g, "
            "\"ms_per_iteration\": %.6g, \"min_ms\": %.6g, \"max_ms\": %.6g}%s\n",
            kRegionName[r], kRegionCovers[r], 1e-3 * sum, sum / n, mn, mx,
            r + 1 < kRegions ? "," : "");
  }
  fprintf(f, " ],\n \"per_iteration_ms\": {\n");
  for (int r = 0; r < kRegions; ++r) {
    fprintf(f, "  \"%s\": [", kRegionName[r]);
    for (int i = 0; i < n; ++i)
      fprintf(f, "%s%.5g", i ? ", " : "", (double)ctx->t_ms[(size_t)i * kRegions + r]);
    fprintf(f, "]%s\n", r + 1 < kRegions ? "," : "");
  }
  fprintf(f, " }\n}\n");
  return fclose(f) == 0 ? PLSQR_OK : PLSQR_ERR_IO;
}

int plsqr_get_x(plsqr_ctx *ctx, double *x) {
  if (!ctx || !x) return PLSQR_ERR_ARG;
  if (!ctx->solved) return PLSQR_ERR_STATE;
  CK(cudaSetDevice(ctx->opts.device));
  CK(cudaMemcpy(x, ctx->x, sizeof(double) * ctx->n, cudaMemcpyDeviceToHost));
  return PLSQR_OK;
}

int plsqr_write_result(plsqr_ctx *ctx, const char *path) {
  if (!ctx || !path) return PLSQR_ERR_ARG;
  std::vector<double> x((size_t)ctx->n);
  int rc = plsqr_get_x(ctx, x.data());
  if (rc) return rc;
  return plsqr_io_write_x(path, ctx->n, x.data());
}

}  // extern "C"
