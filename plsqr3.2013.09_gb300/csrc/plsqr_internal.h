// Internal definitions shared by the device and host sources of the library.
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "dev_types.h"
#include "plsqr_gpu.h"

// One compressed-sparse operand in device memory.
struct DevLines {
  int64_t *ptr = nullptr;
  int32_t *idx = nullptr;
  double *val = nullptr;
  int32_t n_lines = 0;
  int64_t nnz = 0;
  plsqr::Csr csr() const { return plsqr::Csr{ptr, idx, val, n_lines}; }
};

// One operand in the slab layout (slab.cuh), with its block partition.
template <typename T>
struct DevSlab {
  int64_t *ptr = nullptr;
  uint16_t *idx = nullptr;
  T *val = nullptr;
  int32_t n_lines = 0, n_slabs = 0, slab = 0, n_idx = 0;
  int64_t nnz_padded = 0;
  int32_t *lpart = nullptr;  // [n_slabs * (bps + 1)] line ranges of the blocks
  int32_t *order = nullptr;  // [n_slabs * n_lines] visit order inside each range
  int bps = 0;               // blocks per slab
  T *partial = nullptr;      // [n_slabs * n_lines]
  size_t smem = 0;           // shared memory per block
  // persistent form (k_slab_spmv_dyn): per-slab line counters, or null for
  // the static block-per-range form; its grid
  int *next = nullptr;
  int dyn_blocks = 0;
  int chunk = 4;  // passes of lines a warp takes per counter grab
};

// The kernel matrix by column or by row in the unit layout (units.cuh);
// FP64 values for the FP64 products, FP32 for the mixed solver's.
template <typename T>
struct DevUnitsT {
  uint16_t *idx = nullptr;
  T *val = nullptr;
  int64_t *slot0 = nullptr;
  int32_t *q = nullptr, *c = nullptr, *line = nullptr, *unit_begin = nullptr;
  int32_t n_lines = 0, n_slabs = 0, slab = 0, n_idx = 0, n_units = 0;
  int32_t threads = 1024;       // block size of k_slab_units: 1,024 or 512
  bool hilo = false;            // FP32: shared memory sized for hi + lo pairs
  int32_t chains = 2;           // FP64: accumulator chains per lane (2 or 4)
  int32_t pf_dist = 1, pf_pieces = 1;  // L2 prefetch of the unit kernel (set by build_units)
  int64_t slots = 0;
  int *next = nullptr;         // [n_slabs] unit counters, zeroed before every launch
  double *partial = nullptr;   // [n_slabs * n_lines], FP64 for either value type
  int blocks = 0;
  size_t smem = 0;
};
using DevUnits = DevUnitsT<double>;

struct MixedState;  // mixed.cu
struct BatchState;  // batched.cu

struct plsqr_ctx {
  plsqr_opts opts;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_start = nullptr;
  int32_t m_k = 0, m_d = 0, n = 0;
  int64_t nnz_k = 0, nnz_d = 0;
  int sm_count = 0, blocks_per_sm = 0, unroll = 2;
  int m2_blocks_per_sm = 48;
  int32_t *kpart = nullptr, *cpart = nullptr;  // balanced warp -> line ranges
  int32_t *corder = nullptr;                     // column visit order of A^T y
  DevLines K, D, KC, DC;  // kernel/damping by row, kernel/damping by column
  double *u = nullptr, *v = nullptr, *w = nullptr, *x = nullptr, *se = nullptr, *xref = nullptr;
  double *parts_u = nullptr, *parts_v = nullptr, *parts_dk = nullptr, *parts_err = nullptr;
  plsqr::DevState *st = nullptr;
  plsqr_iter *hist = nullptr;
  int hist_cap = 0;
  bool want_se = false, has_ref = false, solved = false;
  int g1k = 1, g1d = 1, g2 = 1, gvu = 1, gvx = 1, gsk = 1, gsd = 1;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_key = -1;
  plsqr_iter *graph_hist = nullptr;
  std::vector<double> b_k;  // right-hand side loaded from the files, if any
  std::vector<std::pair<void *, size_t>> allocs;
  int64_t device_bytes = 0;
  char last_error[512] = {0};
  MixedState *mixed = nullptr;
  // slab layout of the kernel matrix (default FP64 product path)
  bool use_slabs = false;  // FP64 A^T y on slabs
  bool use_slabs_rows = false;  // FP64 A x on slabs
  bool slab_ok = false;    // dimensions fit the slab layout
  int slab_group = 8;      // lanes per segment, FP64 slab products
  int slab_group_f = 16;   // lanes per segment, FP32 slab products
  DevSlab<double> s_rows, s_cols;  // K by row (gathers v), K by column (gathers u_k)
  bool use_units = false;          // FP64 A^T y on the unit layout (default)
  DevUnits u_cols;                 // K by column in the unit layout
  bool use_units_rows = false;     // FP64 A x on the unit layout
  DevUnits u_rows;                 // K by row in the unit layout
  bool lines_released = false;     // opts.lean freed K.idx/val or KC.idx/val
  int gc1k = 1, gc1d = 1, gc2 = 1;  // grids of the combine kernels
  BatchState *batch = nullptr;       // several right-hand sides (batched.cu)
  double *d_val0 = nullptr, *dc_val0 = nullptr;  // damping values before weighting
  // PLSQR_ORDER_REFERENCE: the reference's order of operations (kernels_exact.cuh)
  bool exact = false;
  double *ex_terms = nullptr;  // [max(m, n)] norm and dknorm terms
  double *ex_bmax = nullptr;   // per-chunk maxima of the norm passes
  int ex_nb_k = 0, ex_nb_d = 0, ex_nb_v = 0;  // norm-pass blocks of y_k, y_d, v
  int ex_gk = 1, ex_gd = 1, ex_gc = 1;        // grids of the product kernels
  // timing report (plsqr_set_timing / plsqr_write_timing)
  bool timing = false;
  std::vector<float> t_ms;  // [iterations][regions] device time of each region
  int t_iters = 0;          // iterations of the last timed solve (0: none)
  float t_loop_ms = 0.f, t_startup_ms = 0.f;
};

// plsqr_gpu.cu: PLSQR_ERR_NUMERIC for NaN, Inf, or a largest magnitude
// above 2^500 or (nonzero, unless allow_small) below 2^-500
int magnitude_ok(const double *p, int64_t n, int allow_small = 0);

// slab.cu
template <typename T>
// tgroup > 1: transpose each segment's chunks for products that stream it
// with tgroup lanes (slab_pos in slab.cuh); 0 keeps the order
// dyn_blocks > 0: the persistent form with that many blocks (one range per
// slab, the whole slab in longest-segment-first order); 0: the static form
int build_slab(plsqr_ctx *ctx, const DevLines &L, int32_t n_idx, int32_t slab, int blocks,
               DevSlab<T> *out, int tgroup = 0, int dyn_blocks = 0);
// The scheduling of the slab products from the environment: PLSQR_SLAB_SCHED
// (FP64) or PLSQR_SLAB_SCHED_F (FP32), 1 persistent, 0 static; returns the
// persistent grid or 0.
int slab_dyn_blocks(const plsqr_ctx *ctx, bool fp32);
int slab_plan(plsqr_ctx *ctx);
template <typename T>
int build_units(plsqr_ctx *ctx, const DevLines &L, int32_t n_idx, int32_t slab,
                DevUnitsT<T> *out, bool hilo = false, bool lane_lines = false);
// slabs of `slab` entries over an index space of n_idx: few enough for the
// build, 16-bit indices, and the slab and summing area of 1,024 threads in
// shared memory
template <typename T>
bool units_fit(int32_t n_idx, int32_t slab, bool hilo = false);
// slab.cu / batched.cu: the bounds-check words of their kernels (check.cuh)
unsigned slab_check_word(bool reset);
unsigned batched_check_word(bool reset);
// plsqr_gpu.cu: unit product launch and its shared-memory attribute
// x_lo (FP32 layouts built with hilo): the low halves of the pairs x + x_lo
template <typename T>
void units_spmv(const DevUnitsT<T> &U, const T *x, cudaStream_t s, const T *x_lo = nullptr);
template <typename T>
int units_set_smem(size_t smem);
// plsqr_gpu.cu: slab product launch and its shared-memory attribute
template <typename T>
void slab_spmv(const DevSlab<T> &S, int group, const T *x, cudaStream_t s);
template <typename T>
int slab_set_smem(size_t smem);
// plsqr_gpu.cu: partial-sum counts of the current product path
int ctx_pu_k(const plsqr_ctx *ctx);
int ctx_pu_d(const plsqr_ctx *ctx);
int ctx_pv(const plsqr_ctx *ctx);

void ctx_set_error(plsqr_ctx *ctx, const char *fmt, ...);
int ctx_dev_alloc_bytes(plsqr_ctx *ctx, void **p, size_t bytes);
void ctx_dev_free(plsqr_ctx *ctx, void *p);

template <class T>
inline int dev_alloc(plsqr_ctx *ctx, T **p, size_t count) {
  void *q = nullptr;
  const int rc = ctx_dev_alloc_bytes(ctx, &q, (count > 0 ? count : 1) * sizeof(T));
  *p = (T *)q;
  return rc;
}
inline void dev_free(plsqr_ctx *ctx, void *p) { ctx_dev_free(ctx, p); }

// report.cpp
int write_result_txt(const char *path, int num_row, int n, const plsqr_lsqr_args *args,
                     const plsqr_iter *hist, int itn, const plsqr_result *r);
void print_iterations(const plsqr_iter *hist, int itn, double seconds);

// mixed.cu
int mixed_prepare(plsqr_ctx *ctx);
int mixed_lsqr(plsqr_ctx *ctx, const plsqr_lsqr_args *args, const double *b_k, double *x,
               double *w, double *se, plsqr_iter *hist, plsqr_result *res);
void mixed_free(plsqr_ctx *ctx);
int mixed_bench_aprod(plsqr_ctx *ctx, int mode, int reps, double *ms_per_launch);
int mixed_bench_iteration(plsqr_ctx *ctx, int reps, double *ms_per_iteration);

// batched.cu
void batch_free(plsqr_ctx *ctx);
