// plsqr_ctx_create_files: the loading half of PLSQR3_main
// (source/plsqr3.c:197-589) on one partition: kernel info and records (with
// the optional column permutation of the COL_PERM build), damping row info
// and records, damping column info and records, b_k; then the device
// context.
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "plsqr_internal.h"

namespace {

std::string join(const char *dir, const char *name) {
  std::string d = dir ? dir : ".";
  return d + "/" + (name ? name : "");
}

}  // namespace

extern "C" int plsqr_ctx_create_files(const plsqr_files *f, const plsqr_opts *opts,
                                      plsqr_ctx **out) {
  if (!f || !out || !f->ker_f || !f->ker_i || !f->damp_f || !f->damp_i || !f->damp_f_bycol ||
      !f->damp_i_bycol || !f->b_k)
    return PLSQR_ERR_ARG;
  *out = nullptr;
  const int32_t m_k = f->row_k, m_d = f->row_d, n = f->col;
  if (m_k < 0 || m_d < 0 || n < 1) return PLSQR_ERR_ARG;
  int rc;
  // kernel (plsqr3.c:219-344)
  std::vector<int32_t> cnt((size_t)n);
  std::vector<int64_t> start((size_t)n);
  int64_t nnz_k = 0;
  const std::string ki = join(f->dir, f->ker_i), kf = join(f->dir, f->ker_f);
  if ((rc = plsqr_io_read_kernel_info(ki.c_str(), n, cnt.data(), start.data(), &nnz_k))) return rc;
  std::vector<int64_t> kcp((size_t)n + 1);
  std::vector<int32_t> kri((size_t)nnz_k);
  std::vector<double> kv((size_t)nnz_k);
  if ((rc = plsqr_io_read_kernel(kf.c_str(), ki.c_str(), m_k, n, kcp.data(), kri.data(), kv.data())))
    return rc;
  cnt.clear();
  start.clear();
  if (f->col_perm) {  // COL_PERM (plsqr3.c:261-283, 1652-1713): column i = file column perm[i]
    std::vector<int32_t> perm((size_t)n);
    const std::string pf = join(f->dir, f->col_perm);
    if ((rc = plsqr_io_read_col_perm(pf.c_str(), n, perm.data()))) return rc;
    std::vector<int64_t> pcp((size_t)n + 1);
    for (int32_t i = 0; i < n; ++i) pcp[i + 1] = pcp[i] + (kcp[perm[i] + 1] - kcp[perm[i]]);
    std::vector<int32_t> pri((size_t)pcp[n]);
    std::vector<double> pv((size_t)pcp[n]);
    if ((rc = plsqr_permute_columns(n, kcp.data(), kri.data(), kv.data(), perm.data(), pcp.data(),
                                    pri.data(), pv.data())))
      return rc;
    kcp.swap(pcp);
    kri.swap(pri);
    kv.swap(pv);
    nnz_k = kcp[n];
  }
  // damping by row (plsqr3.c:381-447)
  std::vector<int32_t> dcnt((size_t)m_d);
  int64_t nnz_d = 0;
  const std::string di = join(f->dir, f->damp_i), df = join(f->dir, f->damp_f);
  if ((rc = plsqr_io_read_int32_counts(di.c_str(), m_d, dcnt.data(), &nnz_d))) return rc;
  std::vector<int64_t> drp((size_t)m_d + 1);
  std::vector<int32_t> dci((size_t)nnz_d);
  std::vector<double> dv((size_t)nnz_d);
  if ((rc = plsqr_io_read_damping(df.c_str(), 0, m_d, n, nnz_d, drp.data(), dci.data(), dv.data())))
    return rc;
  for (int32_t r = 0; r < m_d; ++r)
    if (drp[r + 1] - drp[r] != dcnt[r]) return PLSQR_ERR_FORMAT;
  // damping by column (plsqr3.c:496-531)
  std::vector<int32_t> ccnt((size_t)n);
  int64_t nnz_dc = 0;
  const std::string ci = join(f->dir, f->damp_i_bycol), cf = join(f->dir, f->damp_f_bycol);
  if ((rc = plsqr_io_read_int32_counts(ci.c_str(), n, ccnt.data(), &nnz_dc))) return rc;
  if (nnz_dc != nnz_d) return PLSQR_ERR_FORMAT;
  std::vector<int64_t> dcp((size_t)n + 1);
  std::vector<int32_t> dri((size_t)nnz_dc);
  std::vector<double> dcv((size_t)nnz_dc);
  if ((rc = plsqr_io_read_damping(cf.c_str(), 1, m_d, n, nnz_dc, dcp.data(), dri.data(), dcv.data())))
    return rc;
  for (int32_t c = 0; c < n; ++c)
    if (dcp[c + 1] - dcp[c] != ccnt[c]) return PLSQR_ERR_FORMAT;
  // b_k (plsqr3.c:580-589)
  std::vector<double> b((size_t)m_k);
  const std::string bf = join(f->dir, f->b_k);
  if ((rc = plsqr_io_read_rhs(bf.c_str(), m_k, b.data()))) return rc;

  plsqr_sparse K = {m_k, n, nnz_k, nullptr, kcp.data(), kri.data(), kv.data()};
  plsqr_sparse D = {m_d, n, nnz_d, nullptr, drp.data(), dci.data(), dv.data()};
  plsqr_sparse DC = {m_d, n, nnz_dc, nullptr, dcp.data(), dri.data(), dcv.data()};
  plsqr_ctx *ctx = nullptr;
  if ((rc = plsqr_ctx_create(&K, &D, &DC, opts, &ctx))) return rc;
  ctx->b_k.swap(b);
  *out = ctx;
  return PLSQR_OK;
}
