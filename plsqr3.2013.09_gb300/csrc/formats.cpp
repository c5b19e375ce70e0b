// Readers and writers of the PLSQR3 input/output files (host side).
//
// On-disk formats (README:47-148 of the reference):
//  * matrix records: 16 bytes {int32 row, int32 col, float64 value}, 1-based,
//    the NONZERO struct of source/main.h:114-117;
//  * kernel info: ASCII lines "col nnz start", 1-based, start 0 when nnz is 0
//    (written by Ker2PLSQR3.c:499-513, read by plsqr3.c:1379-1409);
//  * damping info: int32 per row (or per column), native endianness;
//  * b_k: ASCII, one %le value per line (plsqr3.c:580-589);
//  * result x: raw float64[n] (plsqr3.c:1986-2013).
//
// The readers follow the reference loaders' semantics on one partition and
// turn every condition on which the reference calls exit(-1) into an error
// code.  Three checks are stricter than the reference, each on inputs for
// which the reference silently produces wrong matrices: a file shorter than
// its info says, negative indices, and damping records that are not sorted
// by row (by column for the column file) or disagree with the info counts.
#include "plsqr_host.h"

#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace {

struct Record {
  int32_t r, c;
  double v;
};
static_assert(sizeof(Record) == 16, "record must be 16 bytes");

const int64_t kChunk = 10000000;  // records per read, as MPIIO_CHUNK_SIZE

struct File {
  FILE *f = nullptr;
  File(const char *p, const char *m) { f = p ? fopen(p, m) : nullptr; }
  ~File() {
    if (f) fclose(f);
  }
};

// Read `count` records starting at record index `first`.
template <class F>
int read_records(const char *path, int64_t first, int64_t count, F &&sink) {
  File in(path, "rb");
  if (!in.f) return PLSQR_ERR_IO;
  if (first > 0 && fseeko(in.f, (off_t)(first * 16), SEEK_SET) != 0) return PLSQR_ERR_FORMAT;
  std::vector<Record> buf((size_t)std::min<int64_t>(std::max<int64_t>(count, 1), kChunk));
  int64_t done = 0;
  while (done < count) {
    const int64_t want = std::min<int64_t>(kChunk, count - done);
    const size_t got = fread(buf.data(), sizeof(Record), (size_t)want, in.f);
    if ((int64_t)got != want) return PLSQR_ERR_FORMAT;  // truncated file
    for (int64_t i = 0; i < want; ++i) {
      int rc = sink(done + i, buf[(size_t)i]);
      if (rc) return rc;
    }
    done += want;
  }
  return PLSQR_OK;
}

}  // namespace

extern "C" {

int plsqr_io_read_kernel_info(const char *path, int32_t n, int32_t *nnz, int64_t *start,
                              int64_t *total) {
  if (!path || n < 0 || (n > 0 && (!nnz || !start))) return PLSQR_ERR_ARG;
  File in(path, "r");
  if (!in.f) return PLSQR_ERR_IO;
  int64_t sum = 0;
  for (int32_t i = 0; i < n; ++i) {
    int col, cnt;
    long long st;
    if (fscanf(in.f, "%d %d %lld", &col, &cnt, &st) != 3) return PLSQR_ERR_FORMAT;
    if (cnt < 0) return PLSQR_ERR_FORMAT;
    nnz[i] = cnt;
    start[i] = (int64_t)st - 1;  // 0-based, -1 where the file has 0
    sum += cnt;
  }
  if (total) *total = sum;
  return PLSQR_OK;
}

int plsqr_io_read_kernel(const char *bin_path, const char *info_path, int32_t m_k,
                         int32_t n, int64_t *col_ptr, int32_t *row_idx, double *val) {
  if (!bin_path || !info_path || m_k < 0 || n < 0 || !col_ptr) return PLSQR_ERR_ARG;
  std::vector<int32_t> cnt((size_t)n + 1);
  std::vector<int64_t> st((size_t)n + 1);
  int64_t total = 0;
  int rc = plsqr_io_read_kernel_info(info_path, n, cnt.data(), st.data(), &total);
  if (rc) return rc;
  // plsqr3.c:1556-1563: the records start at the first non-empty column
  int64_t first = 0;
  for (int32_t i = 0; i < n; ++i)
    if (cnt[(size_t)i] > 0) {
      first = st[(size_t)i];
      break;
    }
  if (first < 0) return PLSQR_ERR_FORMAT;
  col_ptr[0] = 0;
  for (int32_t i = 0; i < n; ++i) col_ptr[i + 1] = col_ptr[i] + cnt[(size_t)i];  // :1599
  if (total > 0 && (!row_idx || !val)) return PLSQR_ERR_ARG;
  return read_records(bin_path, first, total, [&](int64_t e, const Record &rec) {
    const int32_t r0 = rec.r - 1;                     // :1606
    if (r0 >= m_k || r0 < 0) return PLSQR_ERR_FORMAT;  // :1610-1615
    row_idx[e] = r0;
    val[e] = rec.v;
    return PLSQR_OK;
  });
}

int plsqr_io_read_int32_counts(const char *path, int64_t count, int32_t *out, int64_t *total) {
  if (!path || count < 0 || (count > 0 && !out)) return PLSQR_ERR_ARG;
  File in(path, "rb");
  if (!in.f) return PLSQR_ERR_IO;
  if ((int64_t)fread(out, sizeof(int32_t), (size_t)count, in.f) != count) return PLSQR_ERR_FORMAT;
  int64_t s = 0;
  for (int64_t i = 0; i < count; ++i) {
    if (out[i] < 0) return PLSQR_ERR_FORMAT;
    s += out[i];
  }
  if (total) *total = s;
  return PLSQR_OK;
}

// plsqr3.c:1027-1194 for one rank: the records are read in file order; the
// line (row for CSR, column for CSC) of each record decides its line count.
int plsqr_io_read_damping(const char *bin_path, int by_col, int32_t m_d, int32_t n,
                          int64_t nnz, int64_t *ptr, int32_t *idx, double *val) {
  if (!bin_path || m_d < 0 || n < 0 || nnz < 0 || !ptr) return PLSQR_ERR_ARG;
  if (nnz > 0 && (!idx || !val)) return PLSQR_ERR_ARG;
  const int32_t n_lines = by_col ? n : m_d;
  std::vector<int64_t> cnt((size_t)n_lines + 1, 0);
  int64_t prev_line = 0;
  int rc = read_records(bin_path, 0, nnz, [&](int64_t e, const Record &rec) {
    const int32_t r = rec.r - 1, c = rec.c - 1;  // :1143, :1173
    // :1149-1153 and :1178-1182 bounds checks
    if (r < 0 || r >= m_d || c < 0 || c >= n) return PLSQR_ERR_FORMAT;
    const int32_t line = by_col ? c : r;
    if (line < prev_line) return PLSQR_ERR_FORMAT;  // not sorted by line
    prev_line = line;
    cnt[(size_t)line]++;
    idx[e] = by_col ? r : c;
    val[e] = rec.v;
    return PLSQR_OK;
  });
  if (rc) return rc;
  ptr[0] = 0;
  for (int32_t i = 0; i < n_lines; ++i) ptr[i + 1] = ptr[i] + cnt[(size_t)i];  // :1158-1161
  return PLSQR_OK;
}

int plsqr_io_read_rhs(const char *path, int32_t m_k, double *b_k) {
  if (!path || m_k < 0 || (m_k > 0 && !b_k)) return PLSQR_ERR_ARG;
  File in(path, "r");
  if (!in.f) return PLSQR_ERR_IO;
  for (int32_t i = 0; i < m_k; ++i)
    if (fscanf(in.f, "%le", &b_k[i]) != 1) return PLSQR_ERR_FORMAT;
  return PLSQR_OK;
}

int plsqr_io_read_col_perm(const char *path, int32_t n, int32_t *perm) {
  if (!path || n < 0 || (n > 0 && !perm)) return PLSQR_ERR_ARG;
  File in(path, "r");
  if (!in.f) return PLSQR_ERR_IO;
  for (int32_t i = 0; i < n; ++i) {
    int c = 0;
    if (fscanf(in.f, "%d", &c) != 1 || c < 1 || c > n) return PLSQR_ERR_FORMAT;
    perm[i] = c - 1;  // 0-based (plsqr3.c:1357)
  }
  return PLSQR_OK;
}

int plsqr_permute_columns(int32_t n, const int64_t *ptr, const int32_t *idx, const double *val,
                          const int32_t *perm, int64_t *tptr, int32_t *tidx, double *tval) {
  if (n < 0 || !ptr || !perm || !tptr) return PLSQR_ERR_ARG;
  tptr[0] = 0;
  for (int32_t i = 0; i < n; ++i) {
    if (perm[i] < 0 || perm[i] >= n) return PLSQR_ERR_ARG;
    tptr[i + 1] = tptr[i] + (ptr[perm[i] + 1] - ptr[perm[i]]);
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < n; ++i) {
    const int64_t a = ptr[perm[i]], k = ptr[perm[i] + 1] - a;
    if (k > 0) {
      memcpy(tidx + tptr[i], idx + a, sizeof(int32_t) * (size_t)k);
      memcpy(tval + tptr[i], val + a, sizeof(double) * (size_t)k);
    }
  }
  return PLSQR_OK;
}

int plsqr_io_write_kernel(const char *bin_path, const char *info_path, int32_t m_k, int32_t n,
                          const int64_t *col_ptr, const int32_t *row_idx, const double *val) {
  if (!bin_path || !info_path || m_k < 0 || n < 0 || !col_ptr) return PLSQR_ERR_ARG;
  File info(info_path, "w"), bin(bin_path, "wb");
  if (!info.f || !bin.f) return PLSQR_ERR_IO;
  // Ker2PLSQR3.c:505-512: "col nnz start", start is 1-based, 0 for empty
  long long start1 = 1;
  for (int32_t c = 0; c < n; ++c) {
    const long long k = (long long)(col_ptr[c + 1] - col_ptr[c]);
    if (k < 0) return PLSQR_ERR_ARG;
    if (fprintf(info.f, "%d %lld %lld\n", c + 1, k, k == 0 ? 0LL : start1) < 0) return PLSQR_ERR_IO;
    start1 += k;
  }
  std::vector<Record> buf;
  buf.reserve((size_t)std::min<int64_t>(kChunk, std::max<int64_t>(col_ptr[n], 1)));
  for (int32_t c = 0; c < n; ++c) {
    for (int64_t e = col_ptr[c]; e < col_ptr[c + 1]; ++e) {
      if (row_idx[e] < 0 || row_idx[e] >= m_k) return PLSQR_ERR_ARG;
      buf.push_back(Record{row_idx[e] + 1, c + 1, val[e]});
      if ((int64_t)buf.size() == kChunk) {
        if (fwrite(buf.data(), sizeof(Record), buf.size(), bin.f) != buf.size()) return PLSQR_ERR_IO;
        buf.clear();
      }
    }
  }
  if (!buf.empty() && fwrite(buf.data(), sizeof(Record), buf.size(), bin.f) != buf.size())
    return PLSQR_ERR_IO;
  return PLSQR_OK;
}

static int write_lines(const char *bin_path, const char *info_path, int32_t n_lines,
                       int32_t n_idx, int by_col, const int64_t *ptr, const int32_t *idx,
                       const double *val) {
  File info(info_path, "wb"), bin(bin_path, "wb");
  if (!info.f || !bin.f) return PLSQR_ERR_IO;
  std::vector<Record> buf;
  for (int32_t l = 0; l < n_lines; ++l) {
    const int64_t k = ptr[l + 1] - ptr[l];
    if (k < 0 || k > INT32_MAX) return PLSQR_ERR_ARG;
    const int32_t k32 = (int32_t)k;
    if (fwrite(&k32, sizeof(int32_t), 1, info.f) != 1) return PLSQR_ERR_IO;
    for (int64_t e = ptr[l]; e < ptr[l + 1]; ++e) {
      if (idx[e] < 0 || idx[e] >= n_idx) return PLSQR_ERR_ARG;
      buf.push_back(by_col ? Record{idx[e] + 1, l + 1, val[e]} : Record{l + 1, idx[e] + 1, val[e]});
      if ((int64_t)buf.size() == kChunk) {
        if (fwrite(buf.data(), sizeof(Record), buf.size(), bin.f) != buf.size()) return PLSQR_ERR_IO;
        buf.clear();
      }
    }
  }
  if (!buf.empty() && fwrite(buf.data(), sizeof(Record), buf.size(), bin.f) != buf.size())
    return PLSQR_ERR_IO;
  return PLSQR_OK;
}

int plsqr_io_write_damping(const char *row_bin, const char *row_info, const char *col_bin,
                           const char *col_info, int32_t m_d, int32_t n, const int64_t *row_ptr,
                           const int32_t *col_idx, const double *val, const int64_t *col_ptr,
                           const int32_t *row_idx, const double *cval) {
  if (m_d < 0 || n < 0) return PLSQR_ERR_ARG;
  int rc = PLSQR_OK;
  if (row_bin && row_info) rc = write_lines(row_bin, row_info, m_d, n, 0, row_ptr, col_idx, val);
  if (rc) return rc;
  if (col_bin && col_info) rc = write_lines(col_bin, col_info, n, m_d, 1, col_ptr, row_idx, cval);
  return rc;
}

int plsqr_io_write_rhs(const char *path, int32_t m_k, const double *b_k) {
  if (!path || m_k < 0) return PLSQR_ERR_ARG;
  File out(path, "w");
  if (!out.f) return PLSQR_ERR_IO;
  for (int32_t i = 0; i < m_k; ++i)
    if (fprintf(out.f, "%.17e\n", b_k[i]) < 0) return PLSQR_ERR_IO;
  return PLSQR_OK;
}

int plsqr_io_write_x(const char *path, int32_t n, const double *x) {
  if (!path || n < 0 || (n > 0 && !x)) return PLSQR_ERR_ARG;
  File out(path, "wb");
  if (!out.f) return PLSQR_ERR_IO;
  if ((int32_t)fwrite(x, sizeof(double), (size_t)n, out.f) != n) return PLSQR_ERR_IO;
  return PLSQR_OK;
}

}  // extern "C"
