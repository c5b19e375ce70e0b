// Synthetic tomography problems in the reference's data model.
//
// The model grid is nx*ny*nz cells, column index = iz*ny*nx + iy*nx + ix
// (the cell map of PLSQR3_tools/damping_format/damping_binary.py:47-50).
//
//  * Kernel matrix K: one row per ray.  A ray joins two uniform-random points
//    on the two opposite grid faces normal to `face_axis`; its nonzeros are the
//    cells whose centre lies within `tube_radius` of the segment, each valued
//    |N(0,1)| * value_scale.  Columns of a row are ascending.
//  * Damping matrix D, rows in the per-cell order of damping_binary.py:84-511:
//    identity row (weight damp_identity), the forward 1,-2,1 second difference
//    along x, y, z (weight damp_lap), and, when damp_cross != 0, the cross
//    differences 0.5 * (1, -1, -1, 1) over the corners (0,0), (2,0), (0,2),
//    (2,2) of the xy, xz and yz planes (weight damp_cross); a row only where
//    its stencil fits in the grid.  With n_params fields the whole block
//    repeats per field (damping_binary.py:84, 578-610).
//  * x_true: Gaussian blobs (centre uniform in the grid, amplitude N(0,1)) plus
//    an optional +-checker_amp checkerboard of period checker_period cells.
//  * b_k = K x_true + noise_frac * rms(K x_true) * N(0,1).
//
// Every random number comes from a counter-based hash of (seed, stream,
// indices), so any subset can be generated in any order and in parallel.  All
// arithmetic uses + - * / sqrt only (log and exp below are written out from
// their series) so that the same bits come out on x86_64 and aarch64; the
// file must be compiled with -ffp-contract=off.
#include "plsqr_host.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum Stream : uint64_t {
  kRayEnds = 1,
  kValues = 2,
  kBlobs = 3,
  kNoise = 4,
  kRayAxis = 5,
};

inline uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}

inline uint64_t hash4(uint64_t seed, uint64_t stream, uint64_t a, uint64_t b,
                      uint64_t c = 0) {
  uint64_t h = mix64(seed + 0x9e3779b97f4a7c15ULL * (stream + 1));
  h = mix64(h ^ (a + 0x632be59bd9b4e019ULL));
  h = mix64(h ^ (b + 0x8cb92ba72f3d8dd7ULL));
  h = mix64(h ^ (c + 0x3c6ef372fe94f82bULL));
  return h;
}

// uniform in [0, 1)
inline double u01(uint64_t h) { return (double)(h >> 11) * 0x1.0p-53; }

// Natural logarithm for x > 0 from log(x) = e*ln2 + 2*atanh(s),
// s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)), atanh by its odd power series.
double det_log(double x) {
  int e;
  double m = frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
  if (m < 0.70710678118654752440) {
    m *= 2.0;
    e -= 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double p = 0.0;
  for (int k = 14; k >= 0; --k) p = p * s2 + 1.0 / (double)(2 * k + 1);
  return (double)e * 0.69314718055994530942 + 2.0 * s * p;
}

// exp(x) = 2^k * exp(r), r = x - k*ln2, exp(r) by its Taylor series.
double det_exp(double x) {
  if (x < -745.0) return 0.0;
  if (x > 709.0) return HUGE_VAL;
  const double ln2 = 0.69314718055994530942;
  const double k = floor(x / ln2 + 0.5);
  const double r = x - k * ln2;
  double p = 1.0;
  for (int j = 22; j >= 1; --j) p = 1.0 + p * r / (double)j;
  return ldexp(p, (int)k);
}

// Standard normal by Marsaglia's polar method; attempt counter in the key.
double det_normal(uint64_t seed, uint64_t stream, uint64_t a, uint64_t b) {
  for (uint64_t attempt = 0;; ++attempt) {
    const double u = 2.0 * u01(hash4(seed, stream, a, b, 2 * attempt)) - 1.0;
    const double v = 2.0 * u01(hash4(seed, stream, a, b, 2 * attempt + 1)) - 1.0;
    const double s = u * u + v * v;
    if (s >= 1.0 || s == 0.0) continue;
    return u * sqrt(-2.0 * det_log(s) / s);
  }
}

struct Ray {
  double p0[3], d[3], dd;  // segment p0 + t*d, t in [0,1]; dd = |d|^2
  int axis;
};

Ray make_ray(const plsqr_synth_params *P, int64_t r) {
  const int dims[3] = {P->nx, P->ny, P->nz};
  int axis = P->face_axis;
  if (axis < 0 || axis > 2)
    axis = (int)(hash4(P->seed, kRayAxis, (uint64_t)r, 0) % 3ULL);
  Ray ray;
  double p1[3];
  for (int c = 0; c < 3; ++c) {
    if (c == axis) {
      ray.p0[c] = 0.0;
      p1[c] = (double)dims[c];
    } else {
      ray.p0[c] = u01(hash4(P->seed, kRayEnds, (uint64_t)r, (uint64_t)c)) * dims[c];
      p1[c] = u01(hash4(P->seed, kRayEnds, (uint64_t)r, (uint64_t)(c + 3))) * dims[c];
    }
  }
  ray.dd = 0.0;
  for (int c = 0; c < 3; ++c) {
    ray.d[c] = p1[c] - ray.p0[c];
    ray.dd += ray.d[c] * ray.d[c];
  }
  ray.axis = axis;
  return ray;
}

// squared distance from point q to the segment
inline double seg_dist2(const Ray &ray, const double q[3]) {
  double w[3], t = 0.0;
  for (int c = 0; c < 3; ++c) {
    w[c] = q[c] - ray.p0[c];
    t += w[c] * ray.d[c];
  }
  t = ray.dd > 0.0 ? t / ray.dd : 0.0;
  if (t < 0.0) t = 0.0;
  if (t > 1.0) t = 1.0;
  double s = 0.0;
  for (int c = 0; c < 3; ++c) {
    const double e = q[c] - (ray.p0[c] + t * ray.d[c]);
    s += e * e;
  }
  return s;
}

// Visit the cells of one ray's tube in ascending column order.  The
// candidate box per z layer is a superset (the segment's extent over
// z +- radius, widened by the radius); each candidate is tested exactly.
template <class F>
int64_t visit_tube(const plsqr_synth_params *P, const Ray &ray, F &&f) {
  const double R = P->tube_radius, R2 = R * R;
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  int64_t count = 0;
  double zlo_seg = std::min(ray.p0[2], ray.p0[2] + ray.d[2]);
  double zhi_seg = std::max(ray.p0[2], ray.p0[2] + ray.d[2]);
  int iz0 = std::max(0, (int)floor(zlo_seg - R - 0.5));
  int iz1 = std::min(nz - 1, (int)ceil(zhi_seg + R - 0.5));
  for (int iz = iz0; iz <= iz1; ++iz) {
    const double zc = iz + 0.5;
    // parameter range of segment points within R of this layer in z
    double tlo = 0.0, thi = 1.0;
    if (ray.d[2] != 0.0) {
      double ta = (zc - R - ray.p0[2]) / ray.d[2], tb = (zc + R - ray.p0[2]) / ray.d[2];
      if (ta > tb) std::swap(ta, tb);
      tlo = std::max(0.0, ta);
      thi = std::min(1.0, tb);
      if (tlo > thi) continue;
    } else if (fabs(zc - ray.p0[2]) > R) {
      continue;
    }
    double xa = ray.p0[0] + tlo * ray.d[0], xb = ray.p0[0] + thi * ray.d[0];
    double ya = ray.p0[1] + tlo * ray.d[1], yb = ray.p0[1] + thi * ray.d[1];
    int ix0 = std::max(0, (int)floor(std::min(xa, xb) - R - 0.5));
    int ix1 = std::min(nx - 1, (int)ceil(std::max(xa, xb) + R - 0.5));
    int iy0 = std::max(0, (int)floor(std::min(ya, yb) - R - 0.5));
    int iy1 = std::min(ny - 1, (int)ceil(std::max(ya, yb) + R - 0.5));
    for (int iy = iy0; iy <= iy1; ++iy) {
      for (int ix = ix0; ix <= ix1; ++ix) {
        const double q[3] = {ix + 0.5, iy + 0.5, zc};
        if (seg_dist2(ray, q) <= R2) {
          const int64_t col = ((int64_t)iz * ny + iy) * nx + ix;
          f(count, col);
          ++count;
        }
      }
    }
  }
  return count;
}

int check_params(const plsqr_synth_params *P) {
  if (!P) return PLSQR_ERR_ARG;
  if (P->nx < 1 || P->ny < 1 || P->nz < 1 || P->n_rays < 0) return PLSQR_ERR_ARG;
  if ((int64_t)P->nx * P->ny * P->nz > INT32_MAX) return PLSQR_ERR_ARG;
  if (!(P->tube_radius >= 0.0)) return PLSQR_ERR_ARG;
  return 0;
}

}  // namespace

extern "C" {

void plsqr_synth_default_params(plsqr_synth_params *P) {
  memset(P, 0, sizeof(*P));
  P->nx = P->ny = P->nz = 32;
  P->n_rays = 2000;
  P->tube_radius = 1.5;
  P->face_axis = 2;
  P->value_scale = 1e-2;
  P->n_blobs = 8;
  P->blob_sigma = 3.0;
  P->checker_amp = 0.0;
  P->checker_period = 8;
  P->noise_frac = 0.01;
  P->damp_identity = 0.5;
  P->damp_lap = 1.0;
  P->seed = 0;
}

int plsqr_synth_kernel_counts(const plsqr_synth_params *P, int64_t *row_ptr) {
  int rc = check_params(P);
  if (rc) return rc;
  const int64_t m = P->n_rays;
  row_ptr[0] = 0;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t r = 0; r < m; ++r) {
    const Ray ray = make_ray(P, r);
    row_ptr[r + 1] = visit_tube(P, ray, [](int64_t, int64_t) {});
  }
  for (int64_t r = 0; r < m; ++r) row_ptr[r + 1] += row_ptr[r];
  return 0;
}

int plsqr_synth_kernel_fill(const plsqr_synth_params *P, const int64_t *row_ptr,
                            int32_t *col_idx, double *val) {
  int rc = check_params(P);
  if (rc) return rc;
  const int64_t m = P->n_rays;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
  for (int64_t r = 0; r < m; ++r) {
    const Ray ray = make_ray(P, r);
    const int64_t base = row_ptr[r];
    const int64_t cnt = visit_tube(P, ray, [&](int64_t k, int64_t col) {
      col_idx[base + k] = (int32_t)col;
      val[base + k] = fabs(det_normal(P->seed, kValues, (uint64_t)r, (uint64_t)col)) *
                      P->value_scale;
    });
    if (cnt != row_ptr[r + 1] - base) bad = 1;
  }
  return bad ? PLSQR_ERR_INTERNAL : 0;
}

// Rows and nonzeros of one cell's damping rows, in damping_binary.py's order:
// identity, xx, yy, zz, then (damp_cross != 0) xy, xz, yz.
struct CellRows {
  int fx, fy, fz, fxy, fxz, fyz;
  int rows() const { return 1 + fx + fy + fz + fxy + fxz + fyz; }
  int nnz() const { return 1 + 3 * (fx + fy + fz) + 4 * (fxy + fxz + fyz); }
};
static inline CellRows cell_rows(const plsqr_synth_params *P, int ix, int iy, int iz) {
  CellRows c;
  c.fx = ix < P->nx - 2;
  c.fy = iy < P->ny - 2;
  c.fz = iz < P->nz - 2;
  const int cr = P->damp_cross != 0.0;
  c.fxy = cr && c.fx && c.fy;
  c.fxz = cr && c.fx && c.fz;
  c.fyz = cr && c.fy && c.fz;
  return c;
}
static inline int n_fields(const plsqr_synth_params *P) {
  return P->n_params > 1 ? P->n_params : 1;
}

int plsqr_synth_damping_size(const plsqr_synth_params *P, int64_t *m_d, int64_t *nnz_d) {
  int rc = check_params(P);
  if (rc) return rc;
  const int64_t nx = P->nx, ny = P->ny, nz = P->nz, n = nx * ny * nz;
  const int64_t ex = std::max<int64_t>(0, nx - 2), ey = std::max<int64_t>(0, ny - 2),
                ez = std::max<int64_t>(0, nz - 2);
  const int64_t lx = ex * ny * nz, ly = nx * ey * nz, lz = nx * ny * ez;
  int64_t rows = n + lx + ly + lz, nnz = n + 3 * (lx + ly + lz);
  if (P->damp_cross != 0.0) {
    const int64_t cxy = ex * ey * nz, cxz = ex * ny * ez, cyz = nx * ey * ez;
    rows += cxy + cxz + cyz;
    nnz += 4 * (cxy + cxz + cyz);
  }
  *m_d = rows * n_fields(P);
  *nnz_d = nnz * n_fields(P);
  return 0;
}

int plsqr_synth_damping_fill(const plsqr_synth_params *P, int64_t *row_ptr,
                             int32_t *col_idx, double *val) {
  int rc = check_params(P);
  if (rc) return rc;
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  const int64_t ncell = (int64_t)nx * ny * nz;
  // first row and first nonzero of every cell of field 0, by a prefix over cells
  std::vector<int64_t> row0(ncell + 1), nz0(ncell + 1);
  row0[0] = nz0[0] = 0;
  for (int64_t c = 0; c < ncell; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((int64_t)nx * ny));
    const CellRows cr = cell_rows(P, ix, iy, iz);
    row0[c + 1] = row0[c] + cr.rows();
    nz0[c + 1] = nz0[c] + cr.nnz();
  }
  const int64_t rows_f = row0[ncell], nnz_f = nz0[ncell];
  const int64_t sx = 1, sy = nx, sz = (int64_t)nx * ny;
  row_ptr[0] = 0;
  for (int f = 0; f < n_fields(P); ++f) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < ncell; ++c) {
      const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((int64_t)nx * ny));
      const CellRows cr = cell_rows(P, ix, iy, iz);
      const int64_t col0 = c + f * ncell;
      int64_t r = row0[c] + f * rows_f, e = nz0[c] + f * nnz_f;
      auto row = [&](int k, const int64_t *off, const double *w, double weight) {
        for (int j = 0; j < k; ++j) {
          col_idx[e + j] = (int32_t)(col0 + off[j]);
          val[e + j] = w[j] * weight;
        }
        e += k;
        row_ptr[r + 1] = e;
        ++r;
      };
      const int64_t id[1] = {0};
      const double one[1] = {1.0};
      row(1, id, one, P->damp_identity);
      const double lap[3] = {1.0, -2.0, 1.0};
      const int64_t ox[3] = {0, sx, 2 * sx}, oy[3] = {0, sy, 2 * sy}, oz[3] = {0, sz, 2 * sz};
      if (cr.fx) row(3, ox, lap, P->damp_lap);
      if (cr.fy) row(3, oy, lap, P->damp_lap);
      if (cr.fz) row(3, oz, lap, P->damp_lap);
      const double crs[4] = {0.5, -0.5, -0.5, 0.5};
      const int64_t oxy[4] = {0, 2 * sx, 2 * sy, 2 * sx + 2 * sy};
      const int64_t oxz[4] = {0, 2 * sx, 2 * sz, 2 * sx + 2 * sz};
      const int64_t oyz[4] = {0, 2 * sy, 2 * sz, 2 * sy + 2 * sz};
      if (cr.fxy) row(4, oxy, crs, P->damp_cross);
      if (cr.fxz) row(4, oxz, crs, P->damp_cross);
      if (cr.fyz) row(4, oyz, crs, P->damp_cross);
    }
  }
  return 0;
}

int plsqr_synth_xtrue(const plsqr_synth_params *P, double *x) {
  int rc = check_params(P);
  if (rc) return rc;
  const int nx = P->nx, ny = P->ny, nz = P->nz;
  const int nb = P->n_blobs;
  std::vector<double> bc(3 * (size_t)std::max(nb, 1)), ba(std::max(nb, 1));
  for (int b = 0; b < nb; ++b) {
    bc[3 * b + 0] = u01(hash4(P->seed, kBlobs, (uint64_t)b, 0)) * nx;
    bc[3 * b + 1] = u01(hash4(P->seed, kBlobs, (uint64_t)b, 1)) * ny;
    bc[3 * b + 2] = u01(hash4(P->seed, kBlobs, (uint64_t)b, 2)) * nz;
    ba[b] = det_normal(P->seed, kBlobs, (uint64_t)b, 7);
  }
  const double inv2s2 = P->blob_sigma > 0 ? 1.0 / (2.0 * P->blob_sigma * P->blob_sigma) : 0.0;
  const int64_t ncell = (int64_t)nx * ny * nz;
  const int half = P->checker_period > 1 ? P->checker_period / 2 : 1;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < ncell; ++c) {
    const int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((int64_t)nx * ny));
    const double q[3] = {ix + 0.5, iy + 0.5, iz + 0.5};
    double s = 0.0;
    for (int b = 0; b < nb; ++b) {
      double d2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double e = q[k] - bc[3 * b + k];
        d2 += e * e;
      }
      s += ba[b] * det_exp(-d2 * inv2s2);
    }
    if (P->checker_amp != 0.0) {
      const int parity = (ix / half + iy / half + iz / half) & 1;
      s += parity ? -P->checker_amp : P->checker_amp;
    }
    x[c] = s;
  }
  return 0;
}

// b = kx + noise_frac * rms(kx) * N(0,1), the normals drawn from `seed`
// (b may be kx).
static void add_noise(const double *kx, int64_t m, double noise_frac, uint64_t seed, double *b) {
  double ss = 0.0;
  for (int64_t r = 0; r < m; ++r) ss += kx[r] * kx[r];
  const double rms = m > 0 ? sqrt(ss / (double)m) : 0.0;
  const double sigma = noise_frac * rms;
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < m; ++r) b[r] = kx[r] + sigma * det_normal(seed, kNoise, (uint64_t)r, 0);
}

int plsqr_synth_rhs(const plsqr_synth_params *P, const int64_t *row_ptr,
                    const int32_t *col_idx, const double *val, const double *xtrue,
                    double *b) {
  int rc = check_params(P);
  if (rc) return rc;
  const int64_t m = P->n_rays;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t r = 0; r < m; ++r) {
    double s = 0.0;
    for (int64_t e = row_ptr[r]; e < row_ptr[r + 1]; ++e) s += val[e] * xtrue[col_idx[e]];
    b[r] = s;
  }
  add_noise(b, m, P->noise_frac, P->seed, b);
  return 0;
}

int plsqr_synth_noisy(const plsqr_synth_params *P, uint64_t noise_seed, int64_t m,
                      const double *kx, double *b) {
  int rc = check_params(P);
  if (rc) return rc;
  if (m < 0 || (m > 0 && (!kx || !b))) return PLSQR_ERR_ARG;
  add_noise(kx, m, P->noise_frac, noise_seed, b);
  return 0;
}

// Compressed-sparse transpose (CSR <-> CSC) with entries of each output
// line in ascending order of the input line index.  Input lines are split in
// contiguous per-thread blocks, so the scatter keeps that order.
int plsqr_transpose(int64_t n_lines, int64_t n_out, const int64_t *ptr,
                    const int32_t *idx, const double *val, int64_t *tptr,
                    int32_t *tidx, double *tval) {
  if (n_lines < 0 || n_out < 0) return PLSQR_ERR_ARG;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  if (n_lines < 4096) nt = 1;
  std::vector<int64_t> cnt((size_t)nt * (size_t)(n_out + 1), 0);
  int bad = 0;
#pragma omp parallel num_threads(nt) reduction(| : bad)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    const int64_t lo = n_lines * t / nt, hi = n_lines * (t + 1) / nt;
    int64_t *c = &cnt[(size_t)t * (size_t)(n_out + 1)];
    for (int64_t i = lo; i < hi; ++i)
      for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        const int32_t j = idx[e];
        if (j < 0 || j >= n_out) {
          bad = 1;
          continue;
        }
        c[j]++;
      }
  }
  if (bad) return PLSQR_ERR_FORMAT;
  // tptr[j] = sum of counts; per-thread start offsets in cnt
  int64_t run = 0;
  for (int64_t j = 0; j < n_out; ++j) {
    tptr[j] = run;
    for (int t = 0; t < nt; ++t) {
      int64_t &c = cnt[(size_t)t * (size_t)(n_out + 1) + (size_t)j];
      const int64_t k = c;
      c = run;
      run += k;
    }
  }
  tptr[n_out] = run;
#pragma omp parallel num_threads(nt)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    const int64_t lo = n_lines * t / nt, hi = n_lines * (t + 1) / nt;
    int64_t *c = &cnt[(size_t)t * (size_t)(n_out + 1)];
    for (int64_t i = lo; i < hi; ++i)
      for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        const int64_t o = c[idx[e]]++;
        tidx[o] = (int32_t)i;
        if (val) tval[o] = val[e];
      }
  }
  return 0;
}

}  // extern "C"
