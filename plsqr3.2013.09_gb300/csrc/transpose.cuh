// Device transpose of a by-column matrix into a by-row matrix whose rows
// list their entries in ascending column order (the order in which the
// reference's column scatter, CPUSpMV.c:171-179, adds them).
//
// Deterministic counting sort: the columns are cut into `nb` contiguous
// chunks, one block per chunk.  cnt[b][r] counts chunk b's entries of row r;
// an exclusive scan over (r, b) in row-major order turns the counts into
// write cursors; each block then scatters its columns one after another, so
// that within a row the entries land in ascending column order.
#pragma once

#include <stdint.h>

namespace plsqr {

static __global__ void k_tr_count(const int64_t *__restrict__ cp, const int32_t *__restrict__ ri,
                           int n, int nb, int m, int32_t *__restrict__ cnt) {
  const int b = blockIdx.x;
  const int c0 = (int)((int64_t)n * b / nb), c1 = (int)((int64_t)n * (b + 1) / nb);
  int32_t *row = cnt + (int64_t)b * m;
  for (int64_t e = cp[c0] + threadIdx.x; e < cp[c1]; e += blockDim.x) atomicAdd(&row[ri[e]], 1);
}

// rowcnt[r] = sum_b cnt[b][r]
static __global__ void k_tr_rowtot(const int32_t *__restrict__ cnt, int nb, int m,
                            int64_t *__restrict__ rowcnt) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
    int64_t s = 0;
    for (int b = 0; b < nb; ++b) s += cnt[(int64_t)b * m + r];
    rowcnt[r] = s;
  }
}

// Exclusive scan of in[0..m) into out[0..m], one block (setup only).
static __global__ void k_scan_one_block(const int64_t *__restrict__ in, int m, int64_t *__restrict__ out) {
  __shared__ int64_t part[1024];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < m; base += 1024) {
    const int i = base + threadIdx.x;
    int64_t v = i < m ? in[i] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int64_t t = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
      __syncthreads();
      part[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < m) out[i] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[m] = carry;
}

// cnt[b][r] <- rp[r] + sum_{b' < b} cnt[b'][r]
static __global__ void k_tr_cursor(int32_t *__restrict__ cnt, int nb, int m,
                            const int64_t *__restrict__ rp, int64_t *__restrict__ cur) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
    int64_t run = rp[r];
    for (int b = 0; b < nb; ++b) {
      const int64_t k = cnt[(int64_t)b * m + r];
      cur[(int64_t)b * m + r] = run;
      run += k;
    }
  }
}

static __global__ void k_tr_scatter(const int64_t *__restrict__ cp, const int32_t *__restrict__ ri,
                             const double *__restrict__ cv, int n, int nb, int m,
                             unsigned long long *__restrict__ cur, int32_t *__restrict__ ci,
                             double *__restrict__ v) {
  const int b = blockIdx.x;
  const int c0 = (int)((int64_t)n * b / nb), c1 = (int)((int64_t)n * (b + 1) / nb);
  unsigned long long *row = cur + (int64_t)b * m;
  for (int c = c0; c < c1; ++c) {
    for (int64_t e = cp[c] + threadIdx.x; e < cp[c + 1]; e += blockDim.x) {
      const int64_t o = (int64_t)atomicAdd(&row[ri[e]], 1ULL);
      ci[o] = c;
      v[o] = cv[e];
    }
    __syncthreads();  // column c is placed before column c+1
  }
}

}  // namespace plsqr
