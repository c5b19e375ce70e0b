// Kernels of the warm-start network (a 3-D U-Net on the model grid).
//
// Activations are channels-last BF16 blocks X[voxel][C] (voxel = (z*ny +
// y)*nx + x, the column order of the model), C a multiple of 16.  A 3x3x3
// convolution and its input gradient are implicit GEMMs on the tcgen05
// tensor cores (conv_tc.cuh).  The weight gradient dW[co][tap*C + c] =
// sum_p dz[p][co] X[p + offset(tap)][c] goes through im2col (Col[voxel][tap*C
// + c], zero outside the grid), transposes and the GEMM here: C[M][N] =
// sum_k A[m][k] B[n][k] with BF16 operands (k contiguous in both) and FP32
// accumulation on mma.sync m16n8k16, split over the voxel range.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace plsqr {
namespace nn {

constexpr int kGemmThreads = 128;  // four warps, 2 x 2 over a 64 x 64 tile
constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8;

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A tile of kBM (or kBN) rows by kBK k's into shared memory, zeros outside
// [0, rows) x [k0, k1).  Each thread moves 16 bf16 (two 16-byte loads); the
// callers keep lda a multiple of 8 and k0, k1 multiples of 8.
__device__ __forceinline__ void load_tile(const __nv_bfloat16 *__restrict__ g, int64_t ld,
                                          int64_t row0, int64_t rows, int64_t k0, int64_t k1,
                                          __nv_bfloat16 (*s)[kBK + kPad]) {
  const int r = threadIdx.x >> 1, half = threadIdx.x & 1;
  const int64_t row = row0 + r;
  uint4 v[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int64_t k = k0 + half * 16 + q * 8;
    if (row < rows && k < k1)
      v[q] = *reinterpret_cast<const uint4 *>(g + row * ld + k);
    else
      v[q] = make_uint4(0, 0, 0, 0);
  }
  uint4 *d = reinterpret_cast<uint4 *>(&s[r][half * 16]);
  d[0] = v[0];
  d[1] = v[1];
}

// C[z][M][N] = sum over k in [z*kchunk, min(K, (z+1)*kchunk)) of A[m][k] B[n][k].
// Grid (ceil(M/64), ceil(N/64), splits).  kchunk a multiple of kBK.
__global__ void __launch_bounds__(kGemmThreads)
    k_gemm_nt(const __nv_bfloat16 *__restrict__ A, int64_t lda, const __nv_bfloat16 *__restrict__ B,
              int64_t ldb, float *__restrict__ C, int64_t M, int64_t N, int64_t K,
              int64_t kchunk) {
  __shared__ __align__(16) __nv_bfloat16 As[kBM][kBK + kPad];
  __shared__ __align__(16) __nv_bfloat16 Bs[kBN][kBK + kPad];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int gid = lane >> 2, tig = lane & 3;
  const int64_t m0 = (int64_t)blockIdx.x * kBM, n0 = (int64_t)blockIdx.y * kBN;
  const int64_t kb = (int64_t)blockIdx.z * kchunk;
  const int64_t ke = kb + kchunk < K ? kb + kchunk : K;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  for (int64_t k0 = kb; k0 < ke; k0 += kBK) {
    load_tile(A, lda, m0, M, k0, ke, As);
    load_tile(B, ldb, n0, N, k0, ke, Bs);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t a[2][4], b[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm * 32 + i * 16 + gid;
        a[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][kk + tig * 2]);
        a[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + tig * 2]);
        a[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][kk + tig * 2 + 8]);
        a[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][kk + tig * 2 + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn * 32 + j * 8 + gid;
        b[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + tig * 2]);
        b[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][kk + tig * 2 + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  float *Cz = C + (int64_t)blockIdx.z * M * N;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t r = m0 + wm * 32 + i * 16 + gid;
      const int64_t c = n0 + wn * 32 + j * 8 + tig * 2;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t rr = r + (q >= 2 ? 8 : 0), cc = c + (q & 1);
        if (rr < M && cc < N) Cz[rr * N + cc] = acc[i][j][q];
      }
    }
}

// out[i] = sum over z of part[z][i] (fixed order).
__global__ void k_sum_splits(const float *__restrict__ part, int64_t count, int splits,
                             float *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[(int64_t)z * count + i];
    out[i] = s;
  }
}

struct Grid3 {
  int nx, ny, nz;
  __host__ __device__ int64_t n() const { return (int64_t)nx * ny * nz; }
};

// Col[p][t*C + c] = X[p + offset(t)][c] (zero outside), t = (dz+1)*9 + (dy+1)*3 + dx+1.
__global__ void k_im2col(const __nv_bfloat16 *__restrict__ X, Grid3 g, int C,
                         __nv_bfloat16 *__restrict__ col) {
  const int64_t K = 27LL * C, total = g.n() * 27 * (C / 8);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c8 = (int)(i % (C / 8));
    const int64_t pt = i / (C / 8);
    const int t = (int)(pt % 27);
    const int64_t p = pt / 27;
    const int x = (int)(p % g.nx), y = (int)((p / g.nx) % g.ny), z = (int)(p / ((int64_t)g.nx * g.ny));
    const int xx = x + t % 3 - 1, yy = y + (t / 3) % 3 - 1, zz = z + t / 9 - 1;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny && zz >= 0 && zz < g.nz)
      v = *reinterpret_cast<const uint4 *>(X + (((int64_t)zz * g.ny + yy) * g.nx + xx) * C + c8 * 8);
    *reinterpret_cast<uint4 *>(col + p * K + (int64_t)t * C + c8 * 8) = v;
  }
}

// out[c][r] = in[r][c] for a rows x cols BF16 block (32 x 32 tiles).
__global__ void k_transpose_bf16(const __nv_bfloat16 *__restrict__ in, int64_t rows, int64_t cols,
                                 __nv_bfloat16 *__restrict__ out) {
  __shared__ __nv_bfloat16 t[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < rows && c < cols) ? in[r * cols + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t c = c0 + i, r = r0 + threadIdx.x;
    if (c < cols && r < rows) out[c * rows + r] = t[threadIdx.x][i];
  }
}

__global__ void k_f32_to_bf16(const float *__restrict__ in, int64_t n, __nv_bfloat16 *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(in[i]);
}

// dz[p][c] = bf16(d[p][c] * (act[p][c] > 0)), the gradient through the ReLU.
__global__ void k_relu_back(const float *__restrict__ d, const __nv_bfloat16 *__restrict__ act,
                            int64_t total, __nv_bfloat16 *__restrict__ dz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    dz[i] = __float2bfloat16(__bfloat162float(act[i]) > 0.f ? d[i] : 0.f);
}

// db[c] = sum over voxels of dz[p][c] (one block per channel, fixed order).
__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ dz, int64_t n, int C,
                            float *__restrict__ db) {
  __shared__ float red[256];
  const int c = blockIdx.x;
  float s = 0.f;
  for (int64_t p = threadIdx.x; p < n; p += blockDim.x) s += __bfloat162float(dz[p * C + c]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[c] = red[0];
}

// 2x2x2 average pooling of a channels-last block (fine grid g).
__global__ void k_avgpool(const __nv_bfloat16 *__restrict__ in, Grid3 g, int C,
                          __nv_bfloat16 *__restrict__ out) {
  const Grid3 h{g.nx / 2, g.ny / 2, g.nz / 2};
  const int64_t total = h.n() * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t q = i / C;
    const int x = (int)(q % h.nx), y = (int)((q / h.nx) % h.ny), z = (int)(q / ((int64_t)h.nx * h.ny));
    float s = 0.f;
    for (int d = 0; d < 8; ++d) {
      const int xx = 2 * x + (d & 1), yy = 2 * y + ((d >> 1) & 1), zz = 2 * z + (d >> 2);
      s += __bfloat162float(in[(((int64_t)zz * g.ny + yy) * g.nx + xx) * C + c]);
    }
    out[i] = __float2bfloat16(0.125f * s);
  }
}

// The gradient of the pooling: dIn[fine p][c] = dOut[coarse p/2][c] / 8
// (accumulated into dIn when acc != 0).
__global__ void k_avgpool_back(const float *__restrict__ dout, Grid3 g, int C, int acc,
                               float *__restrict__ din) {
  const int64_t total = g.n() * C;
  const Grid3 h{g.nx / 2, g.ny / 2, g.nz / 2};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t p = i / C;
    const int x = (int)(p % g.nx), y = (int)((p / g.nx) % g.ny), z = (int)(p / ((int64_t)g.nx * g.ny));
    const float v = 0.125f * dout[(((int64_t)(z / 2) * h.ny + y / 2) * h.nx + x / 2) * C + c];
    din[i] = acc ? din[i] + v : v;
  }
}

// Nearest upsampling x2 into channels [c0, c0 + C) of a Ct-channel block on
// the fine grid g; the other channels are written by k_copy_channels.
__global__ void k_upsample(const __nv_bfloat16 *__restrict__ in, Grid3 g, int C, int Ct, int c0,
                           __nv_bfloat16 *__restrict__ out) {
  const Grid3 h{g.nx / 2, g.ny / 2, g.nz / 2};
  const int64_t total = g.n() * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t p = i / C;
    const int x = (int)(p % g.nx), y = (int)((p / g.nx) % g.ny), z = (int)(p / ((int64_t)g.nx * g.ny));
    out[p * Ct + c0 + c] = in[(((int64_t)(z / 2) * h.ny + y / 2) * h.nx + x / 2) * C + c];
  }
}

// The gradient of the upsampling: dIn[coarse q][c] = sum of the 8 children's
// dOut[p][c0 + c] (Ct-channel block).
__global__ void k_upsample_back(const float *__restrict__ dout, Grid3 g, int C, int Ct, int c0,
                                float *__restrict__ din) {
  const Grid3 h{g.nx / 2, g.ny / 2, g.nz / 2};
  const int64_t total = h.n() * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const int64_t q = i / C;
    const int x = (int)(q % h.nx), y = (int)((q / h.nx) % h.ny), z = (int)(q / ((int64_t)h.nx * h.ny));
    float s = 0.f;
    for (int d = 0; d < 8; ++d) {
      const int xx = 2 * x + (d & 1), yy = 2 * y + ((d >> 1) & 1), zz = 2 * z + (d >> 2);
      s += dout[(((int64_t)zz * g.ny + yy) * g.nx + xx) * Ct + c0 + c];
    }
    din[i] = s;
  }
}

// out[p][c0 + c] = in[p][c] (a C-channel block into channels of a Ct block).
__global__ void k_copy_channels(const __nv_bfloat16 *__restrict__ in, int64_t n, int C, int Ct,
                                int c0, __nv_bfloat16 *__restrict__ out) {
  const int64_t total = n * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    out[(i / C) * Ct + c0 + i % C] = in[i];
}

// d[p][c] (+)= src[p][c0 + c] (the gradient of a channel copy).
__global__ void k_take_channels(const float *__restrict__ src, int64_t n, int C, int Ct, int c0,
                                int acc, float *__restrict__ d) {
  const int64_t total = n * C;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = src[(i / C) * Ct + c0 + i % C];
    d[i] = acc ? d[i] + v : v;
  }
}

// The input volume (scaled by 1/s) into channel 0 of a 16-channel block.
__global__ void k_input16(const float *__restrict__ in, int64_t n, float inv_s,
                          __nv_bfloat16 *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * 16;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(i % 16 == 0 ? in[i / 16] * inv_s : 0.f);
}

// y[p] = s * (b + sum_c w[c] act[p][c]): the 1x1 output convolution (FP32).
__global__ void k_head(const __nv_bfloat16 *__restrict__ act, int64_t n, int C,
                       const float *__restrict__ w, float b, float s, float *__restrict__ y) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    float t = b;
    for (int c = 0; c < C; ++c) t = fmaf(w[c], __bfloat162float(act[p * C + c]), t);
    y[p] = s * t;
  }
}

// Squared-error loss of the head, in the network's scaled units:
// e[p] = y[p]/s - target[p]/s; d[p][c] = (2/n) e[p] w[c]; per-block partials
// of sum e^2, of dW[c] = (2/n) sum e[p] act[p][c] and of db = (2/n) sum e[p].
__global__ void k_head_back(const __nv_bfloat16 *__restrict__ act, int64_t n, int C,
                            const float *__restrict__ w, const float *__restrict__ y,
                            const float *__restrict__ target, float inv_s, float *__restrict__ d,
                            float *__restrict__ parts /* [grid][C + 2] */) {
  __shared__ float red[256];
  const float k2n = 2.f / (float)n;
  float acc[17];
  for (int c = 0; c < C + 1; ++c) acc[c] = 0.f;
  float se = 0.f;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    const float e = (y[p] - target[p]) * inv_s;
    se = fmaf(e, e, se);
    for (int c = 0; c < C; ++c) {
      d[p * C + c] = k2n * e * w[c];
      acc[c] = fmaf(k2n * e, __bfloat162float(act[p * C + c]), acc[c]);
    }
    acc[C] += k2n * e;
  }
  for (int q = 0; q < C + 2; ++q) {
    red[threadIdx.x] = q < C + 1 ? acc[q] : se;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) parts[blockIdx.x * (C + 2) + q] = red[0];
    __syncthreads();
  }
}

// Adam on FP32 master weights, with their BF16 copy (may be null).
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16 *__restrict__ wb) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

}  // namespace nn
}  // namespace plsqr
