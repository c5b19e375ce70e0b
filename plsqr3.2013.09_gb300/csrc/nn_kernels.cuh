// Kernels of the warm-start network (a 3-D U-Net on the model grid).
//
// Activations are channels-last BF16 blocks X[voxel][C] (voxel = (z*ny +
// y)*nx + x, the column order of the model), C a multiple of 16.  A 3x3x3
// convolution and its input gradient are implicit GEMMs on the tcgen05
// tensor cores (conv_tc.cuh).  The weight gradient dW[co][tap*C + c] =
// sum_p dz[p][co] X[p + offset(tap)][c] is a tcgen05 GEMM (conv_tc.cuh) on
// the transposed im2col block written here (k_im2col_t) and dz transposed.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace plsqr {
namespace nn {

struct Grid3 {
  int nx, ny, nz;
  __host__ __device__ int64_t n() const { return (int64_t)nx * ny * nz; }
};

// Colt[t*C + c][p] = X[p + offset(t)][c] (zero outside the grid): the
// transposed im2col block of the weight gradient, written directly.  A
// thread takes two neighbouring voxels and one tap, reads their channel rows
// in 16-byte pieces and writes bf16 pairs down the C rows, so that a warp
// writes 128 contiguous bytes of each row.  n must be even.
__global__ void k_im2col_t(const __nv_bfloat16 *__restrict__ X, Grid3 g, int C,
                           __nv_bfloat16 *__restrict__ colt) {
  const int64_t n = g.n(), half = n / 2, total = 27 * half;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(i / half);
    const int64_t p = 2 * (i % half);
    const int ox = t % 3 - 1, oy = (t / 3) % 3 - 1, oz = t / 9 - 1;
    const __nv_bfloat16 *src[2];
    for (int v = 0; v < 2; ++v) {
      const int64_t q = p + v;
      const int x = (int)(q % g.nx), y = (int)((q / g.nx) % g.ny), z = (int)(q / ((int64_t)g.nx * g.ny));
      const int xx = x + ox, yy = y + oy, zz = z + oz;
      src[v] = (xx >= 0 && xx < g.nx && yy >= 0 && yy < g.ny && zz >= 0 && zz < g.nz)
                   ? X + (((int64_t)zz * g.ny + yy) * g.nx + xx) * C
                   : nullptr;
    }
    __nv_bfloat16 *dst = colt + (int64_t)t * C * n + p;
    for (int c8 = 0; c8 < C; c8 += 8) {
      uint4 a = make_uint4(0, 0, 0, 0), b = make_uint4(0, 0, 0, 0);
      if (src[0]) a = *reinterpret_cast<const uint4 *>(src[0] + c8);
      if (src[1]) b = *reinterpret_cast<const uint4 *>(src[1] + c8);
      const __nv_bfloat16 *ea = reinterpret_cast<const __nv_bfloat16 *>(&a);
      const __nv_bfloat16 *eb = reinterpret_cast<const __nv_bfloat16 *>(&b);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        __nv_bfloat162 pr;
        pr.x = ea[c];
        pr.y = eb[c];
        *reinterpret_cast<__nv_bfloat162 *>(dst + (int64_t)(c8 + c) * n) = pr;
      }
    }
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

// db[c] = sum over voxels of dz[p][c], in two fixed-order steps: each block
// of kBiasThreads threads reads a grid-strided share of dz in storage order
// (a thread keeps one channel, as kBiasThreads * gridDim is a multiple of
// C) and writes its per-channel sums to parts[block][C]; k_bias_grad_final
// (one warp per channel) adds the blocks' sums in a fixed order.
constexpr int kBiasThreads = 192;  // a multiple of 16, 32, 48, 64 and 96

__global__ void __launch_bounds__(kBiasThreads)
    k_bias_grad(const __nv_bfloat16 *__restrict__ dz, int64_t n, int C, float *__restrict__ parts) {
  __shared__ float red[kBiasThreads];
  const int64_t total = n * C, stride = (int64_t)gridDim.x * kBiasThreads;
  float s = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)kBiasThreads + threadIdx.x; i < total; i += stride)
    s += __bfloat162float(dz[i]);
  red[threadIdx.x] = s;
  __syncthreads();
  // thread c < C sums the threads of channel c (c, c + C, ...) in order
  if ((int)threadIdx.x < C) {
    float t = 0.f;
    for (int k = threadIdx.x; k < kBiasThreads; k += C) t += red[k];
    parts[(int64_t)blockIdx.x * C + threadIdx.x] = t;
  }
}

__global__ void k_bias_grad_final(const float *__restrict__ parts, int blocks, int C,
                                  float *__restrict__ db) {
  const int c = blockIdx.x, lane = threadIdx.x;
  float t = 0.f;
  for (int b = lane; b < blocks; b += 32) t += parts[(int64_t)b * C + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) db[c] = t;
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

// Per-block sums of squares of the input volume (FP64, fixed order), for its
// root mean square.
__global__ void k_sumsq_in(const float *__restrict__ in, int64_t n, double *__restrict__ parts) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += (double)in[i] * in[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = red[0];
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
