// 3x3x3 convolution of a channels-last BF16 block as an implicit GEMM on the
// fifth-generation tensor cores: tcgen05.mma (kind::f16, BF16 operands, FP32
// accumulator in tensor memory), no im2col matrix in HBM.
//
// One CTA owns 128 consecutive voxels (the MMA's M).  For each of the 27
// taps t it gathers the neighbours' channel rows A_t[r][k] = X[p0 + r +
// offset(t)][k] (zero outside the grid) and the weight block B_t[o][k] into
// shared memory with cp.async, and one elected thread issues CI/16 MMAs of
// 128 x CO x 16 that accumulate into the CTA's TMEM columns.  Three stages
// keep the gathers of later taps in flight while the tensor core works; a
// stage is refilled only after the MMAs that read it have committed to its
// mbarrier.  The epilogue reads the accumulator back with tcgen05.ld (warp w
// owns TMEM lanes 32w..32w+31, i.e. voxels p0 + 32w + lane).
//
// The same kernel computes the input gradient of a convolution: the
// gathered block is dz (CO_layer channels), the taps are mirrored
// (offset(26 - t) = -offset(t)) and B_t[ci][co] is read from the transposed
// weights, so dX[p][ci] = sum_t sum_co dz[p - offset(t)][co] W[co][t][ci].
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, core (g, j) of a tile at byte
// (g * CI/8 + j) * 128, so the descriptor's leading byte offset (between
// core matrices along K) is 128 and its stride byte offset (between 8-row
// groups) is CI/8 * 128.
//
// Every wait on an mbarrier is bounded (one second of the global timer); a
// wait that runs out sets *err, skips the remaining MMAs and the epilogue,
// and the CTA still frees its tensor memory.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "nn_kernels.cuh"

namespace plsqr {
namespace nn {

constexpr int kTcRows = 128;    // voxels per CTA (MMA M)
constexpr int kTcThreads = 128; // four warps
constexpr int kTcStages = 3;
constexpr unsigned long long kTcWaitNs = 1000000000ull;

struct ConvTcArgs {
  const __nv_bfloat16 *x;  // gathered block [n][CI]
  const __nv_bfloat16 *w;  // B_t[o][k] = w[tap(t) * tap_stride + o * ldw + k]
  int64_t ldw, tap_stride;
  int flip;                // tap(t) = flip ? 26 - t : t; neighbour offset(t) either way
  const float *bias;       // [CO] added in the epilogue, or null
  int relu;
  __nv_bfloat16 *out_bf16; // [n][CO], or null
  float *out_f32;          // [n][CO], or null
  Grid3 g;
  unsigned int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long tc_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Shared-memory matrix descriptor: start, leading and stride byte offsets
// (all >> 4), the fixed 0b001 at bits 46-48, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// BF16 A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase of `parity` to complete; false when the wait ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = tc_clock();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_try(bar, parity)) return true;
    if (tc_clock() - t0 > kTcWaitNs) return false;
  }
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
               "r"(bytes)
               : "memory");
}

// Columns of tensor memory for a CO-wide FP32 accumulator (a power of two >= 32).
__host__ __device__ constexpr uint32_t tc_cols(int co) {
  return co <= 32 ? 32u : co <= 64 ? 64u : co <= 128 ? 128u : 256u;
}

template <int CI, int CO>
struct ConvTcShape {
  static_assert(CI % 16 == 0 && CO % 16 == 0 && CO >= 16 && CO <= 256, "channel counts");
  static constexpr int kCoresK = CI / 8;
  static constexpr int kABytes = kTcRows * CI * 2;
  static constexpr int kBBytes = CO * CI * 2;
  static constexpr int kStageBytes = kABytes + kBBytes;
  // stages, then the stage mbarriers and the TMEM address slot; +128 for
  // aligning the dynamic block
  static constexpr int kSmemBytes = kTcStages * kStageBytes + 64 + 128;
};

template <int CI, int CO>
__global__ void __launch_bounds__(kTcThreads) k_conv_tc(ConvTcArgs a) {
  using S = ConvTcShape<CI, CO>;
  extern __shared__ uint8_t tc_smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 127) & ~(uintptr_t)127);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTcStages * S::kStageBytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + kTcStages);
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t n = a.g.n();
  const int64_t p0 = (int64_t)blockIdx.x * kTcRows;
  constexpr uint32_t kCols = tc_cols(CO);
  constexpr uint32_t kIdesc = tc_idesc(kTcRows, CO);
  constexpr uint32_t kSbo = S::kCoresK * 128;

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < kTcStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  // this thread's gather rows: task q = it * 128 + tid, row q / (CI/8),
  // chunk q % (CI/8); the voxel coordinates of each row, computed once
  constexpr int kTasksA = kTcRows * S::kCoresK / kTcThreads;  // = CI/8
  int vx[kTasksA], vy[kTasksA], vz[kTasksA];
#pragma unroll
  for (int it = 0; it < kTasksA; ++it) {
    const int q = it * kTcThreads + tid;
    const int64_t p = p0 + q / S::kCoresK;
    if (p < n) {
      vx[it] = (int)(p % a.g.nx);
      vy[it] = (int)((p / a.g.nx) % a.g.ny);
      vz[it] = (int)(p / ((int64_t)a.g.nx * a.g.ny));
    } else {
      vx[it] = -4;  // outside for every tap
      vy[it] = 0;
      vz[it] = 0;
    }
  }

  auto gather = [&](int t, int s) {
    uint8_t *A = smem + s * S::kStageBytes;
    uint8_t *B = A + S::kABytes;
    const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
#pragma unroll
    for (int it = 0; it < kTasksA; ++it) {
      const int q = it * kTcThreads + tid;
      const int r = q / S::kCoresK, j = q % S::kCoresK;
      const int xx = vx[it] + dx, yy = vy[it] + dy, zz = vz[it] + dz;
      const bool in = xx >= 0 && xx < a.g.nx && yy >= 0 && yy < a.g.ny && zz >= 0 && zz < a.g.nz;
      const __nv_bfloat16 *src =
          in ? a.x + (((int64_t)zz * a.g.ny + yy) * a.g.nx + xx) * CI + j * 8 : a.x;
      const uint32_t dst = smem_u32(A + ((r >> 3) * S::kCoresK + j) * 128 + (r & 7) * 16);
      cp_async16(dst, src, in ? 16u : 0u);
    }
    const int tap = a.flip ? 26 - t : t;
    const __nv_bfloat16 *wt = a.w + (int64_t)tap * a.tap_stride;
    for (int q = tid; q < CO * S::kCoresK; q += kTcThreads) {
      const int o = q / S::kCoresK, j = q % S::kCoresK;
      const uint32_t dst = smem_u32(B + ((o >> 3) * S::kCoresK + j) * 128 + (o & 7) * 16);
      cp_async16(dst, wt + (int64_t)o * a.ldw + j * 8, 16u);
    }
  };

  bool ok = true;  // this thread's waits all completed
  auto wait_mma = [&](int t) {  // the MMAs of tap t have read their stage
    if (!ok) return;
    if (!mbar_wait(smem_u32(&bars[t % kTcStages]), (uint32_t)((t / kTcStages) & 1))) {
      ok = false;
      abort_flag = 1;
      atomicExch(a.err, 1u);
    }
  };

#pragma unroll 1
  for (int t = 0; t < kTcStages - 1; ++t) {
    gather(t, t);
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
#pragma unroll 1
  for (int t = 0; t < 27; ++t) {
    const int tn = t + kTcStages - 1;
    if (tn < 27) {
      if (t >= 1) wait_mma(t - 1);  // stage tn % S last held tap t - 1
      gather(tn, tn % kTcStages);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group %0;" ::"n"(kTcStages - 1) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0 && !abort_flag) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int s = t % kTcStages;
      const uint32_t A = smem_u32(smem + s * S::kStageBytes);
      const uint32_t B = A + S::kABytes;
#pragma unroll
      for (int kk = 0; kk < CI / 16; ++kk)
        tc_mma(tmem, tc_desc(A + kk * 256, 128, kSbo), tc_desc(B + kk * 256, 128, kSbo), kIdesc,
               (t > 0 || kk > 0) ? 1u : 0u);
      tc_commit(smem_u32(&bars[s]));
    }
  }
  // the last commit follows every MMA of the CTA
  wait_mma(26);
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (!abort_flag) {
    const int64_t p = p0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < CO; c0 += 16) {
      uint32_t v[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
          "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(trow + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      float f[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        f[i] = __uint_as_float(v[i]);
        if (a.bias) f[i] += a.bias[c0 + i];
        if (a.relu) f[i] = fmaxf(f[i], 0.f);
      }
      if (p < n) {
        if (a.out_bf16) {
          __align__(16) __nv_bfloat16 h[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16(f[i]);
          uint4 *d = reinterpret_cast<uint4 *>(a.out_bf16 + p * CO + c0);
          d[0] = reinterpret_cast<const uint4 *>(h)[0];
          d[1] = reinterpret_cast<const uint4 *>(h)[1];
        } else {
          float4 *d = reinterpret_cast<float4 *>(a.out_f32 + p * CO + c0);
#pragma unroll
          for (int i = 0; i < 4; ++i) d[i] = make_float4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols)
                 : "memory");
}

}  // namespace nn
}  // namespace plsqr
