// plsqr_aprod1_nrm2_noalloc: the kernel-row product y <- y + A x with the
// 2-norm of the result, for callers that cannot allocate device memory.
//
// Who needs it: code whose device memory is owned by another allocator or a
// fixed budget (a framework's caching allocator, an MPI rank that sized its
// buffers up front, the way the reference's driver allocates everything
// before the solve), and real-time callers that cannot block on the driver's
// allocator (cudaMalloc and cudaFree may synchronise the device).  They pass
// every input and output; the only extra memory the product needs, one
// partial sum of squares per block, lives in a fixed array of this library's
// module.
//
// The scratch: `g_noalloc_parts`, kNoAllocParts doubles (128 KB), a static
// __device__ array.  Every GPU that loads the library holds it until the
// process exits.  Host code cannot use the array's name as a device address,
// so the first call on a device, with that device current, looks the address
// up with cudaGetSymbolAddress and keeps it; make that first call before any
// stream capture (the lookup may initialise the module): a first call on a
// stream that is being captured is refused with PLSQR_ERR_STATE before it
// touches the runtime.  The kept address belongs to the device's current
// context: after cudaDeviceReset in the same process the module is loaded
// again and the address may change, so calls after a reset are not
// supported.  All calls share the array and every call overwrites the
// entries it uses, so nothing needs to start at zero, but calls that overlap
// on the GPU (different streams, no ordering between them) race on it.
#include <cuda_runtime.h>

#include <stdint.h>

#include <mutex>

#include "kernels_fp64.cuh"
#include "plsqr_gpu.h"

using namespace plsqr;

namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerWarp = 8;
constexpr int kRowsPerBlock = kRowsPerWarp * (kThreads / 32);  // 64
constexpr int kNoAllocParts = PLSQR_NOALLOC_MAX_ROWS / kRowsPerBlock;  // 16,384
static_assert(PLSQR_NOALLOC_MAX_ROWS % kRowsPerBlock == 0, "row limit must fill whole blocks");
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_parts[kNoAllocParts];

std::mutex g_mu;
double *g_parts_addr[kMaxDevices] = {nullptr};

// Warp w of block b owns rows [(b*8 + w)*8, +8): the rows of k_aprod1 with a
// fixed row-to-warp map (a balanced map would need a device array).
__global__ void __launch_bounds__(kThreads)
    k_noalloc_rows(int n_rows, const int64_t *__restrict__ ptr, const int32_t *__restrict__ idx,
                   const double *__restrict__ val, const double *__restrict__ x,
                   double *__restrict__ y, double *__restrict__ parts) {
  __shared__ double smem[kThreads / 32];
  const int lane = threadIdx.x & 31;
  const int r0 = (blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5)) * kRowsPerWarp;
  double sq = 0.0;
  for (int r = r0; r < min(r0 + kRowsPerWarp, n_rows); ++r) {
    const double t = warp_sum(lane_dot<double, 2>(idx, val, x, ptr[r], ptr[r + 1], lane));
    if (lane == 0) {
      const double v = y[r] + t;
      y[r] = v;
      sq = fma(v, v, sq);
    }
  }
  const double b = block_sum<kThreads>(sq, smem);
  if (threadIdx.x == 0) parts[blockIdx.x] = b;
}

// nrm2 = sqrt(sum of the blocks' partials), summed in block order.
__global__ void __launch_bounds__(kThreads)
    k_noalloc_finish(const double *__restrict__ parts, int n_parts, double *__restrict__ nrm2) {
  __shared__ double smem[kThreads / 32];
  const double s = sum_parts<kThreads>(parts, n_parts, smem);
  if (threadIdx.x == 0) *nrm2 = sqrt(s);
}

}  // namespace

extern "C" int plsqr_aprod1_nrm2_noalloc(int32_t n_rows, const int64_t *row_ptr,
                                         const int32_t *col_idx, const double *val,
                                         const double *x, double *y, double *nrm2,
                                         void *stream) {
  if (n_rows < 0 || n_rows > PLSQR_NOALLOC_MAX_ROWS) return PLSQR_ERR_ARG;
  if (!row_ptr || !nrm2 || (n_rows > 0 && (!y || !x || !col_idx || !val))) return PLSQR_ERR_ARG;
  // the product reads indices and values with 16-byte loads
  if (((uintptr_t)col_idx | (uintptr_t)val) % 16 != 0) return PLSQR_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return PLSQR_ERR_NODEV;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double *parts = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_parts_addr[dev]) {
      // the set-up call must not run while the stream is being captured
      cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        cudaGetLastError();
        return PLSQR_ERR_CUDA;
      }
      if (cap != cudaStreamCaptureStatusNone) return PLSQR_ERR_STATE;
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_parts) != cudaSuccess || !p) {
        cudaGetLastError();
        return PLSQR_ERR_CUDA;
      }
      g_parts_addr[dev] = (double *)p;
    }
    parts = g_parts_addr[dev];
  }
  const int blocks = n_rows > 0 ? (n_rows + kRowsPerBlock - 1) / kRowsPerBlock : 0;
  if (blocks > 0)
    k_noalloc_rows<<<blocks, kThreads, 0, s>>>(n_rows, row_ptr, col_idx, val, x, y, parts);
  k_noalloc_finish<<<1, kThreads, 0, s>>>(parts, blocks, nrm2);
  return cudaGetLastError() == cudaSuccess ? PLSQR_OK : PLSQR_ERR_CUDA;
}
