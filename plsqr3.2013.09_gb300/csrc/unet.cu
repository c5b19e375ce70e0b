// The warm-start network: a 3-D U-Net (3 levels, 16/32/64 channels) from the
// column-norm-scaled back-projection A^T b to a starting solution x0 on the
// model grid, trained on (A^T b, x_LSQR) pairs that this library's solvers
// produce.  Weights are FP32 masters with BF16 copies.  Every contraction
// runs on the tcgen05 tensor cores (BF16 operands, FP32 accumulation in
// tensor memory, conv_tc.cuh): the forward convolutions and their input
// gradients as implicit GEMMs, the weight gradients as a split-K GEMM on the
// transposed im2col block (nn_kernels.cuh).  One volume per step, Adam.
//
//   x16 = input / s (channel 0 of 16)                          level 0
//   e1 = relu(conv(relu(conv(x16, 16)), 16))                   level 0
//   e2 = relu(conv(relu(conv(pool(e1), 32)), 32))              level 1
//   b  = relu(conv(relu(conv(pool(e2), 64)), 64))              level 2
//   d2 = relu(conv(relu(conv([up(b), e2], 32)), 32))           level 1
//   d1 = relu(conv(relu(conv([up(d2), e1], 16)), 16))          level 0
//   x0 = s * (w . d1 + c)                                      1x1 head
//
// s is the input's root mean square, so the map is scale-equivariant.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <memory>
#include <vector>

#include "conv_tc.cuh"
#include "nn_kernels.cuh"
#include "plsqr_gpu.h"

using namespace plsqr::nn;
typedef __nv_bfloat16 bf16;

namespace {

constexpr int kT = 256;  // threads of the elementwise kernels
constexpr int kBiasBlocks = 304;  // blocks of the bias-gradient reduction

int grid_for(int64_t work) {
  int64_t g = (work + kT - 1) / kT;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g < 1 ? 1 : g);
}

struct Buf {
  void *p = nullptr;
  size_t bytes = 0;
};

struct Conv {
  int cin = 0, cout = 0;
  Grid3 g{0, 0, 0};
  int64_t K() const { return 27LL * cin; }
  float *w = nullptr, *b = nullptr;    // FP32 masters [cout][K], [cout]
  bf16 *wb = nullptr, *wbt = nullptr;  // BF16 copy [cout][K] and its transpose [K][cout]
  float *gw = nullptr, *gb = nullptr;
  float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
};

}  // namespace

struct plsqr_unet {
  int device = 0;
  cudaStream_t stream = nullptr;
  Grid3 g0{0, 0, 0}, g1{0, 0, 0}, g2{0, 0, 0};
  std::vector<void *> allocs;
  Conv e1a, e1b, e2a, e2b, ba, bb, d2a, d2b, d1a, d1b;
  float *hw = nullptr, *hm = nullptr, *hv = nullptr, *hg = nullptr;  // head: 16 weights + bias
  // activations (BF16, channels last)
  bf16 *x16, *a_e1a, *a_e1b, *a_p1, *a_e2a, *a_e2b, *a_p2, *a_ba, *a_bb, *a_c2, *a_d2a, *a_d2b,
      *a_c1, *a_d1a, *a_d1b;
  // gradients (FP32)
  float *g_e1a, *g_e1b, *g_p1, *g_e2a, *g_e2b, *g_p2, *g_ba, *g_bb, *g_c2, *g_d2a, *g_d2b, *g_c1,
      *g_d1a, *g_d1b;
  // scratch
  bf16 *colt = nullptr, *dz = nullptr, *dzt = nullptr;
  float *part = nullptr, *in = nullptr, *out = nullptr, *target = nullptr, *hparts = nullptr,
        *bparts = nullptr;
  unsigned int *dflag = nullptr;  // set by a tensor-core kernel whose wait ran out
  double *sparts = nullptr;       // per-block sums of squares of the input
  cudaEvent_t ev = nullptr;       // orders the device-array calls with the caller's stream
  int64_t part_cap = 0;           // floats of part
  int64_t step = 0;
  char err[256] = {0};
};

namespace {

#define UK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      snprintf(net->err, sizeof net->err, "%s: %s", #call, cudaGetErrorString(e_));        \
      return PLSQR_ERR_CUDA;                                                              \
    }                                                                                     \
  } while (0)

template <class T>
int nalloc(plsqr_unet *net, T **p, int64_t count) {
  void *q = nullptr;
  UK(cudaMalloc(&q, (size_t)(count > 0 ? count : 1) * sizeof(T)));
  UK(cudaMemset(q, 0, (size_t)(count > 0 ? count : 1) * sizeof(T)));
  net->allocs.push_back(q);
  *p = (T *)q;
  return PLSQR_OK;
}

uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

// Deterministic normal deviates (Box-Muller on a counter hash).
double det_normal(uint64_t seed, uint64_t i) {
  const double u1 = ((mix64(seed * 2654435761ULL + 2 * i) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = ((mix64(seed * 2654435761ULL + 2 * i + 1) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// He initialisation (std sqrt(2 / fan_in), fan_in = 27 * real input channels).
int init_conv(plsqr_unet *net, Conv &L, int cin, int cout, Grid3 g, int fan_c, uint64_t seed) {
  L.cin = cin;
  L.cout = cout;
  L.g = g;
  const int64_t nw = (int64_t)cout * L.K();
  int rc;
  if ((rc = nalloc(net, &L.w, nw)) || (rc = nalloc(net, &L.b, cout)) ||
      (rc = nalloc(net, &L.wb, nw)) || (rc = nalloc(net, &L.wbt, nw)) ||
      (rc = nalloc(net, &L.gw, nw)) || (rc = nalloc(net, &L.gb, cout)) ||
      (rc = nalloc(net, &L.mw, nw)) || (rc = nalloc(net, &L.vw, nw)) ||
      (rc = nalloc(net, &L.mb, cout)) || (rc = nalloc(net, &L.vb, cout)))
    return rc;
  std::vector<float> h((size_t)nw);
  const double sd = sqrt(2.0 / (27.0 * fan_c));
  for (int64_t i = 0; i < nw; ++i) h[(size_t)i] = (float)(sd * det_normal(seed, (uint64_t)i));
  UK(cudaMemcpy(L.w, h.data(), sizeof(float) * nw, cudaMemcpyHostToDevice));
  k_f32_to_bf16<<<grid_for(nw), kT, 0, net->stream>>>(L.w, nw, L.wb);
  UK(cudaGetLastError());
  return PLSQR_OK;
}

// The halo-staged kernel, with all 27 weight taps resident where they fit
// in one CTA's shared memory beside the halo, else one plane's taps at a time.
template <int CI, int CO, bool kAllW>
int conv_tc_launch(plsqr_unet *net, const ConvTcArgs &a) {
  // at most 512 / cols CTAs per SM (of 228 KB of shared memory), so that
  // every resident CTA's tensor-memory allocation succeeds at once
  constexpr uint32_t cols = tc_cols(CO);
  constexpr int floor_bytes = cols >= 128 ? 58 * 1024 : cols >= 64 ? 30 * 1024 : 0;
  constexpr int need = ConvTc2Shape<CI, CO, kAllW>::kSmemBytes;
  constexpr int bytes = need > floor_bytes ? need : floor_bytes;
  static_assert(bytes <= 227 * 1024, "shared memory of one CTA");
  UK(cudaFuncSetAttribute(k_conv_tc2<CI, CO, kAllW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          bytes));
  const int64_t blocks = (int64_t)((a.g.nx + 7) / 8) * ((a.g.ny + 15) / 16) * a.g.nz;
  k_conv_tc2<CI, CO, kAllW><<<(unsigned)blocks, kTcThreads, bytes, net->stream>>>(a);
  UK(cudaGetLastError());
  return PLSQR_OK;
}

template <int CI, int CO>
int conv_tc_run(plsqr_unet *net, const ConvTcArgs &a) {
  if constexpr (ConvTc2Shape<CI, CO, true>::kSmemBytes <= 227 * 1024)
    return conv_tc_launch<CI, CO, true>(net, a);
  else
    return conv_tc_launch<CI, CO, false>(net, a);
}

// The channel pairs of the network's layers (forward: cin -> cout; input
// gradient: cout -> cin).
int conv_tc(plsqr_unet *net, int ci, int co, const ConvTcArgs &a) {
#define PLSQR_TC_PAIR(I, O) \
  if (ci == I && co == O) return conv_tc_run<I, O>(net, a);
  PLSQR_TC_PAIR(16, 16)
  PLSQR_TC_PAIR(16, 32)
  PLSQR_TC_PAIR(32, 32)
  PLSQR_TC_PAIR(32, 64)
  PLSQR_TC_PAIR(64, 64)
  PLSQR_TC_PAIR(96, 32)
  PLSQR_TC_PAIR(48, 16)
  PLSQR_TC_PAIR(32, 16)
  PLSQR_TC_PAIR(64, 32)
  PLSQR_TC_PAIR(32, 96)
  PLSQR_TC_PAIR(16, 48)
#undef PLSQR_TC_PAIR
  snprintf(net->err, sizeof net->err, "no tensor-core convolution for %d -> %d channels", ci, co);
  return PLSQR_ERR_ARG;
}

bool conv_tc_supported(int cin, int cout) {
  const int pairs[][2] = {{16, 16}, {16, 32}, {32, 32}, {32, 64}, {64, 64}, {96, 32}, {48, 16}};
  for (auto &p : pairs)
    if (p[0] == cin && p[1] == cout) return true;
  return false;
}

// The device flag of the tensor-core convolutions, after the stream has
// drained: PLSQR_ERR_TIMEOUT (and the flag cleared) when a wait ran out.
int check_flag(plsqr_unet *net) {
  unsigned int f = 0;
  UK(cudaMemcpy(&f, net->dflag, sizeof f, cudaMemcpyDeviceToHost));
  if (f) {
    UK(cudaMemset(net->dflag, 0, sizeof f));
    snprintf(net->err, sizeof net->err,
             "a tensor-core convolution's wait on its MMAs ran out (one second)");
    return PLSQR_ERR_TIMEOUT;
  }
  return PLSQR_OK;
}

template <int N>
int gemm_tc_run(plsqr_unet *net, const GemmTcArgs &a, int mtiles, int splits) {
  constexpr uint32_t cols = tc_cols(N);
  constexpr int floor_bytes = cols >= 128 ? 58 * 1024 : cols >= 64 ? 30 * 1024 : 0;
  constexpr int need = GemmTcShape<N>::kSmemBytes;
  constexpr int bytes = need > floor_bytes ? need : floor_bytes;
  static_assert(bytes <= 227 * 1024, "shared memory of one CTA");
  UK(cudaFuncSetAttribute(k_gemm_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  k_gemm_tc<N><<<dim3((unsigned)mtiles, (unsigned)splits), kTcThreads, bytes, net->stream>>>(a);
  UK(cudaGetLastError());
  return PLSQR_OK;
}

// gw[n][m] = sum_k A[m][k] B[n][k] (A [M][K], B [N][K], BF16) on the
// tensor cores, split over k so that about two CTAs per SM run.
int gemm_tc(plsqr_unet *net, const bf16 *A, const bf16 *B, int64_t M, int64_t K, int N,
            float *gw) {
  const int mtiles = (int)((M + kTcRows - 1) / kTcRows);
  int64_t splits = std::max<int64_t>(1, std::min<int64_t>((K + 63) / 64, 304 / mtiles));
  while (splits > 1 && splits * M * N > net->part_cap) --splits;
  int64_t kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + 63) / 64 * 64;
  splits = (K + kchunk - 1) / kchunk;
  if (splits * M * N > net->part_cap) {
    snprintf(net->err, sizeof net->err, "weight-gradient scratch too small");
    return PLSQR_ERR_ARG;
  }
  GemmTcArgs a{A, B, M, K, kchunk, net->part, net->dflag};
  int rc = PLSQR_ERR_ARG;
  if (N == 16) rc = gemm_tc_run<16>(net, a, mtiles, (int)splits);
  else if (N == 32) rc = gemm_tc_run<32>(net, a, mtiles, (int)splits);
  else if (N == 64) rc = gemm_tc_run<64>(net, a, mtiles, (int)splits);
  else snprintf(net->err, sizeof net->err, "no tensor-core weight gradient for %d channels", N);
  if (rc) return rc;
  k_gemm_tc_reduce<<<grid_for(M * N), kT, 0, net->stream>>>(net->part, (int)splits, M, N, gw);
  UK(cudaGetLastError());
  return PLSQR_OK;
}

// act = relu(conv(x) + b): one implicit-GEMM launch.
int conv_fwd(plsqr_unet *net, Conv &L, const bf16 *x, bf16 *act) {
  ConvTcArgs a{};
  a.x = x;
  a.w = L.wb;  // B_t[co][ci] = wb[co][t*cin + ci]
  a.ldw = L.K();
  a.tap_stride = L.cin;
  a.flip = 0;
  a.bias = L.b;
  a.relu = 1;
  a.out_bf16 = act;
  a.g = L.g;
  a.err = net->dflag;
  return conv_tc(net, L.cin, L.cout, a);
}

// The gradients of one layer from d(act) (FP32 [n][cout]): gw, gb, and dx
// (FP32 [n][cin]) when dx is given.
int conv_bwd(plsqr_unet *net, Conv &L, const bf16 *x, const bf16 *act, const float *dact,
             float *dx) {
  cudaStream_t s = net->stream;
  const int64_t n = L.g.n(), K = L.K();
  int rc;
  k_relu_back<<<grid_for(n * L.cout), kT, 0, s>>>(dact, act, n * L.cout, net->dz);
  k_bias_grad<<<kBiasBlocks, kBiasThreads, 0, s>>>(net->dz, n, L.cout, net->bparts);
  k_bias_grad_final<<<L.cout, 32, 0, s>>>(net->bparts, kBiasBlocks, L.cout, L.gb);
  k_im2col_t<<<grid_for(27 * n / 2), kT, 0, s>>>(x, L.g, L.cin, net->colt);
  const dim3 tb(32, 8);
  k_transpose_bf16<<<dim3((unsigned)((L.cout + 31) / 32), (unsigned)((n + 31) / 32)), tb, 0, s>>>(
      net->dz, n, L.cout, net->dzt);
  UK(cudaGetLastError());
  // dW[co][k] = sum_p dz[p][co] colt[k][p]
  if ((rc = gemm_tc(net, net->colt, net->dzt, K, n, L.cout, L.gw))) return rc;
  if (dx) {
    // dx[p][ci] = sum_t sum_co dz[p - offset(t)][co] W[co][t*cin + ci]: the
    // implicit GEMM on dz with mirrored taps and B_t[ci][co] = wbt[t*cin + ci][co]
    k_transpose_bf16<<<dim3((unsigned)((K + 31) / 32), (unsigned)((L.cout + 31) / 32)), tb, 0, s>>>(
        L.wb, L.cout, K, L.wbt);
    UK(cudaGetLastError());
    ConvTcArgs a{};
    a.x = net->dz;
    a.w = L.wbt;
    a.ldw = L.cout;
    a.tap_stride = (int64_t)L.cin * L.cout;
    a.flip = 1;
    a.out_f32 = dx;
    a.g = L.g;
    a.err = net->dflag;
    if ((rc = conv_tc(net, L.cout, L.cin, a))) return rc;
  }
  return PLSQR_OK;
}

int adam_layer(plsqr_unet *net, Conv &L, float lr, float c1, float c2) {
  const int64_t nw = (int64_t)L.cout * L.K();
  k_adam<<<grid_for(nw), kT, 0, net->stream>>>(L.w, L.gw, L.mw, L.vw, nw, lr, 0.9f, 0.999f, 1e-8f,
                                               c1, c2, L.wb);
  k_adam<<<1, kT, 0, net->stream>>>(L.b, L.gb, L.mb, L.vb, L.cout, lr, 0.9f, 0.999f, 1e-8f, c1, c2,
                                    nullptr);
  UK(cudaGetLastError());
  return PLSQR_OK;
}

// The forward pass from net->in (n floats, host-scaled by 1/s inside) to
// net->out (x0 = s * head).
int forward(plsqr_unet *net, float s) {
  cudaStream_t st = net->stream;
  const Grid3 g0 = net->g0, g1 = net->g1, g2 = net->g2;
  const int64_t n0 = g0.n(), n1 = g1.n();
  int rc;
  k_input16<<<grid_for(n0 * 16), kT, 0, st>>>(net->in, n0, 1.f / s, net->x16);
  if ((rc = conv_fwd(net, net->e1a, net->x16, net->a_e1a)) ||
      (rc = conv_fwd(net, net->e1b, net->a_e1a, net->a_e1b)))
    return rc;
  k_avgpool<<<grid_for(n1 * 16), kT, 0, st>>>(net->a_e1b, g0, 16, net->a_p1);
  if ((rc = conv_fwd(net, net->e2a, net->a_p1, net->a_e2a)) ||
      (rc = conv_fwd(net, net->e2b, net->a_e2a, net->a_e2b)))
    return rc;
  k_avgpool<<<grid_for(g2.n() * 32), kT, 0, st>>>(net->a_e2b, g1, 32, net->a_p2);
  if ((rc = conv_fwd(net, net->ba, net->a_p2, net->a_ba)) ||
      (rc = conv_fwd(net, net->bb, net->a_ba, net->a_bb)))
    return rc;
  k_upsample<<<grid_for(n1 * 64), kT, 0, st>>>(net->a_bb, g1, 64, 96, 0, net->a_c2);
  k_copy_channels<<<grid_for(n1 * 32), kT, 0, st>>>(net->a_e2b, n1, 32, 96, 64, net->a_c2);
  if ((rc = conv_fwd(net, net->d2a, net->a_c2, net->a_d2a)) ||
      (rc = conv_fwd(net, net->d2b, net->a_d2a, net->a_d2b)))
    return rc;
  k_upsample<<<grid_for(n0 * 32), kT, 0, st>>>(net->a_d2b, g0, 32, 48, 0, net->a_c1);
  k_copy_channels<<<grid_for(n0 * 16), kT, 0, st>>>(net->a_e1b, n0, 16, 48, 32, net->a_c1);
  if ((rc = conv_fwd(net, net->d1a, net->a_c1, net->a_d1a)) ||
      (rc = conv_fwd(net, net->d1b, net->a_d1a, net->a_d1b)))
    return rc;
  float hb = 0.f;
  UK(cudaMemcpyAsync(&hb, net->hw + 16, sizeof(float), cudaMemcpyDeviceToHost, st));
  UK(cudaStreamSynchronize(st));
  if ((rc = check_flag(net))) return rc;
  k_head<<<grid_for(n0), kT, 0, st>>>(net->a_d1b, n0, 16, net->hw, hb, s, net->out);
  UK(cudaGetLastError());
  return PLSQR_OK;
}

// Backward pass and Adam step after forward(); loss = mean squared error in
// the scaled units.
int backward(plsqr_unet *net, float s, float lr, float *loss) {
  cudaStream_t st = net->stream;
  const Grid3 g0 = net->g0, g1 = net->g1;
  const int64_t n0 = g0.n(), n1 = g1.n();
  const int hgrid = 152 * 4;
  int rc;
  k_head_back<<<hgrid, kT, 0, st>>>(net->a_d1b, n0, 16, net->hw, net->out, net->target, 1.f / s,
                                     net->g_d1b, net->hparts);
  UK(cudaGetLastError());
  std::vector<float> hp((size_t)hgrid * 18);
  UK(cudaMemcpyAsync(hp.data(), net->hparts, sizeof(float) * hp.size(), cudaMemcpyDeviceToHost, st));
  // level 0 decoder
  if ((rc = conv_bwd(net, net->d1b, net->a_d1a, net->a_d1b, net->g_d1b, net->g_d1a)) ||
      (rc = conv_bwd(net, net->d1a, net->a_c1, net->a_d1a, net->g_d1a, net->g_c1)))
    return rc;
  k_upsample_back<<<grid_for(n1 * 32), kT, 0, st>>>(net->g_c1, g0, 32, 48, 0, net->g_d2b);
  k_take_channels<<<grid_for(n0 * 16), kT, 0, st>>>(net->g_c1, n0, 16, 48, 32, 0, net->g_e1b);
  if ((rc = conv_bwd(net, net->d2b, net->a_d2a, net->a_d2b, net->g_d2b, net->g_d2a)) ||
      (rc = conv_bwd(net, net->d2a, net->a_c2, net->a_d2a, net->g_d2a, net->g_c2)))
    return rc;
  k_upsample_back<<<grid_for(net->g2.n() * 64), kT, 0, st>>>(net->g_c2, g1, 64, 96, 0, net->g_bb);
  k_take_channels<<<grid_for(n1 * 32), kT, 0, st>>>(net->g_c2, n1, 32, 96, 64, 0, net->g_e2b);
  if ((rc = conv_bwd(net, net->bb, net->a_ba, net->a_bb, net->g_bb, net->g_ba)) ||
      (rc = conv_bwd(net, net->ba, net->a_p2, net->a_ba, net->g_ba, net->g_p2)))
    return rc;
  k_avgpool_back<<<grid_for(n1 * 32), kT, 0, st>>>(net->g_p2, g1, 32, 1, net->g_e2b);
  if ((rc = conv_bwd(net, net->e2b, net->a_e2a, net->a_e2b, net->g_e2b, net->g_e2a)) ||
      (rc = conv_bwd(net, net->e2a, net->a_p1, net->a_e2a, net->g_e2a, net->g_p1)))
    return rc;
  k_avgpool_back<<<grid_for(n0 * 16), kT, 0, st>>>(net->g_p1, g0, 16, 1, net->g_e1b);
  if ((rc = conv_bwd(net, net->e1b, net->a_e1a, net->a_e1b, net->g_e1b, net->g_e1a)) ||
      (rc = conv_bwd(net, net->e1a, net->x16, net->a_e1a, net->g_e1a, nullptr)))
    return rc;
  UK(cudaGetLastError());
  UK(cudaStreamSynchronize(st));
  if ((rc = check_flag(net))) return rc;
  // head gradient (fixed order over the partials) and the loss
  float hg[17] = {0.f}, se = 0.f;
  for (int b = 0; b < hgrid; ++b) {
    for (int c = 0; c < 17; ++c) hg[c] += hp[(size_t)b * 18 + c];
    se += hp[(size_t)b * 18 + 17];
  }
  if (loss) *loss = se / (float)n0;
  UK(cudaMemcpyAsync(net->hg, hg, sizeof(hg), cudaMemcpyHostToDevice, st));
  ++net->step;
  const float c1 = 1.f - powf(0.9f, (float)net->step), c2 = 1.f - powf(0.999f, (float)net->step);
  Conv *layers[] = {&net->e1a, &net->e1b, &net->e2a, &net->e2b, &net->ba,
                    &net->bb,  &net->d2a, &net->d2b, &net->d1a, &net->d1b};
  for (Conv *L : layers)
    if ((rc = adam_layer(net, *L, lr, c1, c2))) return rc;
  k_adam<<<1, 32, 0, st>>>(net->hw, net->hg, net->hm, net->hv, 17, lr, 0.9f, 0.999f, 1e-8f, c1, c2,
                           nullptr);
  UK(cudaGetLastError());
  UK(cudaStreamSynchronize(st));
  return PLSQR_OK;
}

constexpr int kRmsBlocks = 304;

// The root mean square of net->in (1 for a zero volume): FP64 block sums on
// the device, added in block order on the host.
int input_rms(plsqr_unet *net, float *s) {
  const int64_t n = net->g0.n();
  k_sumsq_in<<<kRmsBlocks, 256, 0, net->stream>>>(net->in, n, net->sparts);
  UK(cudaGetLastError());
  double h[kRmsBlocks];
  UK(cudaMemcpyAsync(h, net->sparts, sizeof h, cudaMemcpyDeviceToHost, net->stream));
  UK(cudaStreamSynchronize(net->stream));
  double t = 0.0;
  for (int b = 0; b < kRmsBlocks; ++b) t += h[b];
  const double r = n > 0 ? sqrt(t / (double)n) : 0.0;
  *s = r > 0.0 ? (float)r : 1.f;
  return PLSQR_OK;
}

}  // namespace

namespace {

// Scratch of the convolutions for layers of up to max_nk = n * K im2col
// entries, n * cout outputs and cout x K weights.
int alloc_scratch(plsqr_unet *net, int64_t max_nk, int64_t max_ncout, int64_t max_wk) {
  int rc;
  if ((rc = nalloc(net, &net->colt, max_nk)) || (rc = nalloc(net, &net->bparts, kBiasBlocks * 128)) ||
      (rc = nalloc(net, &net->dz, max_ncout)) || (rc = nalloc(net, &net->dzt, max_ncout)) ||
      (rc = nalloc(net, &net->part, 64 * max_wk)) || (rc = nalloc(net, &net->dflag, 1)))
    return rc;
  net->part_cap = 64 * max_wk;
  return PLSQR_OK;
}

void free_net(plsqr_unet *net) {
  if (!net) return;
  cudaSetDevice(net->device);
  for (void *p : net->allocs) cudaFree(p);
  if (net->ev) cudaEventDestroy(net->ev);
  if (net->stream) cudaStreamDestroy(net->stream);
  delete net;
}

int build_net(plsqr_unet *net, uint64_t seed) {
  const Grid3 g0 = net->g0, g1 = net->g1, g2 = net->g2;
  const int64_t n0 = g0.n(), n1 = g1.n(), n2 = g2.n();
  UK(cudaSetDevice(net->device));
  UK(cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking));
  int rc;
  struct Spec {
    Conv *L;
    int cin, cout;
    Grid3 g;
    int fan;
  } specs[] = {{&net->e1a, 16, 16, g0, 1},  {&net->e1b, 16, 16, g0, 16}, {&net->e2a, 16, 32, g1, 16},
               {&net->e2b, 32, 32, g1, 32}, {&net->ba, 32, 64, g2, 32},  {&net->bb, 64, 64, g2, 64},
               {&net->d2a, 96, 32, g1, 96}, {&net->d2b, 32, 32, g1, 32}, {&net->d1a, 48, 16, g0, 48},
               {&net->d1b, 16, 16, g0, 16}};
  int64_t max_nk = 0, max_nc = 0, max_wk = 0;
  uint64_t sd = seed;
  for (auto &sp : specs) {
    if ((rc = init_conv(net, *sp.L, sp.cin, sp.cout, sp.g, sp.fan, ++sd))) return rc;
    max_nk = std::max(max_nk, sp.g.n() * sp.L->K());
    max_nc = std::max(max_nc, sp.g.n() * sp.cout);
    max_wk = std::max(max_wk, (int64_t)sp.cout * sp.L->K());
  }
  if ((rc = alloc_scratch(net, max_nk, max_nc, max_wk))) return rc;
  struct A {
    bf16 **a;
    float **g;
    int64_t n;
  } acts[] = {{&net->a_e1a, &net->g_e1a, n0 * 16}, {&net->a_e1b, &net->g_e1b, n0 * 16},
              {&net->a_p1, &net->g_p1, n1 * 16},   {&net->a_e2a, &net->g_e2a, n1 * 32},
              {&net->a_e2b, &net->g_e2b, n1 * 32}, {&net->a_p2, &net->g_p2, n2 * 32},
              {&net->a_ba, &net->g_ba, n2 * 64},   {&net->a_bb, &net->g_bb, n2 * 64},
              {&net->a_c2, &net->g_c2, n1 * 96},   {&net->a_d2a, &net->g_d2a, n1 * 32},
              {&net->a_d2b, &net->g_d2b, n1 * 32}, {&net->a_c1, &net->g_c1, n0 * 48},
              {&net->a_d1a, &net->g_d1a, n0 * 16}, {&net->a_d1b, &net->g_d1b, n0 * 16}};
  for (auto &a : acts)
    if ((rc = nalloc(net, a.a, a.n)) || (rc = nalloc(net, a.g, a.n))) return rc;
  if ((rc = nalloc(net, &net->x16, n0 * 16)) || (rc = nalloc(net, &net->in, n0)) ||
      (rc = nalloc(net, &net->out, n0)) || (rc = nalloc(net, &net->target, n0)) ||
      (rc = nalloc(net, &net->hparts, 152 * 4 * 18)) || (rc = nalloc(net, &net->hw, 17)) ||
      (rc = nalloc(net, &net->hm, 17)) || (rc = nalloc(net, &net->hv, 17)) ||
      (rc = nalloc(net, &net->hg, 17)) || (rc = nalloc(net, &net->sparts, kRmsBlocks)))
    return rc;
  UK(cudaEventCreateWithFlags(&net->ev, cudaEventDisableTiming));
  float h[17];
  for (int c = 0; c < 16; ++c) h[c] = (float)(0.25 * det_normal(seed + 77, (uint64_t)c));
  h[16] = 0.f;
  UK(cudaMemcpy(net->hw, h, sizeof(h), cudaMemcpyHostToDevice));
  UK(cudaStreamSynchronize(net->stream));
  return PLSQR_OK;
}

Conv *layer_list(plsqr_unet *net, int i) {
  Conv *l[] = {&net->e1a, &net->e1b, &net->e2a, &net->e2b, &net->ba,
               &net->bb,  &net->d2a, &net->d2b, &net->d1a, &net->d1b};
  return i < 10 ? l[i] : nullptr;
}

}  // namespace

// ---- C ABI ----------------------------------------------------------------------
extern "C" int plsqr_unet_create(int32_t nx, int32_t ny, int32_t nz, uint64_t seed,
                                 int32_t device, plsqr_unet **out) {
  if (!out || nx < 4 || ny < 4 || nz < 4 || nx % 4 || ny % 4 || nz % 4 ||
      ((int64_t)nx * ny * nz / 64) % 8)
    return PLSQR_ERR_ARG;
  *out = nullptr;
  int32_t ndev = 0;
  plsqr_device_count(&ndev);
  if (device < 0 || device >= ndev) return PLSQR_ERR_NODEV;
  plsqr_unet *net = new plsqr_unet();
  net->device = device;
  net->g0 = Grid3{nx, ny, nz};
  net->g1 = Grid3{nx / 2, ny / 2, nz / 2};
  net->g2 = Grid3{nx / 4, ny / 4, nz / 4};
  const int rc = build_net(net, seed);
  if (rc) {
    free_net(net);
    return rc;
  }
  *out = net;
  return PLSQR_OK;
}

extern "C" void plsqr_unet_destroy(plsqr_unet *net) { free_net(net); }

extern "C" const char *plsqr_unet_last_error(const plsqr_unet *net) { return net ? net->err : ""; }

// The calls on host arrays (kind = cudaMemcpyHostToDevice / DeviceToHost)
// and on device arrays ordered on the caller's stream (DeviceToDevice).
static int predict_impl(plsqr_unet *net, const float *in, float *out, cudaMemcpyKind kin,
                        cudaMemcpyKind kout) {
  const int64_t n = net->g0.n();
  UK(cudaSetDevice(net->device));
  UK(cudaMemcpyAsync(net->in, in, sizeof(float) * n, kin, net->stream));
  float s = 1.f;
  int rc;
  if ((rc = input_rms(net, &s)) || (rc = forward(net, s))) return rc;
  UK(cudaMemcpyAsync(out, net->out, sizeof(float) * n, kout, net->stream));
  return PLSQR_OK;
}

static int train_impl(plsqr_unet *net, const float *in, const float *target, float lr,
                      float *loss, cudaMemcpyKind kin) {
  const int64_t n = net->g0.n();
  UK(cudaSetDevice(net->device));
  UK(cudaMemcpyAsync(net->in, in, sizeof(float) * n, kin, net->stream));
  UK(cudaMemcpyAsync(net->target, target, sizeof(float) * n, kin, net->stream));
  float s = 1.f;
  int rc;
  if ((rc = input_rms(net, &s)) || (rc = forward(net, s))) return rc;
  return backward(net, s, lr, loss);
}

// Make the network's stream wait for `from`.
static int stream_after(plsqr_unet *net, cudaStream_t to, cudaStream_t from) {
  UK(cudaEventRecord(net->ev, from));
  UK(cudaStreamWaitEvent(to, net->ev, 0));
  return PLSQR_OK;
}

extern "C" int plsqr_unet_predict(plsqr_unet *net, const float *in, float *out) {
  if (!net || !in || !out) return PLSQR_ERR_ARG;
  int rc;
  if ((rc = predict_impl(net, in, out, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost))) return rc;
  UK(cudaStreamSynchronize(net->stream));
  return PLSQR_OK;
}

extern "C" int plsqr_unet_train_step(plsqr_unet *net, const float *in, const float *target,
                                     float lr, float *loss) {
  if (!net || !in || !target || !(lr > 0.f)) return PLSQR_ERR_ARG;
  return train_impl(net, in, target, lr, loss, cudaMemcpyHostToDevice);
}

extern "C" int plsqr_unet_predict_device(plsqr_unet *net, const float *in, float *out,
                                         void *stream) {
  if (!net || !in || !out) return PLSQR_ERR_ARG;
  const cudaStream_t cs = (cudaStream_t)stream;
  UK(cudaSetDevice(net->device));
  int rc;
  if ((rc = stream_after(net, net->stream, cs)) ||
      (rc = predict_impl(net, in, out, cudaMemcpyDeviceToDevice, cudaMemcpyDeviceToDevice)) ||
      (rc = stream_after(net, cs, net->stream)))
    return rc;
  return PLSQR_OK;
}

extern "C" int plsqr_unet_train_step_device(plsqr_unet *net, const float *in, const float *target,
                                            float lr, float *loss, void *stream) {
  if (!net || !in || !target || !(lr > 0.f)) return PLSQR_ERR_ARG;
  const cudaStream_t cs = (cudaStream_t)stream;
  UK(cudaSetDevice(net->device));
  int rc;
  if ((rc = stream_after(net, net->stream, cs)) ||
      (rc = train_impl(net, in, target, lr, loss, cudaMemcpyDeviceToDevice)) ||
      (rc = stream_after(net, cs, net->stream)))
    return rc;
  return PLSQR_OK;
}

// All trainable values, layer by layer (w then b), then the head (16 + 1).
extern "C" int plsqr_unet_weights(plsqr_unet *net, float *buf, int64_t *count, int32_t set) {
  if (!net || !count) return PLSQR_ERR_ARG;
  int64_t total = 17;
  for (int i = 0; i < 10; ++i) total += (int64_t)layer_list(net, i)->cout * (layer_list(net, i)->K() + 1);
  if (!buf) {
    *count = total;
    return PLSQR_OK;
  }
  if (*count < total) return PLSQR_ERR_ARG;
  UK(cudaSetDevice(net->device));
  int64_t off = 0;
  for (int i = 0; i < 10; ++i) {
    Conv &L = *layer_list(net, i);
    const int64_t nw = (int64_t)L.cout * L.K();
    if (set) {
      UK(cudaMemcpy(L.w, buf + off, sizeof(float) * nw, cudaMemcpyHostToDevice));
      UK(cudaMemcpy(L.b, buf + off + nw, sizeof(float) * L.cout, cudaMemcpyHostToDevice));
      k_f32_to_bf16<<<grid_for(nw), kT, 0, net->stream>>>(L.w, nw, L.wb);
      UK(cudaGetLastError());
    } else {
      UK(cudaMemcpy(buf + off, L.w, sizeof(float) * nw, cudaMemcpyDeviceToHost));
      UK(cudaMemcpy(buf + off + nw, L.b, sizeof(float) * L.cout, cudaMemcpyDeviceToHost));
    }
    off += nw + L.cout;
  }
  if (set)
    UK(cudaMemcpy(net->hw, buf + off, sizeof(float) * 17, cudaMemcpyHostToDevice));
  else
    UK(cudaMemcpy(buf + off, net->hw, sizeof(float) * 17, cudaMemcpyDeviceToHost));
  UK(cudaStreamSynchronize(net->stream));
  *count = total;
  return PLSQR_OK;
}

// One 3x3x3 convolution layer with its ReLU, forward and backward, on host
// arrays: the kernels of the network checked in isolation.
extern "C" int plsqr_nn_conv3d_check(int32_t nx, int32_t ny, int32_t nz, int32_t cin,
                                     int32_t cout, const float *x, const float *w,
                                     const float *b, const float *dy, float *y, float *dx,
                                     float *dw, float *db) {
  if (nx < 1 || ny < 1 || nz < 1 || !conv_tc_supported(cin, cout) ||
      ((int64_t)nx * ny * nz) % 8 || !x || !w || !b || !dy || !y || !dx || !dw || !db)
    return PLSQR_ERR_ARG;
  int32_t ndev = 0;
  plsqr_device_count(&ndev);
  if (ndev < 1) return PLSQR_ERR_NODEV;
  plsqr_unet *net = new plsqr_unet();
  int rc = PLSQR_OK;
  do {
    net->device = 0;
    if (cudaSetDevice(0) != cudaSuccess ||
        cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) != cudaSuccess) {
      rc = PLSQR_ERR_CUDA;
      break;
    }
    Conv L;
    L.cin = cin;
    L.cout = cout;
    L.g = Grid3{nx, ny, nz};
    const int64_t n = L.g.n(), K = L.K(), nw = (int64_t)cout * K;
    bf16 *xb, *act;
    float *xf, *dyf, *dxf;
    if ((rc = nalloc(net, &L.w, nw)) || (rc = nalloc(net, &L.b, cout)) ||
        (rc = nalloc(net, &L.wb, nw)) || (rc = nalloc(net, &L.wbt, nw)) ||
        (rc = nalloc(net, &L.gw, nw)) || (rc = nalloc(net, &L.gb, cout)) ||
        (rc = nalloc(net, &xb, n * cin)) || (rc = nalloc(net, &xf, n * cin)) ||
        (rc = nalloc(net, &act, n * cout)) || (rc = nalloc(net, &dyf, n * cout)) ||
        (rc = nalloc(net, &dxf, n * cin)) || (rc = alloc_scratch(net, n * K, n * cout, nw)))
      break;
    if (cudaMemcpy(L.w, w, sizeof(float) * nw, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(L.b, b, sizeof(float) * cout, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(xf, x, sizeof(float) * n * cin, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dyf, dy, sizeof(float) * n * cout, cudaMemcpyHostToDevice) != cudaSuccess) {
      rc = PLSQR_ERR_CUDA;
      break;
    }
    k_f32_to_bf16<<<grid_for(nw), kT, 0, net->stream>>>(L.w, nw, L.wb);
    k_f32_to_bf16<<<grid_for(n * cin), kT, 0, net->stream>>>(xf, n * cin, xb);
    if ((rc = conv_fwd(net, L, xb, act)) || (rc = conv_bwd(net, L, xb, act, dyf, dxf))) break;
    std::vector<bf16> hb((size_t)(n * cout));
    if (cudaStreamSynchronize(net->stream) != cudaSuccess ||
        cudaMemcpy(hb.data(), act, sizeof(bf16) * n * cout, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dx, dxf, sizeof(float) * n * cin, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dw, L.gw, sizeof(float) * nw, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(db, L.gb, sizeof(float) * cout, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = PLSQR_ERR_CUDA;
      break;
    }
    if ((rc = check_flag(net))) break;
    for (int64_t i = 0; i < n * cout; ++i) y[i] = __bfloat162float(hb[(size_t)i]);
  } while (0);
  free_net(net);
  return rc;
}
