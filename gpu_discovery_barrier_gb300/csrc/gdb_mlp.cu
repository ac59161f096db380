// Schedule selector: loading the network, and its training on the GPU.
//
// Training is full-batch Adam over a masked squared loss.  One step is
// three kernels:
//   k_mlp_fwd_bwd  one thread per sample: forward pass, output error and the
//                  back-propagated errors of both hidden layers, stored
//                  feature-major (act[f * n + s]);
//   k_mlp_wgrad    one warp per gradient entry: the sum over samples of
//                  (input activation x output error), accumulated in FP64
//                  in a fixed lane-stride order and a fixed shuffle tree,
//                  so gradients are bit-identical from run to run;
//   k_mlp_adam     one thread per parameter.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gdb_internal.h"
#include "gdb_selector.cuh"

using namespace gdbi;
using namespace gdb;

namespace {

// Per-sample activation rows: xn 12, h1 32, h2 32, dh1 32, dh2 32, dy 6, loss 1.
constexpr int kAXn = 0, kAH1 = kAXn + kFeat, kAH2 = kAH1 + kH1, kADh1 = kAH2 + kH2,
              kADh2 = kADh1 + kH1, kADy = kADh2 + kH2, kALoss = kADy + kOut, kActRows = kALoss + 1;
// Gradient entries: W1, b1, W2, b2, W3, b3 (the blob minus shift/scale), then the loss.
constexpr int kGradEntries = kParams - kPW1;

__device__ __forceinline__ void mlp_thread(const float* p, const float* x, float* xn, float* h1,
                                           float* h2, float* y) {
  for (int i = 0; i < kFeat; ++i) xn[i] = __fmul_rn(__fsub_rn(x[i], p[kPShift + i]), p[kPScale + i]);
  for (int j = 0; j < kH1; ++j) {
    float h = p[kPB1 + j];
    for (int i = 0; i < kFeat; ++i) h = __fmaf_rn(xn[i], p[kPW1 + i * kH1 + j], h);
    h1[j] = fmaxf(h, 0.f);
  }
  for (int j = 0; j < kH2; ++j) {
    float h = p[kPB2 + j];
    for (int k = 0; k < kH1; ++k) h = __fmaf_rn(h1[k], p[kPW2 + k * kH2 + j], h);
    h2[j] = fmaxf(h, 0.f);
  }
  for (int j = 0; j < kOut; ++j) {
    float o = p[kPB3 + j];
    for (int k = 0; k < kH2; ++k) o = __fmaf_rn(h2[k], p[kPW3 + k * kOut + j], o);
    y[j] = o;
  }
}

__global__ void k_mlp_forward(const float* __restrict__ p, const float* __restrict__ X, uint32_t n,
                              float* __restrict__ Y) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[kFeat], xn[kFeat], h1[kH1], h2[kH2], y[kOut];
  for (int i = 0; i < kFeat; ++i) x[i] = X[(size_t)s * kFeat + i];
  mlp_thread(p, x, xn, h1, h2, y);
  for (int j = 0; j < kOut; ++j) Y[(size_t)s * kOut + j] = y[j];
}

__global__ void k_mlp_fwd_bwd(const float* __restrict__ p, const float* __restrict__ X,
                              const float* __restrict__ T, const float* __restrict__ M, uint32_t n,
                              float inv_m, float* __restrict__ act) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[kFeat], xn[kFeat], h1[kH1], h2[kH2], y[kOut], dy[kOut];
  for (int i = 0; i < kFeat; ++i) x[i] = X[(size_t)s * kFeat + i];
  mlp_thread(p, x, xn, h1, h2, y);
  float loss = 0.f;
  for (int j = 0; j < kOut; ++j) {
    const float m = M[(size_t)s * kOut + j];
    const float e = y[j] - T[(size_t)s * kOut + j];
    dy[j] = m != 0.f ? 2.f * m * e * inv_m : 0.f;
    if (m != 0.f) loss = __fmaf_rn(m * e, e * inv_m, loss);
  }
  auto put = [&](int row, float v) { act[(size_t)row * n + s] = v; };
  for (int i = 0; i < kFeat; ++i) put(kAXn + i, xn[i]);
  for (int j = 0; j < kH1; ++j) put(kAH1 + j, h1[j]);
  for (int j = 0; j < kH2; ++j) put(kAH2 + j, h2[j]);
  for (int j = 0; j < kOut; ++j) put(kADy + j, dy[j]);
  put(kALoss, loss);
  // dh2 = W3 . dy masked by ReLU; dh1 = W2 . dh2 masked by ReLU
  float dh2[kH2];
  for (int k = 0; k < kH2; ++k) {
    float a = 0.f;
    for (int j = 0; j < kOut; ++j) a = __fmaf_rn(p[kPW3 + k * kOut + j], dy[j], a);
    dh2[k] = h2[k] > 0.f ? a : 0.f;
    put(kADh2 + k, dh2[k]);
  }
  for (int k = 0; k < kH1; ++k) {
    float a = 0.f;
    for (int j = 0; j < kH2; ++j) a = __fmaf_rn(p[kPW2 + k * kH2 + j], dh2[j], a);
    put(kADh1 + k, h1[k] > 0.f ? a : 0.f);
  }
}

// Gradient entry e (0-based over W1, b1, W2, b2, W3, b3) as a pair of
// activation rows (a row < 0 means the constant 1 of a bias).
__device__ __forceinline__ void grad_rows(int e, int& ra, int& rd) {
  if (e < kFeat * kH1) {
    ra = kAXn + e / kH1;
    rd = kADh1 + e % kH1;
    return;
  }
  e -= kFeat * kH1;
  if (e < kH1) {
    ra = -1;
    rd = kADh1 + e;
    return;
  }
  e -= kH1;
  if (e < kH1 * kH2) {
    ra = kAH1 + e / kH2;
    rd = kADh2 + e % kH2;
    return;
  }
  e -= kH1 * kH2;
  if (e < kH2) {
    ra = -1;
    rd = kADh2 + e;
    return;
  }
  e -= kH2;
  if (e < kH2 * kOut) {
    ra = kAH2 + e / kOut;
    rd = kADy + e % kOut;
    return;
  }
  e -= kH2 * kOut;
  ra = -1;
  rd = kADy + e;
}

__global__ void k_mlp_wgrad(const float* __restrict__ act, uint32_t n, float* __restrict__ grad,
                            double* __restrict__ loss) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e > kGradEntries) return;
  double acc = 0.0;
  if (e == kGradEntries) {
    for (uint32_t s = lane; s < n; s += 32) acc += (double)act[(size_t)kALoss * n + s];
  } else {
    int ra, rd;
    grad_rows(e, ra, rd);
    const float* A = ra >= 0 ? act + (size_t)ra * n : nullptr;
    const float* D = act + (size_t)rd * n;
    for (uint32_t s = lane; s < n; s += 32) acc += (A ? (double)A[s] : 1.0) * (double)D[s];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    if (e == kGradEntries) *loss = acc;
    else grad[kPW1 + e] = (float)acc;
  }
}

__global__ void k_mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                           float* __restrict__ m2, float lr_t, float wd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kPW1 || i >= kParams) return;
  const bool weight = (i >= kPW1 && i < kPB1) || (i >= kPW2 && i < kPB2) || (i >= kPW3 && i < kPB3);
  float gi = g[i];
  if (weight) gi += wd * p[i];
  m1[i] = 0.9f * m1[i] + 0.1f * gi;
  m2[i] = 0.999f * m2[i] + 0.001f * gi * gi;
  p[i] -= lr_t * m1[i] / (sqrtf(m2[i]) + 1e-8f);
}

// Device buffers of one training / gradient call.
struct MlpBufs {
  float *p = nullptr, *x = nullptr, *t = nullptr, *m = nullptr, *act = nullptr, *g = nullptr,
        *m1 = nullptr, *m2 = nullptr;
  double* loss = nullptr;
  char* base = nullptr;
};

int mlp_upload(gdb_ctx* c, MlpBufs& b, const float* params, const float* x, const float* t,
               const float* m, uint32_t n, bool adam) {
  Bump bp;
  const size_t o_p = bp.take(kParams * 4), o_x = bp.take((size_t)n * kFeat * 4),
               o_t = bp.take((size_t)n * kOut * 4), o_m = bp.take((size_t)n * kOut * 4),
               o_a = bp.take((size_t)n * kActRows * 4), o_g = bp.take(kParams * 4),
               o_m1 = bp.take(adam ? kParams * 4 : 0), o_m2 = bp.take(adam ? kParams * 4 : 0),
               o_l = bp.take(8);
  GDB_CUDA(c, cudaMallocAsync((void**)&b.base, bp.off, c->stream));
  b.p = (float*)(b.base + o_p);
  b.x = (float*)(b.base + o_x);
  b.t = (float*)(b.base + o_t);
  b.m = (float*)(b.base + o_m);
  b.act = (float*)(b.base + o_a);
  b.g = (float*)(b.base + o_g);
  b.m1 = (float*)(b.base + o_m1);
  b.m2 = (float*)(b.base + o_m2);
  b.loss = (double*)(b.base + o_l);
  GDB_CUDA(c, cudaMemcpyAsync(b.p, params, kParams * 4, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaMemcpyAsync(b.x, x, (size_t)n * kFeat * 4, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaMemcpyAsync(b.t, t, (size_t)n * kOut * 4, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaMemcpyAsync(b.m, m, (size_t)n * kOut * 4, cudaMemcpyHostToDevice, c->stream));
  GDB_CUDA(c, cudaMemsetAsync(b.g, 0, kParams * 4, c->stream));
  if (adam) {
    GDB_CUDA(c, cudaMemsetAsync(b.m1, 0, kParams * 4, c->stream));
    GDB_CUDA(c, cudaMemsetAsync(b.m2, 0, kParams * 4, c->stream));
  }
  return GDB_OK;
}

int mlp_step(gdb_ctx* c, MlpBufs& b, uint32_t n, float inv_m) {
  k_mlp_fwd_bwd<<<(n + 127) / 128, 128, 0, c->stream>>>(b.p, b.x, b.t, b.m, n, inv_m, b.act);
  k_mlp_wgrad<<<(kGradEntries + 1 + 7) / 8, 256, 0, c->stream>>>(b.act, n, b.g, b.loss);
  GDB_CUDA(c, cudaGetLastError());
  return GDB_OK;
}

float mask_inverse(const float* m, uint32_t n) {
  double s = 0;
  for (size_t i = 0; i < (size_t)n * kOut; ++i) s += m[i];
  return s > 0 ? (float)(1.0 / s) : 0.f;
}

}  // namespace

extern "C" {

int gdb_selector_set(gdb_ctx* c, const float* params) {
  if (!c) return GDB_ERR_INVALID;
  if (!params) {
    if (c->d_mlp) cudaFree(c->d_mlp);
    c->d_mlp = nullptr;
    c->h_mlp.clear();
    return GDB_OK;
  }
  for (int i = 0; i < kParams; ++i)
    if (!std::isfinite(params[i])) return set_error(c, GDB_ERR_INVALID, "selector parameters not finite");
  if (!c->d_mlp) GDB_CUDA(c, cudaMalloc((void**)&c->d_mlp, kParams * 4));
  GDB_CUDA(c, cudaMemcpy(c->d_mlp, params, kParams * 4, cudaMemcpyHostToDevice));
  c->h_mlp.assign(params, params + kParams);
  return GDB_OK;
}

int gdb_mlp_forward(gdb_ctx* c, const float* params, const float* x, uint32_t n, float* y) {
  if (!c || !params || !x || !y) return GDB_ERR_INVALID;
  if (n == 0) return GDB_OK;
  char* d = nullptr;
  const size_t bp = kParams * 4, bx = (size_t)n * kFeat * 4, by = (size_t)n * kOut * 4;
  GDB_CUDA(c, cudaMallocAsync((void**)&d, bp + bx + by, c->stream));
  cudaError_t e = cudaMemcpyAsync(d, params, bp, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d + bp, x, bx, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    k_mlp_forward<<<(n + 127) / 128, 128, 0, c->stream>>>((float*)d, (float*)(d + bp), n,
                                                          (float*)(d + bp + bx));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, d + bp + bx, by, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? GDB_OK : set_cuda_error(c, e, "mlp forward");
}

int gdb_mlp_loss_grad(gdb_ctx* c, const float* params, const float* x, const float* t, const float* m,
                      uint32_t n, float* grad, double* loss) {
  if (!c || !params || !x || !t || !m || !grad || n == 0) return GDB_ERR_INVALID;
  MlpBufs b;
  int rc = mlp_upload(c, b, params, x, t, m, n, false);
  if (rc == GDB_OK) rc = mlp_step(c, b, n, mask_inverse(m, n));
  cudaError_t e = cudaSuccess;
  if (rc == GDB_OK) {
    e = cudaMemcpyAsync(grad, b.g, kParams * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, b.loss, 8, cudaMemcpyDeviceToHost, c->stream);
  }
  if (b.base) cudaFreeAsync(b.base, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (rc == GDB_OK && e != cudaSuccess) rc = set_cuda_error(c, e, "mlp gradient");
  return rc;
}

int gdb_mlp_train(gdb_ctx* c, float* params, const float* x, const float* t, const float* m, uint32_t n,
                  uint32_t epochs, float lr, float wd, double* loss) {
  if (!c || !params || !x || !t || !m || n == 0 || !(lr > 0.f)) return GDB_ERR_INVALID;
  MlpBufs b;
  int rc = mlp_upload(c, b, params, x, t, m, n, true);
  const float inv_m = mask_inverse(m, n);
  double b1t = 1.0, b2t = 1.0;
  for (uint32_t k = 0; rc == GDB_OK && k < epochs; ++k) {
    rc = mlp_step(c, b, n, inv_m);
    if (rc) break;
    b1t *= 0.9;
    b2t *= 0.999;
    const float lr_t = (float)(lr * std::sqrt(1.0 - b2t) / (1.0 - b1t));
    k_mlp_adam<<<(kParams + 255) / 256, 256, 0, c->stream>>>(b.p, b.g, b.m1, b.m2, lr_t, wd);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = set_cuda_error(c, e, "mlp adam");
  }
  cudaError_t e = cudaSuccess;
  if (rc == GDB_OK) {
    e = cudaMemcpyAsync(params, b.p, kParams * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, b.loss, 8, cudaMemcpyDeviceToHost, c->stream);
  }
  if (b.base) cudaFreeAsync(b.base, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (rc == GDB_OK && e != cudaSuccess) rc = set_cuda_error(c, e, "mlp training");
  return rc;
}

int gdb_sssp_features(gdb_ctx* c, gdb_graph* g, uint32_t nsrc, float* x) {
  if (!graph_ok(c, g) || !x || nsrc == 0) return GDB_ERR_INVALID;
  gdbi::sssp_features(c, g, nsrc, x);
  return GDB_OK;
}

}  // extern "C"

void gdbi::sssp_features(gdb_ctx* c, const gdb_graph* g, uint32_t nsrc, float* x) {
  const double V = g->V, E = (double)g->E;
  const double nf = std::min<double>(nsrc, V);
  const double mf = nf * E / std::max(V, 1.0);
  // warps of the launch: the traversal kernels' resident CTAs, capped by max_ctas
  double ctas = (double)c->sm_count * std::max(gdbi::traversal_occupancy(c, c->opt.block_size), 1);
  if (c->opt.max_ctas > 0) ctas = std::min(ctas, (double)c->opt.max_ctas);
  const double warps = ctas * (c->opt.block_size / 32);
  bfs_features(x, (float)nf, (float)mf, (float)std::max(E - mf, 0.0), (float)V, (float)E,
               (float)std::max(V - nf, 0.0), 0, 2, (float)g->maxdeg, (float)warps);
}
