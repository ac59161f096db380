// Learned schedule selector: a 12-32-32-6 ReLU MLP in FP32.
//
// Parameter blob (kParams floats, shared by the device, the host and the
// training kernels):
//   [0, 12)    feature shift      x_n = (x - shift) * scale
//   [12, 24)   feature scale
//   W1 [12][32] row-major (input-major), b1 [32]
//   W2 [32][32], b2 [32]
//   W3 [32][6],  b3 [6]
// The shift/scale pair is fitted on the training set and kept fixed.
//
// Outputs are predicted log2 costs of the options of one decision:
//   0 / 1  one BFS level run top-down from the queue (push) / bottom-up
//          against the previous level (pull);
//   2..5   one SSSP run: label-correcting worklist, near-far with the
//          automatic bucket width, near-far with 4x that width, worklist
//          under graph relaunch (one launch per superstep).
// A decision takes the argmin over its options; no output ever changes a
// result, only the time to reach it.
//
// Features (all float):
//   0 log2(1 + frontier vertices)     1 log2(1 + frontier arcs)
//   2 log2(1 + unvisited arcs)        3 log2(1 + V)
//   4 log2(1 + E)                     5 min(frontier arcs / unvisited arcs, 4)
//   6 frontier vertices / V           7 unvisited vertices / V
//   8 log2(1 + level)                 9 decision kind: previous BFS mode (0, 1)
//                                       or 2 for an SSSP run
//  10 log2(1 + max degree)           11 log2(1 + warps of the launch)
#pragma once

#include <cmath>
#include <cstdint>

namespace gdb {

constexpr int kFeat = 12, kH1 = 32, kH2 = 32, kOut = 6;
constexpr int kPShift = 0, kPScale = kFeat;
constexpr int kPW1 = 2 * kFeat;
constexpr int kPB1 = kPW1 + kFeat * kH1;
constexpr int kPW2 = kPB1 + kH1;
constexpr int kPB2 = kPW2 + kH1 * kH2;
constexpr int kPW3 = kPB2 + kH2;
constexpr int kPB3 = kPW3 + kH2 * kOut;
constexpr int kParams = kPB3 + kOut;  // 1694

enum SelOut {
  kOutPush = 0,
  kOutPull = 1,
  kOutSsspPlain = 2,
  kOutSsspNearFar = 3,
  kOutSsspNearFarWide = 4,
  kOutSsspRelaunch = 5
};

// BFS level features from the frontier and visit counters (float math,
// the same on every path that evaluates it on the device).
__host__ __device__ inline void bfs_features(float* x, float nf, float mf, float mu, float V, float E,
                                             float unvisited_v, uint32_t level, uint32_t prev_mode,
                                             float maxdeg, float warps) {
  x[0] = log2f(1.f + nf);
  x[1] = log2f(1.f + mf);
  x[2] = log2f(1.f + mu);
  x[3] = log2f(1.f + V);
  x[4] = log2f(1.f + E);
  x[5] = fminf(mf / fmaxf(mu, 1.f), 4.f);
  x[6] = nf / fmaxf(V, 1.f);
  x[7] = unvisited_v / fmaxf(V, 1.f);
  x[8] = log2f(1.f + (float)level);
  x[9] = (float)prev_mode;
  x[10] = log2f(1.f + maxdeg);
  x[11] = log2f(1.f + warps);
}

#ifdef __CUDACC__
// One warp evaluates the network; every lane receives all kOut outputs.
// x: the kFeat features, identical in every lane.  p: parameter blob.
// The accumulation order is fixed and every step is an explicit fused
// multiply-add, so the host mirror below gives identical values.
__device__ __forceinline__ void mlp_warp(const float* p, const float* x, float* out) {
  const int lane = threadIdx.x & 31;
  float h1 = p[kPB1 + lane];
#pragma unroll
  for (int i = 0; i < kFeat; ++i) {
    const float xn = __fmul_rn(__fsub_rn(x[i], p[kPShift + i]), p[kPScale + i]);
    h1 = __fmaf_rn(xn, p[kPW1 + i * kH1 + lane], h1);
  }
  h1 = fmaxf(h1, 0.f);
  float h2 = p[kPB2 + lane];
#pragma unroll
  for (int k = 0; k < kH1; ++k) h2 = __fmaf_rn(__shfl_sync(0xffffffffu, h1, k), p[kPW2 + k * kH2 + lane], h2);
  h2 = fmaxf(h2, 0.f);
  const int j = lane < kOut ? lane : 0;
  float o = p[kPB3 + j];
#pragma unroll
  for (int k = 0; k < kH2; ++k) o = __fmaf_rn(__shfl_sync(0xffffffffu, h2, k), p[kPW3 + k * kOut + j], o);
#pragma unroll
  for (int q = 0; q < kOut; ++q) out[q] = __shfl_sync(0xffffffffu, o, q);
}
#endif

// Host mirror of mlp_warp (same operation order, explicit fma).
inline void mlp_host(const float* p, const float* x, float* out) {
  float h1[kH1], h2[kH2];
  for (int j = 0; j < kH1; ++j) {
    float h = p[kPB1 + j];
    for (int i = 0; i < kFeat; ++i) {
      const float xn = (x[i] - p[kPShift + i]) * p[kPScale + i];
      h = std::fma(xn, p[kPW1 + i * kH1 + j], h);
    }
    h1[j] = h > 0.f ? h : 0.f;
  }
  for (int j = 0; j < kH2; ++j) {
    float h = p[kPB2 + j];
    for (int k = 0; k < kH1; ++k) h = std::fma(h1[k], p[kPW2 + k * kH2 + j], h);
    h2[j] = h > 0.f ? h : 0.f;
  }
  for (int j = 0; j < kOut; ++j) {
    float o = p[kPB3 + j];
    for (int k = 0; k < kH2; ++k) o = std::fma(h2[k], p[kPW3 + k * kOut + j], o);
    out[j] = o;
  }
}

}  // namespace gdb
