// bfs_sched_dev.cuh -- device side of the learned per-level scheduler:
// level features, MLP forward pass and arm choice by one warp.  Used by the
// scheduler kernel (host-driven loop, recorder) and by init and the last
// block of level generation (CUDA-graph loop, where the next level's arm is
// picked without a kernel of its own).
#pragma once
#include <cuda_runtime.h>

#include "bfs_sched.h"

namespace bfsgb {

constexpr uint32_t kFullMask = 0xFFFFFFFFu;

// The level counters the features are made of.
struct LevelCounters {
  uint32_t F, EF, reached, lvl;
};

__device__ __forceinline__ LevelCounters level_counters(const BfsDevState *st) {
  return LevelCounters{st->F, st->EF, st->reached, st->lvl};
}

__device__ __forceinline__ void level_features(const LevelCounters &c, uint32_t n_cols,
                                               SchedGraphConst gc, float x[kSchedIn]) {
  x[0] = log2f(1.f + (float)c.F) / 32.f;
  x[1] = log2f(1.f + (float)c.EF) / 32.f;
  x[2] = 1.f - (float)c.reached / (float)n_cols;
  x[3] = fminf((float)c.lvl / gc.diam, 8.f) / 8.f;
  x[4] = gc.avg_deg_x;
}

// Forward pass of one sample by one warp.  Returns this lane's output logit
// (meaningful on lanes < 9) and the lane's hidden activations.  TRANSPOSED:
// W2 and W3 are stored column-major (W2[k][j] at kW2 + 32 k + j, W3[k][a] at
// kW3 + 9 k + a), the shared-memory copy the level loop stages, so that the
// 32 lanes read 32 different banks; otherwise the row-major layout of the
// parameter vector.  The dot products keep four partial sums (k mod 4), in
// the same order for both layouts, so every caller gets identical logits.
template <bool TRANSPOSED>
__device__ __forceinline__ float mlp_forward(const float *__restrict__ w,
                                             const float x[kSchedIn], uint32_t lane,
                                             float *h1_out, float *h2_out) {
  float a = w[kB1 + lane];
#pragma unroll
  for (int i = 0; i < kSchedIn; i++) a = fmaf(w[kW1 + lane * kSchedIn + i], x[i], a);
  const float h1 = fmaxf(a, 0.f);
  float b[4] = {w[kB2 + lane], 0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < kSchedHidden; k++) {
    const float wk = TRANSPOSED ? w[kW2 + k * kSchedHidden + lane] : w[kW2 + lane * kSchedHidden + k];
    b[k & 3] = fmaf(wk, __shfl_sync(kFullMask, h1, k), b[k & 3]);
  }
  const float h2 = fmaxf((b[0] + b[1]) + (b[2] + b[3]), 0.f);
  const bool out_lane = lane < (uint32_t)kSchedArms;
  const uint32_t ol = out_lane ? lane : 0u;
  float c[4] = {out_lane ? w[kB3 + lane] : 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < kSchedHidden; k++) {
    const float hk = __shfl_sync(kFullMask, h2, k);
    const float wk = TRANSPOSED ? w[kW3 + k * kSchedArms + ol] : w[kW3 + ol * kSchedHidden + k];
    if (out_lane) c[k & 3] = fmaf(wk, hk, c[k & 3]);
  }
  *h1_out = h1;
  *h2_out = h2;
  return (c[0] + c[1]) + (c[2] + c[3]);
}

// Index of parameter i in the transposed (shared-memory) layout.
__host__ __device__ __forceinline__ int sched_transposed_index(int i) {
  if (i >= kW2 && i < kB2) {
    const int j = (i - kW2) / kSchedHidden, k = (i - kW2) % kSchedHidden;
    return kW2 + k * kSchedHidden + j;
  }
  if (i >= kW3 && i < kB3) {
    const int a = (i - kW3) / kSchedHidden, k = (i - kW3) % kSchedHidden;
    return kW3 + k * kSchedArms + a;
  }
  return i;
}

// Softmax over lanes 0..8: returns p on output lanes, 0 elsewhere; *best and
// *pbest receive the argmax (lowest lane on ties) and its probability.
__device__ __forceinline__ float softmax9(float z, uint32_t lane, int *best, float *pbest) {
  const bool out_lane = lane < (uint32_t)kSchedArms;
  float m = out_lane ? z : -INFINITY;
  int idx = out_lane ? (int)lane : 1 << 20;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const float om = __shfl_xor_sync(kFullMask, m, d);
    const int oi = __shfl_xor_sync(kFullMask, idx, d);
    if (om > m || (om == m && oi < idx)) {
      m = om;
      idx = oi;
    }
  }
  const float e = out_lane ? expf(z - m) : 0.f;
  float s = e;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(kFullMask, s, d);
  *best = idx;
  *pbest = 1.f / s;  // exp(0) / sum
  return e / s;
}

// One warp: the arm for the level whose counters are c (kFallbackArm without
// a model, on an empty frontier or below min_conf).  Lane 0 stores it in
// st->arm and the level record.
template <bool TRANSPOSED>
__device__ __forceinline__ int sched_pick_warp(BfsDevState *st, const LevelCounters &c,
                                               const float *__restrict__ w, float min_conf,
                                               SchedGraphConst gc) {
  const uint32_t lane = threadIdx.x & 31u;
  int arm = kFallbackArm;
  if (w != nullptr && c.F > 0) {
    float x[kSchedIn];
    level_features(c, st->n_cols, gc, x);
    float h1, h2, pbest;
    int best;
    const float z = mlp_forward<TRANSPOSED>(w, x, lane, &h1, &h2);
    softmax9(z, lane, &best, &pbest);
    arm = (pbest >= min_conf) ? best : kFallbackArm;
  }
  if (lane == 0) {
    st->arm = arm;
    if (c.lvl < st->rec_cap) st->rec_arm[c.lvl] = arm;
  }
  return arm;
}

}  // namespace bfsgb
