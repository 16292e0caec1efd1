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

__device__ __forceinline__ void level_features(const BfsDevState *st, SchedGraphConst gc,
                                               float x[kSchedIn]) {
  x[0] = log2f(1.f + (float)st->F) / 32.f;
  x[1] = log2f(1.f + (float)st->EF) / 32.f;
  x[2] = 1.f - (float)st->reached / (float)st->n_cols;
  x[3] = fminf((float)st->lvl / gc.diam, 8.f) / 8.f;
  x[4] = gc.avg_deg_x;
}

// Forward pass of one sample by one warp.  Returns this lane's output logit
// (meaningful on lanes < 9) and the lane's hidden activations.
__device__ __forceinline__ float mlp_forward(const float *__restrict__ w,
                                             const float x[kSchedIn], uint32_t lane,
                                             float *h1_out, float *h2_out) {
  float a = w[kB1 + lane];
#pragma unroll
  for (int i = 0; i < kSchedIn; i++) a = fmaf(w[kW1 + lane * kSchedIn + i], x[i], a);
  const float h1 = fmaxf(a, 0.f);
  float b = w[kB2 + lane];
#pragma unroll 8
  for (int k = 0; k < kSchedHidden; k++)
    b = fmaf(w[kW2 + lane * kSchedHidden + k], __shfl_sync(kFullMask, h1, k), b);
  const float h2 = fmaxf(b, 0.f);
  const bool out_lane = lane < (uint32_t)kSchedArms;
  float c = out_lane ? w[kB3 + lane] : 0.f;
#pragma unroll 8
  for (int k = 0; k < kSchedHidden; k++) {
    const float hk = __shfl_sync(kFullMask, h2, k);
    if (out_lane) c = fmaf(w[kW3 + lane * kSchedHidden + k], hk, c);
  }
  *h1_out = h1;
  *h2_out = h2;
  return c;
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

// One warp: the arm for the state's current level (kFallbackArm without a
// model, on an empty frontier or below min_conf).  Lane 0 stores it in
// st->arm and the level record.
__device__ __forceinline__ int sched_pick_warp(BfsDevState *st, const float *__restrict__ w,
                                               float min_conf, SchedGraphConst gc) {
  const uint32_t lane = threadIdx.x & 31u;
  int arm = kFallbackArm;
  if (w != nullptr && st->F > 0) {
    float x[kSchedIn];
    level_features(st, gc, x);
    float h1, h2, pbest;
    int best;
    const float z = mlp_forward(w, x, lane, &h1, &h2);
    softmax9(z, lane, &best, &pbest);
    arm = (pbest >= min_conf) ? best : kFallbackArm;
  }
  if (lane == 0) {
    st->arm = arm;
    if (st->lvl < st->rec_cap) st->rec_arm[st->lvl] = arm;
  }
  return arm;
}

}  // namespace bfsgb
