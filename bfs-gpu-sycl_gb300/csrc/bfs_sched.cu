// bfs_sched.cu -- learned per-level scheduler: features, MLP inference and
// training kernels, per-level recorder.
//
// The reference chooses its load-balancing form and work-group size once, at
// compile time (src/CMakeLists.txt:10-11, run_bfs_gpu.hpp:195, 403, 493).
// This engine chooses per level among 9 arms ({LLB, GLB, SLB} x {128, 256,
// 512} threads) with a 5 -> 32 -> 32 -> 9 FP32 MLP.
//
//   inference  one warp: lane j owns hidden unit j of both hidden layers;
//              layer inputs are broadcast with shuffles; lanes 0..8 own the
//              output logits; argmax and softmax confidence by warp
//              reductions.  It runs as a kernel node inside the CUDA-graph
//              level loop and sets the switch node that selects the explore
//              kernel, so scheduling needs no host round trip.
//   training   full-batch Adam (Kingma & Ba, ICLR 2015).  A warp processes
//              samples with the same lane layout and keeps its gradient
//              partial sums in registers (dW2 row per lane, dW3 column per
//              lane), then adds them to the global gradient once.  Loss per
//              sample: sum_a softmax(z)_a * c_a with c_a = (t_a - t_best) /
//              t_ref, the expected excess explore time; its gradient is
//              dL/dz_a = p_a * (c_a - sum_b p_b c_b).
//   recorder   runs a BFS in the host loop; on every level it snapshots the
//              visited bitmap, then times each arm's explore kernel from the
//              same state (restoring the bitmap between runs).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "kernels.h"
#include "bfs_sched.h"
#include "dev_alloc.h"
#include "bfs_sched_dev.cuh"

namespace bfsgb {

SchedGraphConst sched_graph_const(uint32_t n_cols, uint64_t nnz) {
  SchedGraphConst c;
  const double avg = n_cols ? (double)nnz / (double)n_cols : 0.0;
  const double d = std::log((double)std::max<uint32_t>(n_cols, 2)) / std::log(std::max(avg, 2.0));
  c.diam = (float)std::max(2.0, d);
  c.avg_deg_x = (float)(std::log2(1.0 + avg) / 8.0);
  return c;
}

__global__ void sched_kernel(BfsDevState *st, const float *__restrict__ w, float min_conf,
                             SchedGraphConst gc) {
  if (threadIdx.x >= 32) return;
  sched_pick_warp<false>(st, level_counters(st), w, min_conf, gc);
  if (threadIdx.x == 0) st->launches += 1;
}

__global__ void features_kernel(const BfsDevState *st, SchedGraphConst gc, float *out) {
  if (threadIdx.x == 0) {
    float x[kSchedIn];
    level_features(level_counters(st), st->n_cols, gc, x);
    for (int i = 0; i < kSchedIn; i++) out[i] = x[i];
  }
}

__global__ void predict_kernel(const float *__restrict__ w, const float *__restrict__ X,
                               uint32_t n, int32_t *arms, float *conf) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t s = gwarp; s < n; s += nwarps) {
    float x[kSchedIn];
#pragma unroll
    for (int i = 0; i < kSchedIn; i++) x[i] = X[(size_t)s * kSchedIn + i];
    float h1, h2, pbest;
    int best;
    const float z = mlp_forward<false>(w, x, lane, &h1, &h2);
    softmax9(z, lane, &best, &pbest);
    if (lane == 0) {
      if (arms) arms[s] = best;
      if (conf) conf[s] = pbest;
    }
  }
}

// One full-batch gradient of the expected-excess-time loss (scaled by 1/n).
__global__ void __launch_bounds__(256) train_grad_kernel(const float *__restrict__ w,
                                                         const float *__restrict__ X,
                                                         const float *__restrict__ Cst,
                                                         uint32_t n, float inv_n, float *grad,
                                                         float *loss) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool out_lane = lane < (uint32_t)kSchedArms;
  float g_w1[kSchedIn] = {}, g_b1 = 0.f, g_w2[kSchedHidden] = {}, g_b2 = 0.f;
  float g_w3[kSchedArms] = {}, g_b3 = 0.f, l_acc = 0.f;
  for (uint32_t s = gwarp; s < n; s += nwarps) {
    float x[kSchedIn];
#pragma unroll
    for (int i = 0; i < kSchedIn; i++) x[i] = X[(size_t)s * kSchedIn + i];
    float h1, h2, pbest;
    int best;
    const float z = mlp_forward<false>(w, x, lane, &h1, &h2);
    const float p = softmax9(z, lane, &best, &pbest);
    const float c = out_lane ? Cst[(size_t)s * kSchedArms + lane] : 0.f;
    float ec = p * c;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) ec += __shfl_xor_sync(kFullMask, ec, d);
    l_acc += ec;
    const float dz = out_lane ? p * (c - ec) * inv_n : 0.f;
    g_b3 += dz;
    // output layer: lane k owns column k of W3
    float dh2 = 0.f;
#pragma unroll
    for (int a = 0; a < kSchedArms; a++) {
      const float dza = __shfl_sync(kFullMask, dz, a);
      g_w3[a] = fmaf(dza, h2, g_w3[a]);
      dh2 = fmaf(w[kW3 + a * kSchedHidden + lane], dza, dh2);
    }
    dh2 = h2 > 0.f ? dh2 : 0.f;
    g_b2 += dh2;
    // hidden layer 2: lane j owns row j of W2
    float dh1 = 0.f;
#pragma unroll 8
    for (int k = 0; k < kSchedHidden; k++) {
      g_w2[k] = fmaf(dh2, __shfl_sync(kFullMask, h1, k), g_w2[k]);
      dh1 = fmaf(w[kW2 + k * kSchedHidden + lane], __shfl_sync(kFullMask, dh2, k), dh1);
    }
    dh1 = h1 > 0.f ? dh1 : 0.f;
    g_b1 += dh1;
#pragma unroll
    for (int i = 0; i < kSchedIn; i++) g_w1[i] = fmaf(dh1, x[i], g_w1[i]);
  }
  if (gwarp >= n) return;  // warp saw no sample
#pragma unroll
  for (int i = 0; i < kSchedIn; i++) atomicAdd(grad + kW1 + lane * kSchedIn + i, g_w1[i]);
  atomicAdd(grad + kB1 + lane, g_b1);
#pragma unroll 8
  for (int k = 0; k < kSchedHidden; k++) atomicAdd(grad + kW2 + lane * kSchedHidden + k, g_w2[k]);
  atomicAdd(grad + kB2 + lane, g_b2);
#pragma unroll
  for (int a = 0; a < kSchedArms; a++) atomicAdd(grad + kW3 + a * kSchedHidden + lane, g_w3[a]);
  if (out_lane) atomicAdd(grad + kB3 + lane, g_b3);
  if (lane == 0) atomicAdd(loss, l_acc * inv_n);
}

__global__ void adam_kernel(float *w, float *grad, float *m, float *v, float lr, float beta1,
                            float beta2, float eps, float corr1, float corr2, int n) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const float g = grad[p];
    const float mp = beta1 * m[p] + (1.f - beta1) * g;
    const float vp = beta2 * v[p] + (1.f - beta2) * g * g;
    m[p] = mp;
    v[p] = vp;
    w[p] -= lr * (mp * corr1) / (sqrtf(vp * corr2) + eps);
    grad[p] = 0.f;
  }
}

const void *sched_kernel_fn() { return (const void *)sched_kernel; }

void free_sched(bfs_graph *g) {
  if (!g->sched) return;
  cudaFree(g->sched->d_w);
  delete g->sched;
  g->sched = nullptr;
}

// ---- recorder ---------------------------------------------------------------

namespace {

struct RecCtx {
  int ipt = 4;
  int reps = 3;
  uint32_t *backup = nullptr;
  float *d_feat = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SchedGraphConst gc{};
  bfs_level_sample *out = nullptr;
  uint32_t max = 0, n = 0;
  bfs_status err = BFS_OK;
  std::string msg;
};

#define RK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) {                                            \
      c->err = BFS_ERR_CUDA;                                            \
      c->msg = std::string(#call) + ": " + cudaGetErrorString(e_);      \
      return kFallbackArm;                                              \
    }                                                                   \
  } while (0)

int record_choose(void *ctx, bfs_graph *g, uint32_t level, uint32_t F, uint32_t EF) {
  RecCtx *c = (RecCtx *)ctx;
  if (c->err != BFS_OK || c->n >= c->max) return kFallbackArm;
  bfs_level_sample &smp = c->out[c->n];
  std::memset(&smp, 0, sizeof(smp));
  smp.level = level;
  smp.frontier = F;
  smp.edges = EF;
  const size_t vbytes = (size_t)g->words * 4;
  features_kernel<<<1, 32, 0, g->stream>>>(g->d_st, c->gc, c->d_feat);
  RK(cudaGetLastError());
  RK(cudaMemcpyAsync(smp.features, c->d_feat, sizeof(smp.features), cudaMemcpyDeviceToHost,
                     g->stream));
  RK(cudaMemcpyAsync(c->backup, g->tmpl.vis, vbytes, cudaMemcpyDeviceToDevice, g->stream));
  for (int arm = 0; arm < kNumArms; arm++) {
    float best = INFINITY;
    for (int r = 0; r < c->reps; r++) {
      RK(cudaMemcpyAsync(g->tmpl.vis, c->backup, vbytes, cudaMemcpyDeviceToDevice, g->stream));
      RK(cudaEventRecord(c->e0, g->stream));
      RK(launch_explore(g, arm, c->ipt, 0, F, EF, true));
      RK(cudaEventRecord(c->e1, g->stream));
      RK(cudaEventSynchronize(c->e1));
      float ms = 0.f;
      RK(cudaEventElapsedTime(&ms, c->e0, c->e1));
      best = std::min(best, ms);
    }
    smp.arm_ms[arm] = best;
  }
  RK(cudaMemcpyAsync(g->tmpl.vis, c->backup, vbytes, cudaMemcpyDeviceToDevice, g->stream));
  RK(cudaStreamSynchronize(g->stream));
  c->n++;
  // advance with the fastest arm of this level (the levels do not depend on it)
  int fastest = 0;
  for (int a = 1; a < kNumArms; a++)
    if (smp.arm_ms[a] < smp.arm_ms[fastest]) fastest = a;
  return fastest;
}
#undef RK

}  // namespace

}  // namespace bfsgb

using namespace bfsgb;

#define SK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      rc = fail(e_ == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,    \
                std::string(#call) + ": " + cudaGetErrorString(e_));             \
      goto done;                                                                 \
    }                                                                            \
  } while (0)

extern "C" {

bfs_status bfs_sched_record(bfs_graph *g, uint32_t root, int32_t ipt, int32_t reps,
                            bfs_level_sample *out, uint32_t max_levels, uint32_t *n_out) {
  if (!g || !out || !n_out) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (reps < 1 || reps > 64) return fail(BFS_ERR_INVALID_ARG, "reps must be 1..64");
  if (ipt == 0) ipt = 4;
  if (ipt != 4 && ipt != 8) return fail(BFS_ERR_INVALID_ARG, "ipt must be 4 or 8");
  *n_out = 0;
  bfs_status rc = BFS_OK;
  RecCtx ctx;
  ctx.ipt = ipt;
  ctx.reps = reps;
  ctx.out = out;
  ctx.max = max_levels;
  ctx.gc = sched_graph_const(g->n_cols, g->nnz);
  int32_t *levels = nullptr;
  LevelTimer timer;
  bfs_options o;
  SK(cudaSetDevice(g->device));
  SK(dev_malloc(&ctx.backup, (size_t)g->words * 4));
  SK(dev_malloc(&ctx.d_feat, sizeof(float) * kSchedIn));
  SK(dev_malloc(&levels, sizeof(int32_t) * (size_t)g->n_cols));
  SK(cudaEventCreate(&ctx.e0));
  SK(cudaEventCreate(&ctx.e1));
  timer.ctx = &ctx;
  timer.choose = record_choose;
  bfs_options_default(&o);
  o.loop = BFS_LOOP_HOST;
  o.ipt = ipt;
  o.l2_pin = 1;
  rc = run_device_impl(g, root, &o, levels, nullptr, nullptr, &timer);
  if (rc == BFS_OK && ctx.err != BFS_OK) rc = fail(ctx.err, ctx.msg);
  *n_out = ctx.n;
done:
  cudaFree(ctx.backup);
  cudaFree(ctx.d_feat);
  cudaFree(levels);
  if (ctx.e0) cudaEventDestroy(ctx.e0);
  if (ctx.e1) cudaEventDestroy(ctx.e1);
  return rc;
}

bfs_status bfs_sched_train(const bfs_level_sample *samples, uint32_t n,
                           const bfs_sched_train_opts *opts, float *weights_out,
                           float *final_loss) {
  if (!samples || !weights_out || n == 0) return fail(BFS_ERR_INVALID_ARG, "no samples");
  bfs_sched_train_opts o{1500, 3e-3f, 1};
  if (opts) {
    o = *opts;
    if (o.epochs == 0) o.epochs = 1500;
    if (!(o.lr > 0.f)) o.lr = 3e-3f;
  }
  // costs: excess time over the level's best arm, in units of the mean best
  std::vector<float> X((size_t)n * kSchedIn), Cst((size_t)n * kSchedArms);
  double tref = 0;
  for (uint32_t s = 0; s < n; s++) {
    float best = samples[s].arm_ms[0];
    for (int a = 1; a < kSchedArms; a++) best = std::min(best, samples[s].arm_ms[a]);
    tref += best;
  }
  tref = std::max(tref / n, 1e-6);
  for (uint32_t s = 0; s < n; s++) {
    float best = samples[s].arm_ms[0];
    for (int a = 1; a < kSchedArms; a++) best = std::min(best, samples[s].arm_ms[a]);
    for (int i = 0; i < kSchedIn; i++) X[(size_t)s * kSchedIn + i] = samples[s].features[i];
    for (int a = 0; a < kSchedArms; a++)
      Cst[(size_t)s * kSchedArms + a] = (float)((samples[s].arm_ms[a] - best) / tref);
  }
  // He-uniform initialisation from the counter-based hash
  std::vector<float> w0(kSchedParams, 0.f);
  {
    const uint64_t sm = mix64(o.seed ^ 0x7363686564ull);  // "sched"
    auto unif = [&](uint64_t i) { return (float)((mix64(sm + i) >> 11) * (1.0 / 9007199254740992.0)); };
    auto fill = [&](int off, int cnt, int fan_in, float gain) {
      const float lim = gain * std::sqrt(6.f / (float)fan_in);
      for (int i = 0; i < cnt; i++) w0[off + i] = (2.f * unif(off + i) - 1.f) * lim;
    };
    fill(kW1, kSchedHidden * kSchedIn, kSchedIn, 1.f);
    fill(kW2, kSchedHidden * kSchedHidden, kSchedHidden, 1.f);
    fill(kW3, kSchedArms * kSchedHidden, kSchedHidden, 0.1f);
  }
  bfs_status rc = BFS_OK;
  float *d_w = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr, *d_X = nullptr,
        *d_C = nullptr, *d_loss = nullptr;
  cudaStream_t st = nullptr;
  const int blocks = (int)std::min<uint32_t>(1024, (n + 7) / 8);
  const double b1 = 0.9, b2 = 0.999;
  float loss = 0.f;
  SK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  SK(dev_malloc(&d_w, sizeof(float) * kSchedParams));
  SK(dev_malloc(&d_g, sizeof(float) * kSchedParams));
  SK(dev_malloc(&d_m, sizeof(float) * kSchedParams));
  SK(dev_malloc(&d_v, sizeof(float) * kSchedParams));
  SK(dev_malloc(&d_X, sizeof(float) * X.size()));
  SK(dev_malloc(&d_C, sizeof(float) * Cst.size()));
  SK(dev_malloc(&d_loss, sizeof(float)));
  SK(cudaMemcpyAsync(d_w, w0.data(), sizeof(float) * kSchedParams, cudaMemcpyHostToDevice, st));
  SK(cudaMemsetAsync(d_g, 0, sizeof(float) * kSchedParams, st));
  SK(cudaMemsetAsync(d_m, 0, sizeof(float) * kSchedParams, st));
  SK(cudaMemsetAsync(d_v, 0, sizeof(float) * kSchedParams, st));
  SK(cudaMemcpyAsync(d_X, X.data(), sizeof(float) * X.size(), cudaMemcpyHostToDevice, st));
  SK(cudaMemcpyAsync(d_C, Cst.data(), sizeof(float) * Cst.size(), cudaMemcpyHostToDevice, st));
  for (uint32_t ep = 1; ep <= o.epochs; ep++) {
    SK(cudaMemsetAsync(d_loss, 0, sizeof(float), st));
    train_grad_kernel<<<blocks, 256, 0, st>>>(d_w, d_X, d_C, n, 1.f / (float)n, d_g, d_loss);
    SK(cudaGetLastError());
    const float c1 = (float)(1.0 / (1.0 - std::pow(b1, (double)ep)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(b2, (double)ep)));
    adam_kernel<<<(kSchedParams + 255) / 256, 256, 0, st>>>(d_w, d_g, d_m, d_v, o.lr, (float)b1,
                                                          (float)b2, 1e-8f, c1, c2, kSchedParams);
    SK(cudaGetLastError());
  }
  SK(cudaMemcpyAsync(weights_out, d_w, sizeof(float) * kSchedParams, cudaMemcpyDeviceToHost, st));
  SK(cudaMemcpyAsync(&loss, d_loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  SK(cudaStreamSynchronize(st));
  if (final_loss) *final_loss = loss;
done:
  cudaFree(d_w);
  cudaFree(d_g);
  cudaFree(d_m);
  cudaFree(d_v);
  cudaFree(d_X);
  cudaFree(d_C);
  cudaFree(d_loss);
  if (st) cudaStreamDestroy(st);
  return rc;
}

bfs_status bfs_sched_predict(const float *weights, const float *features, uint32_t n,
                             int32_t *arms_out, float *conf_out) {
  if (!weights || !features) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (n == 0) return BFS_OK;
  bfs_status rc = BFS_OK;
  float *d_w = nullptr, *d_X = nullptr, *d_conf = nullptr;
  int32_t *d_arms = nullptr;
  SK(dev_malloc(&d_w, sizeof(float) * kSchedParams));
  SK(dev_malloc(&d_X, sizeof(float) * (size_t)n * kSchedIn));
  SK(dev_malloc(&d_arms, sizeof(int32_t) * n));
  SK(dev_malloc(&d_conf, sizeof(float) * n));
  SK(cudaMemcpy(d_w, weights, sizeof(float) * kSchedParams, cudaMemcpyHostToDevice));
  SK(cudaMemcpy(d_X, features, sizeof(float) * (size_t)n * kSchedIn, cudaMemcpyHostToDevice));
  predict_kernel<<<std::min<uint32_t>(1024, (n + 7) / 8), 256>>>(d_w, d_X, n, d_arms, d_conf);
  SK(cudaGetLastError());
  if (arms_out) SK(cudaMemcpy(arms_out, d_arms, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  if (conf_out) SK(cudaMemcpy(conf_out, d_conf, sizeof(float) * n, cudaMemcpyDeviceToHost));
done:
  cudaFree(d_w);
  cudaFree(d_X);
  cudaFree(d_arms);
  cudaFree(d_conf);
  return rc;
}

bfs_status bfs_sched_attach(bfs_graph *g, const float *weights, float min_confidence) {
  if (!g) return fail(BFS_ERR_INVALID_ARG, "null graph");
  if (cudaSetDevice(g->device) != cudaSuccess) return fail(BFS_ERR_CUDA, "cudaSetDevice");
  if (!weights) {
    free_sched(g);
    return BFS_OK;
  }
  for (int i = 0; i < kSchedParams; i++)
    if (!std::isfinite(weights[i])) return fail(BFS_ERR_INVALID_ARG, "non-finite weight");
  if (!g->sched) g->sched = new SchedModel();
  if (!g->sched->d_w) {
    cudaError_t e = dev_malloc(&g->sched->d_w, sizeof(float) * kSchedParams);
    if (e != cudaSuccess) return fail(BFS_ERR_OOM, "scheduler weights");
  }
  if (cudaMemcpy(g->sched->d_w, weights, sizeof(float) * kSchedParams, cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return fail(BFS_ERR_CUDA, "scheduler weight upload");
  g->sched->min_conf = min_confidence;
  return BFS_OK;
}

}  // extern "C"
