// bfs_sched.h -- learned per-level scheduler, engine-facing part.
#pragma once
#include <cuda_runtime.h>

#include "bfs_internal.h"

namespace bfsgb {

constexpr int kSchedIn = BFS_SCHED_INPUTS;
constexpr int kSchedHidden = 32;
constexpr int kSchedArms = BFS_SCHED_ARMS;
constexpr int kSchedParams = BFS_SCHED_PARAMS;
constexpr int kFallbackArm = 1;  // LLB, 256 threads: the reference's fixed choice

// Weight offsets in the flat parameter vector.
constexpr int kW1 = 0;
constexpr int kB1 = kW1 + kSchedHidden * kSchedIn;
constexpr int kW2 = kB1 + kSchedHidden;
constexpr int kB2 = kW2 + kSchedHidden * kSchedHidden;
constexpr int kW3 = kB2 + kSchedHidden;
constexpr int kB3 = kW3 + kSchedArms * kSchedHidden;
static_assert(kB3 + kSchedArms == kSchedParams, "parameter layout");

// Graph-level feature constants.
struct SchedGraphConst {
  float diam;        // diameter estimate
  float avg_deg_x;   // x4 feature
};

struct SchedModel {
  float *d_w = nullptr;     // kSchedParams floats on the device (null: untrained)
  float min_conf = 0.f;     // below this top probability use kFallbackArm
};

SchedGraphConst sched_graph_const(uint32_t n_cols, uint64_t nnz);

// Kernel (one warp) of the host-driven level loop: reads the level's
// features from the device state, picks an arm and stores it in st->arm and
// st->rec_arm[lvl].
// Arguments: (BfsDevState*, const float* w, float min_conf, SchedGraphConst)
const void *sched_kernel_fn();

}  // namespace bfsgb
