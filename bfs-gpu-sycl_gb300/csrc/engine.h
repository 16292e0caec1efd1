// engine.h -- the graph handle and engine-internal hooks.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <vector>

#include "bfs_internal.h"

namespace bfsgb {

struct GraphEntry {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

struct SchedModel;
struct HubLayout;

// Hooks of the host-driven level loop: `choose` picks the explore arm of a
// level (learned scheduler, recorder), `before`/`after` bracket the explore
// launch (per-level timing).  Any of them may be null.
struct LevelTimer {
  void *ctx = nullptr;
  int (*choose)(void *ctx, bfs_graph *g, uint32_t level, uint32_t F, uint32_t EF) = nullptr;
  void (*before)(void *ctx, bfs_graph *g, uint32_t level, int arm) = nullptr;
  void (*after)(void *ctx, bfs_graph *g, uint32_t level, int arm) = nullptr;
};

// after_launch (optional) runs once the BFS is queued on the handle's stream
// and before the call waits for it: work issued there (e.g. copies on another
// stream) is queued ahead of the run's final state read.
bfs_status run_device_impl(bfs_graph *g, uint32_t root, const bfs_options *opts,
                           int32_t *levels_dev, int32_t *parents_dev, bfs_stats *stats,
                           LevelTimer *timer,
                           const std::function<bfs_status()> *after_launch = nullptr);
// Launches one explore kernel on the handle's stream for a frontier of F
// entries and EF edges; persistent = full persistent grid (as in the graph
// loop) instead of a grid sized to the frontier.
cudaError_t launch_explore(bfs_graph *g, int arm, int ipt, int sm_factor, uint32_t F,
                           uint32_t EF, bool persistent);
// Builds the hub layout the handle's request asks for (once per request).
bfs_status ensure_hub(bfs_graph *g);
// Default hub prefix (vertices) and the smallest level (frontier edges) for
// which the explore kernel loads it: a 32 KiB shared-memory bitmap (larger
// prefixes take L1 capacity that the remaining bitmap probes need), loaded by
// every block, pays off once the level has millions of edges.
constexpr uint32_t kHubDefaultVertices = 1u << 18;
constexpr uint32_t kHubMinEdges = 1u << 21;
void free_sched(bfs_graph *g);   // bfs_sched.cu
void free_msbfs(bfs_graph *g);   // msbfs.cu

}  // namespace bfsgb

struct MsWorkspace;

struct bfs_graph {
  int device = 0;
  int num_sms = 0;
  uint32_t *indptr = nullptr;
  uint32_t *inds = nullptr;
  bool owns_csc = false;
  uint32_t n_rows = 0, n_cols = 0;
  uint64_t nnz = 0;
  uint32_t words = 0;
  void *ws = nullptr;  // bitmaps, queues, per-level records
  size_t ws_bytes = 0;
  size_t bitmap_bytes = 0;
  bfsgb::BfsDevState tmpl{};  // host template of the device state
  bfsgb::BfsDevState *d_st = nullptr;
  bfsgb::BfsDevState *h_st = nullptr;  // pinned mirror
  int32_t *d_out_levels = nullptr;     // scratch outputs of bfs_run
  int32_t *d_out_parents = nullptr;
  int32_t *d_ring[2][2] = {};          // bfs_run_roots: [slot][levels, parents]
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // bfs_run_roots: device-to-host copies
  cudaEvent_t ev_ready = nullptr, ev_copied[2] = {nullptr, nullptr};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t lvl_ev[3] = {nullptr, nullptr, nullptr};  // per-level kernel timing
  float *prof_explore = nullptr;  // host arrays filled by the host loop (record == 2)
  float *prof_gen = nullptr;
  int occ[2][bfsgb::kNumArms] = {};  // blocks per SM, [ipt == 8][arm]
  int occ_any[2] = {};                // blocks per SM of explore_any, [ipt == 8]
  int lg_grid[2] = {0, 0};  // level generation, without / with parents
  bool l2_pinned = false;
  bool use_l2_pin = true;
  bool run_parents = false;  // current run records parents
  cudaAccessPolicyWindow l2_window{};
  std::map<int, bfsgb::GraphEntry> graphs;
  int32_t host_arms[BFS_MAX_RECORDED_LEVELS] = {};
  uint32_t host_launches = 0;
  bfsgb::SchedModel *sched = nullptr;
  MsWorkspace *ms = nullptr;  // multi-source BFS workspace (lazy)
  // hub layout of the single-root path (hub_layout.cu), built on the first
  // run that wants it; hub_request: -1 = automatic size, 0 = off, else the
  // prefix size in vertices
  bfsgb::HubLayout *hub = nullptr;
  int64_t hub_request = -1;
  uint32_t hub_max = 0;        // largest prefix the device's shared memory holds
  uint32_t hub_min_edges = 0;  // level size from which explore loads it (0: automatic)
  uint32_t hub_built_for = 0;  // the request the current layout was built for
  uint32_t hub_gen = 0;        // bumped whenever the layout is rebuilt or freed
  bool hub_tried = false;
};
