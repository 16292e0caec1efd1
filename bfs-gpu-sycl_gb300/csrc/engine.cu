// engine.cu -- graph handles, workspace, level loop and the C ABI run calls.
//
// The reference's GPURun (src/run_bfs_gpu.hpp:534-808) allocates and uploads
// the graph for every run (:620-670), drives the level loop from the host with
// a blocking read-back of the frontier size per level (:682-727) and frees
// everything after each run (:732-746).  Here the graph is uploaded once per
// handle, the workspace lives as long as the handle, and the level loop runs
// on the device: a CUDA graph whose conditional WHILE node repeats
// {explore, level generation} until the last level-generation block reports
// an empty frontier.  A host-driven loop with the reference's per-level
// read-back is kept as BFS_LOOP_HOST (it is also what the per-level recorder
// of the learned scheduler uses).  bfs_run_roots runs the reference's
// num_runs loop in one call: each run's level array goes to the host on a
// second stream while the next run proceeds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "bfs_internal.h"
#include "dev_alloc.h"
#include "engine.h"
#include "kernels.h"
#include "bfs_sched.h"
#include "hub_layout.h"

namespace bfsgb {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
bfs_status fail(bfs_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      return fail(e_ == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,    \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
    }                                                                              \
  } while (0)

namespace {

std::mutex g_l2_mutex;
int g_l2_users = 0;
size_t g_l2_prev_limit = 0;

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

// ---- handle lifetime ---------------------------------------------------------

static void free_workspace(bfs_graph *g) {
  for (auto &kv : g->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  g->graphs.clear();
  cudaFree(g->ws);
  g->ws = nullptr;
  cudaFree(g->d_st);
  g->d_st = nullptr;
  cudaFree(g->d_out_levels);
  cudaFree(g->d_out_parents);
  g->d_out_levels = g->d_out_parents = nullptr;
  for (auto &slot : g->d_ring)
    for (auto &p : slot) {
      cudaFree(p);
      p = nullptr;
    }
  if (g->ev_ready) cudaEventDestroy(g->ev_ready);
  g->ev_ready = nullptr;
  for (auto &e : g->ev_copied) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
  g->copy_stream = nullptr;
  if (g->h_st) cudaFreeHost(g->h_st);
  g->h_st = nullptr;
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  g->ev0 = g->ev1 = nullptr;
  for (auto &e : g->lvl_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  if (g->l2_pinned) {
    std::lock_guard<std::mutex> lk(g_l2_mutex);
    if (--g_l2_users == 0) {
      cudaCtxResetPersistingL2Cache();
      cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, g_l2_prev_limit);
      cudaGetLastError();
    }
    g->l2_pinned = false;
  }
  if (g->stream) cudaStreamDestroy(g->stream);
  g->stream = nullptr;
}

static bfs_status setup_workspace(bfs_graph *g) {
  CK(cudaGetDevice(&g->device));
  CK(cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device));
  CK(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&g->ev0));
  CK(cudaEventCreate(&g->ev1));
  for (auto &e : g->lvl_ev) CK(cudaEventCreate(&e));
  g->words = (uint32_t)align_up(((size_t)g->n_cols + 31) / 32, 32);
  // one allocation: bitmaps (vis, prev), working levels (one byte per id),
  // four queue arrays x 2, record arrays
  const size_t bm = align_up((size_t)g->words * 4, 256);
  const size_t l8 = align_up((size_t)g->words * 32, 256);
  const size_t nq = std::max<size_t>(g->n_rows, 1);
  const size_t q4 = align_up(nq * 4, 256), qp4 = align_up((nq + 1) * 4, 256);
  const size_t rec = align_up((size_t)BFS_MAX_RECORDED_LEVELS * 4, 256);
  g->ws_bytes = 2 * bm + l8 + 2 * (3 * q4 + qp4) + 4 * rec;
  CK(dev_malloc(&g->ws, g->ws_bytes));
  char *p = (char *)g->ws;
  BfsDevState &s = g->tmpl;
  std::memset(&s, 0, sizeof(s));
  s.indptr = g->indptr;
  s.inds = g->inds;
  s.nnz = (uint32_t)g->nnz;
  s.inds_off = (uint32_t)((reinterpret_cast<uintptr_t>(g->inds) & 15u) >> 2);
  s.n_rows = g->n_rows;
  s.n_cols = g->n_cols;
  s.words = g->words;
  s.vis = (uint32_t *)p; p += bm;
  s.prev = (uint32_t *)p; p += bm;
  s.lv8 = (uint8_t *)p; p += l8;
  for (int b = 0; b < 2; b++) {
    s.qb[b] = (uint32_t *)p; p += q4;
    s.qd[b] = (uint32_t *)p; p += q4;
    s.qc[b] = (uint32_t *)p; p += qp4;
    s.qv[b] = (uint32_t *)p; p += q4;
  }
  s.rec_frontier = (uint32_t *)p; p += rec;
  s.rec_edges = (uint32_t *)p; p += rec;
  s.rec_arm = (int32_t *)p; p += rec;
  s.rec_ran = (int32_t *)p; p += rec;
  s.rec_cap = BFS_MAX_RECORDED_LEVELS;
  s.fixed_arm = 0;
  s.level_cap = g->n_cols + 1u;
  g->bitmap_bytes = 2 * bm;
  CK(dev_malloc(&g->d_st, sizeof(BfsDevState)));
  CK(cudaMallocHost(&g->h_st, sizeof(BfsDevState)));

  // persistent grid sizes (occupancy x SMs)
  for (int u = 0; u < 2; u++) {
    for (int arm = 0; arm < kNumArms; arm++) {
      int occ = 0;
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &occ, explore_kernel_fn(arm, u ? 8 : 4, false), arm_block(arm), 0));
      g->occ[u][arm] = std::max(occ, 1);
    }
    int occ = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, explore_any_kernel_fn(u ? 8 : 4, false),
                                                     kAnyBlock, 0));
    g->occ_any[u] = std::max(occ, 1);
  }
  for (int par = 0; par < 2; par++) {
    const void *fn = levelgen_kernel_fn(par != 0);
    const size_t smem = levelgen_smem(par != 0);
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ_lg = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_lg, fn, kLevelgenBlock, smem));
    g->lg_grid[par] = g->num_sms * std::max(occ_lg, 1);
  }
  // explore_any takes the hub prefix in dynamic shared memory, up to what
  // the device allows a block beside the kernel's own static arrays
  size_t static_max = 0;
  for (int u = 0; u < 2; u++)
    for (int par = 0; par < 2; par++) {
      cudaFuncAttributes fa;
      CK(cudaFuncGetAttributes(&fa, explore_any_kernel_fn(u ? 8 : 4, par != 0)));
      static_max = std::max(static_max, fa.sharedSizeBytes);
    }
  g->hub_max = hub_max_vertices(g, static_max);
  if (g->hub_max > 0) {
    for (int u = 0; u < 2; u++)
      for (int par = 0; par < 2; par++)
        CK(cudaFuncSetAttribute(explore_any_kernel_fn(u ? 8 : 4, par != 0),
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(g->hub_max / 8)));
  }

  // L2 access-policy window over the two visited bitmaps
  int max_persist = 0, max_window = 0;
  cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, g->device);
  cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, g->device);
  cudaGetLastError();
  if (max_persist > 0 && max_window > 0) {
    std::lock_guard<std::mutex> lk(g_l2_mutex);
    bool ok = true;
    if (g_l2_users == 0) {
      size_t prev = 0;
      ok = cudaDeviceGetLimit(&prev, cudaLimitPersistingL2CacheSize) == cudaSuccess;
      if (ok) g_l2_prev_limit = prev;
      ok = ok && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)max_persist) ==
                     cudaSuccess;
    }
    if (ok) {
      g_l2_users++;
      g->l2_pinned = true;
      const size_t win = std::min<size_t>(g->bitmap_bytes, (size_t)max_window);
      g->l2_window.base_ptr = (void *)s.vis;
      g->l2_window.num_bytes = win;
      g->l2_window.hitRatio =
          (float)std::min(1.0, (double)max_persist / (double)std::max<size_t>(win, 1));
      g->l2_window.hitProp = cudaAccessPropertyPersisting;
      g->l2_window.missProp = cudaAccessPropertyStreaming;
    }
    cudaGetLastError();
  }
  return BFS_OK;
}

static bfs_status make_graph(const uint32_t *d_indptr, const uint32_t *d_inds,
                             uint32_t n_rows, uint32_t n_cols, uint64_t nnz, bool owns,
                             int validate, bfs_graph **out) {
  bfs_graph *g = new (std::nothrow) bfs_graph();
  if (!g) return fail(BFS_ERR_OOM, "host allocation failed");
  g->indptr = const_cast<uint32_t *>(d_indptr);
  g->inds = const_cast<uint32_t *>(d_inds);
  g->owns_csc = owns;
  g->n_rows = n_rows;
  g->n_cols = n_cols;
  g->nnz = nnz;
  bfs_status rc = setup_workspace(g);
  if (rc == BFS_OK && validate) {
    unsigned long long *bad = nullptr, h_bad = 0;
    cudaError_t e = dev_malloc(&bad, sizeof(*bad));
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(*bad), g->stream);
    if (e == cudaSuccess) e = launch_check_csc(g->indptr, g->inds, n_cols, nnz, bad, g->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&h_bad, bad, sizeof(h_bad), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(bad);
    if (e != cudaSuccess)
      rc = fail(e == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,
                std::string("CSC check: ") + cudaGetErrorString(e));
    else if (h_bad)
      rc = fail(BFS_ERR_GRAPH, "malformed CSC: " + std::to_string(h_bad) +
                                   " bad offsets or destinations");
  }
  if (rc != BFS_OK) {
    free_workspace(g);
    if (!owns) g->indptr = g->inds = nullptr;
    if (owns) {
      cudaFree(g->indptr);
      cudaFree(g->inds);
    }
    delete g;
    return rc;
  }
  *out = g;
  return BFS_OK;
}

static bfs_status check_dims(uint32_t n_rows, uint32_t n_cols, uint64_t nnz) {
  if (n_cols == 0) return fail(BFS_ERR_INVALID_ARG, "n_cols must be > 0");
  if (n_rows > n_cols) return fail(BFS_ERR_INVALID_ARG, "n_rows must be <= n_cols");
  if (n_cols > 0xFFFFF000u) return fail(BFS_ERR_INVALID_ARG, "n_cols too large");
  if (nnz > BFS_MAX_EDGES)
    return fail(BFS_ERR_INVALID_ARG, "nnz must be <= BFS_MAX_EDGES (2^32 - 4096)");
  return BFS_OK;
}

bfs_status graph_from_owned_device(uint32_t *d_indptr, uint32_t *d_inds, uint32_t n_rows,
                                   uint32_t n_cols, uint64_t nnz, bfs_graph **out) {
  bfs_status rc = check_dims(n_rows, n_cols, nnz);
  if (rc != BFS_OK) return rc;
  return make_graph(d_indptr, d_inds, n_rows, n_cols, nnz, true, 0, out);
}

bfs_status graph_download_impl(const bfs_graph *g, bfs_csc_host *out) {
  if (!g || !out) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  std::memset(out, 0, sizeof(*out));
  CK(cudaSetDevice(g->device));
  out->indptr = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)g->n_cols + 1));
  out->inds = (uint32_t *)malloc(sizeof(uint32_t) * (g->nnz ? g->nnz : 1));
  if (!out->indptr || !out->inds) {
    bfs_csc_host_free(out);
    return fail(BFS_ERR_OOM, "host allocation failed");
  }
  CK(cudaMemcpy(out->indptr, g->indptr, sizeof(uint32_t) * ((size_t)g->n_cols + 1),
                cudaMemcpyDeviceToHost));
  if (g->nnz)
    CK(cudaMemcpy(out->inds, g->inds, sizeof(uint32_t) * g->nnz, cudaMemcpyDeviceToHost));
  out->n_rows = g->n_rows;
  out->n_cols = g->n_cols;
  out->nnz = g->nnz;
  return BFS_OK;
}

// ---- launch geometry -----------------------------------------------------------

static int persistent_blocks(const bfs_graph *g, int arm, int sm_factor, int ipt) {
  int per_sm = g->occ[ipt == 8 ? 1 : 0][arm];
  if (sm_factor > 0) per_sm = sm_factor;
  return std::max(1, g->num_sms * per_sm);
}

static int any_blocks(const bfs_graph *g, int ipt) {
  return std::max(1, g->num_sms * g->occ_any[ipt == 8 ? 1 : 0]);
}

// Grid for a host-driven launch with known frontier F (entries) and EF (edges).
static int host_blocks(const bfs_graph *g, int arm, int sm_factor, int ipt, uint32_t F,
                       uint32_t EF) {
  const int B = arm_block(arm);
  uint64_t want;
  if (arm_lb(arm) == BFS_LB_GLB) {
    const uint64_t chunks = ((uint64_t)EF + glb_chunk_edges(ipt) - 1) / glb_chunk_edges(ipt);
    want = (chunks + (B / 32) - 1) / (B / 32);
  } else {
    want = ((uint64_t)F + B - 1) / B;
  }
  return (int)std::max<uint64_t>(
      1, std::min<uint64_t>(want, persistent_blocks(g, arm, sm_factor, ipt)));
}

// Dynamic shared memory of explore_any for the handle's current layout.
static size_t hub_smem(const bfs_graph *g) {
  return g->hub ? (size_t)g->hub->vertices / 8 : 0;
}

cudaError_t launch_explore(bfs_graph *g, int arm, int ipt, int sm_factor, uint32_t F,
                           uint32_t EF, bool persistent) {
  BfsDevState *st = g->d_st;
  if (arm_lb(arm) == BFS_LB_GLB) {
    // GLB runs in explore_any (chunk walk, hub filter): one block per SM
    void *aargs[] = {&st, &arm};
    const int full = any_blocks(g, ipt);
    const int grid = persistent ? full : std::min(full, host_blocks(g, arm, 0, ipt, F, EF));
    return cudaLaunchKernel(explore_any_kernel_fn(ipt, g->run_parents), dim3(grid),
                            dim3(kAnyBlock), aargs, hub_smem(g), g->stream);
  }
  void *args[] = {&st};
  const int grid = persistent ? persistent_blocks(g, arm, sm_factor, ipt)
                              : host_blocks(g, arm, sm_factor, ipt, F, EF);
  return cudaLaunchKernel(explore_kernel_fn(arm, ipt, g->run_parents), dim3(grid),
                          dim3(arm_block(arm)), args, 0, g->stream);
}

static void set_window(const bfs_graph *g, cudaGraphNode_t node) {
  if (!g->l2_pinned || !g->use_l2_pin) return;
  cudaLaunchAttributeValue v;
  std::memset(&v, 0, sizeof(v));
  v.accessPolicyWindow = g->l2_window;
  cudaGraphKernelNodeSetAttribute(node, cudaLaunchAttributeAccessPolicyWindow, &v);
  cudaGetLastError();
}

static cudaError_t add_kernel(cudaGraph_t graph, cudaGraphNode_t *node,
                              const cudaGraphNode_t *deps, size_t ndeps, const void *fn,
                              int grid, int block, void **args, size_t smem = 0) {
  cudaKernelNodeParams kp;
  std::memset(&kp, 0, sizeof(kp));
  kp.func = const_cast<void *>(fn);
  kp.gridDim = dim3(grid);
  kp.blockDim = dim3(block);
  kp.sharedMemBytes = (unsigned)smem;
  kp.kernelParams = args;
  return cudaGraphAddKernelNode(node, graph, deps, ndeps, &kp);
}

// Builds the device-side level loop:
//   fill(levels/parents, bitmaps) -> init(root) -> while(F > 0) {
//     explore -> levelgen (last block sets the while condition) }
// With a fixed arm the explore node is that arm's kernel (explore_any for the
// GLB arms).  With arm < 0 (learned schedule) it is explore_any, which runs
// the arm in st->arm: the scheduler runs inside init (level 0) and inside the
// last block of level generation (the next level), so the loop has no node
// of its own for it.  (A switch node selecting each arm's own kernel was
// measured: about 4.5 us more per level than explore_any's uniform branch.)
static bfs_status build_loop_graph(bfs_graph *g, int arm, int sm_factor, int ipt,
                                   GraphEntry *ge) {
  cudaGraph_t graph = nullptr;
  CK(cudaGraphCreate(&graph, 0));
  ge->graph = graph;
  cudaGraphConditionalHandle cond;
  CK(cudaGraphConditionalHandleCreate(&cond, graph, 0, cudaGraphCondAssignDefault));
  unsigned long long cond_arg = (unsigned long long)cond;
  int one = 1;
  BfsDevState *st = g->d_st;

  cudaGraphNode_t n_fill, n_init, n_while, n_explore, n_lg;
  void *fill_args[] = {&st};  // levels (and parents) to -1, bitmaps cleared
  CK(add_kernel(graph, &n_fill, nullptr, 0, fill_kernel_fn(), g->num_sms * 4, 256, fill_args));
  void *init_args[] = {&st, &cond_arg, &one};
  CK(add_kernel(graph, &n_init, &n_fill, 1, init_kernel_fn(), 1, 32, init_args));

  // cudaGraphNodeParams has no usable default constructor (union members)
  alignas(cudaGraphNodeParams) unsigned char wbuf[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams &wp = *reinterpret_cast<cudaGraphNodeParams *>(wbuf);
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = cond;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  CK(cudaGraphAddNode(&n_while, graph, &n_init, nullptr, 1, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  cudaGraphNode_t n_out;
  CK(add_kernel(graph, &n_out, &n_while, 1, level_out_kernel_fn(), g->num_sms * 8, 256,
                fill_args));

  void *ex_args[] = {&st};
  int arm_arg = arm;  // < 0: the scheduler's arm in st->arm
  void *any_args[] = {&st, &arm_arg};
  if (arm >= 0 && arm_lb(arm) != BFS_LB_GLB) {
    CK(add_kernel(body, &n_explore, nullptr, 0, explore_kernel_fn(arm, ipt, g->run_parents),
                  persistent_blocks(g, arm, sm_factor, ipt), arm_block(arm), ex_args));
  } else {
    CK(add_kernel(body, &n_explore, nullptr, 0, explore_any_kernel_fn(ipt, g->run_parents),
                  any_blocks(g, ipt), kAnyBlock, any_args, hub_smem(g)));
  }
  set_window(g, n_explore);
  void *lg_args[] = {&st, &cond_arg, &one};
  CK(add_kernel(body, &n_lg, &n_explore, 1, levelgen_kernel_fn(g->run_parents),
                g->lg_grid[g->run_parents], kLevelgenBlock, lg_args,
                levelgen_smem(g->run_parents)));
  set_window(g, n_lg);
  CK(cudaGraphInstantiate(&ge->exec, graph, 0));
  return BFS_OK;
}

static bfs_status get_loop_graph(bfs_graph *g, int arm, int sm_factor, int ipt,
                                 GraphEntry **out) {
  const int key = (arm + 1) * 8192 + (g->run_parents ? 4096 : 0) + (ipt == 8 ? 2048 : 0) +
                  (g->use_l2_pin ? 1024 : 0) + sm_factor;
  auto it = g->graphs.find(key);
  if (it != g->graphs.end()) {
    *out = &it->second;
    return BFS_OK;
  }
  GraphEntry ge;
  bfs_status rc = build_loop_graph(g, arm, sm_factor, ipt, &ge);
  if (rc != BFS_OK) {
    if (ge.exec) cudaGraphExecDestroy(ge.exec);
    if (ge.graph) cudaGraphDestroy(ge.graph);
    return rc;
  }
  auto res = g->graphs.emplace(key, ge);
  *out = &res.first->second;
  return BFS_OK;
}

// ---- one BFS ------------------------------------------------------------------

static bfs_status read_state(bfs_graph *g) {
  CK(cudaMemcpyAsync(g->h_st, g->d_st, sizeof(BfsDevState), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return BFS_OK;
}

static bfs_status launch_sched(bfs_graph *g) {
  BfsDevState *st = g->d_st;
  const float *w = g->sched ? g->sched->d_w : nullptr;
  float min_conf = g->sched ? g->sched->min_conf : 0.f;
  SchedGraphConst gc = sched_graph_const(g->n_cols, g->nnz);
  void *args[] = {&st, &w, &min_conf, &gc};
  CK(cudaLaunchKernel(sched_kernel_fn(), dim3(1), dim3(32), args, 0, g->stream));
  return BFS_OK;
}

// arm_fixed < 0: the learned scheduler picks every level's arm on the device.
static bfs_status host_loop(bfs_graph *g, int arm_fixed, int sm_factor, int ipt,
                            LevelTimer *timer) {
  BfsDevState *st = g->d_st;
  unsigned long long no_cond = 0;
  int zero = 0;
  const bool prof = g->prof_explore != nullptr;
  const bool learned = arm_fixed < 0;
  void *fill_args[] = {&st};
  CK(cudaLaunchKernel(fill_kernel_fn(), dim3(g->num_sms * 4), dim3(256), fill_args, 0, g->stream));
  void *init_args[] = {&st, &no_cond, &zero};
  CK(cudaLaunchKernel(init_kernel_fn(), dim3(1), dim3(32), init_args, 0, g->stream));
  uint32_t launches = 2;
  for (uint32_t level = 0;; level++) {
    if (learned) {
      bfs_status rs = launch_sched(g);
      if (rs != BFS_OK) return rs;
      launches++;
    }
    bfs_status rc = read_state(g);
    if (rc != BFS_OK) return rc;
    if (prof && level > 0 && level - 1 < BFS_MAX_RECORDED_LEVELS) {
      CK(cudaEventElapsedTime(&g->prof_explore[level - 1], g->lvl_ev[0], g->lvl_ev[1]));
      CK(cudaEventElapsedTime(&g->prof_gen[level - 1], g->lvl_ev[1], g->lvl_ev[2]));
    }
    const uint32_t F = g->h_st->F, EF = g->h_st->EF;
    if (F == 0) break;
    int arm = learned ? g->h_st->arm : arm_fixed;
    if (timer && timer->choose) arm = timer->choose(timer->ctx, g, level, F, EF);
    if (arm < 0 || arm >= kNumArms) return fail(BFS_ERR_INVALID_ARG, "scheduler chose a bad arm");
    if (timer && timer->before) timer->before(timer->ctx, g, level, arm);
    if (prof) CK(cudaEventRecord(g->lvl_ev[0], g->stream));
    CK(launch_explore(g, arm, ipt, sm_factor, F, EF, false));
    if (prof) CK(cudaEventRecord(g->lvl_ev[1], g->stream));
    if (timer && timer->after) timer->after(timer->ctx, g, level, arm);
    void *lg_args[] = {&st, &no_cond, &zero};
    CK(cudaLaunchKernel(levelgen_kernel_fn(g->run_parents), dim3(g->lg_grid[g->run_parents]),
                        dim3(kLevelgenBlock), lg_args, levelgen_smem(g->run_parents), g->stream));
    if (prof) CK(cudaEventRecord(g->lvl_ev[2], g->stream));
    launches += 2;
    if (level < BFS_MAX_RECORDED_LEVELS) g->host_arms[level] = arm;
  }
  CK(cudaLaunchKernel(level_out_kernel_fn(), dim3(g->num_sms * 8), dim3(256), fill_args, 0,
                      g->stream));
  g->host_launches = launches + 1;
  return BFS_OK;
}

// The hub prefix size a request asks for on this handle (0: no layout).
static uint32_t hub_target(const bfs_graph *g) {
  if (g->hub_max == 0 || g->hub_request == 0) return 0;
  uint64_t k = g->hub_request < 0 ? (uint64_t)kHubDefaultVertices : (uint64_t)g->hub_request;
  k = std::min<uint64_t>(k, g->hub_max);
  return (uint32_t)(k / 128u * 128u);
}

// Builds the hub layout the handle's request asks for, once; a build that
// ran out of device memory is not retried until the request is made again.
bfs_status ensure_hub(bfs_graph *g) {
  const uint32_t want = hub_target(g);
  if (g->hub_tried && g->hub_built_for == want) return BFS_OK;
  g->hub_tried = true;
  g->hub_built_for = want;
  g->hub_gen++;  // workspaces that copied the layout's pointers rebuild
  bfs_status rc = build_hub(g, want);
  // cached loop graphs were built for the previous layout's launch shapes
  for (auto &kv : g->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  g->graphs.clear();
  return rc;
}

bfs_status run_device_impl(bfs_graph *g, uint32_t root, const bfs_options *opts_in,
                           int32_t *levels_dev, int32_t *parents_dev, bfs_stats *stats,
                           LevelTimer *timer, const std::function<bfs_status()> *after_launch) {
  if (!g || !levels_dev) return fail(BFS_ERR_INVALID_ARG, "null graph or level buffer");
  if (root >= g->n_cols) return fail(BFS_ERR_ROOT, "root out of range");
  bfs_options o;
  bfs_options_default(&o);
  if (opts_in) o = *opts_in;
  if (o.block == 0) o.block = 256;
  if (o.block != 128 && o.block != 256 && o.block != 512)
    return fail(BFS_ERR_INVALID_ARG, "block must be 128, 256 or 512");
  if (o.lb < BFS_LB_LLB || o.lb > BFS_LB_LEARNED)
    return fail(BFS_ERR_INVALID_ARG, "unknown load-balancing form");
  if (o.loop != BFS_LOOP_GRAPH && o.loop != BFS_LOOP_HOST)
    return fail(BFS_ERR_INVALID_ARG, "unknown loop mode");
  if (o.sm_factor < 0 || o.sm_factor > 64) return fail(BFS_ERR_INVALID_ARG, "sm_factor out of range");
  if (o.ipt == 0) o.ipt = 4;
  if (o.ipt != 4 && o.ipt != 8) return fail(BFS_ERR_INVALID_ARG, "ipt must be 4 or 8");
  CK(cudaSetDevice(g->device));
  g->use_l2_pin = o.l2_pin != 0;
  g->run_parents = parents_dev != nullptr;
  if (o.loop == BFS_LOOP_HOST) {
    cudaStreamAttrValue v;
    std::memset(&v, 0, sizeof(v));
    if (g->l2_pinned && g->use_l2_pin) v.accessPolicyWindow = g->l2_window;
    cudaStreamSetAttribute(g->stream, cudaStreamAttributeAccessPolicyWindow, &v);
    cudaGetLastError();
  }

  // learned without a model: the scheduler's fallback arm on every level
  const bool have_model = g->sched != nullptr && g->sched->d_w != nullptr;
  const int arm = (o.lb == BFS_LB_LEARNED) ? (have_model ? -1 : kFallbackArm)
                                           : arm_of(o.lb, o.block);
  g->prof_explore = g->prof_gen = nullptr;
  if (o.record >= 2 && stats) {
    g->prof_explore = stats->level_explore_ms;
    g->prof_gen = stats->level_gen_ms;
    std::memset(stats->level_explore_ms, 0, sizeof(stats->level_explore_ms));
    std::memset(stats->level_gen_ms, 0, sizeof(stats->level_gen_ms));
  }
  bfs_status hrc = ensure_hub(g);
  if (hrc != BFS_OK) return hrc;
  BfsDevState &s = *g->h_st;
  s = g->tmpl;
  s.root = root;
  s.level = levels_dev;
  s.parent = parents_dev;
  s.fixed_arm = arm;
  // The layout serves plans that run GLB levels (fixed GLB arms, the learned
  // schedule, the per-level recorder).  Fixed LLB and SLB keep the original
  // numbering: their tile-local balancing suffers when the hubs are
  // consecutive ids, i.e. consecutive queue entries.
  const bool use_hub = g->hub != nullptr &&
                       (o.lb == BFS_LB_GLB || o.lb == BFS_LB_LEARNED || timer != nullptr);
  if (use_hub) {
    s.indptr = g->hub->indptr;
    s.inds = g->hub->inds;
    s.inds_off = (uint32_t)((reinterpret_cast<uintptr_t>(g->hub->inds) & 15u) >> 2);
    s.perm = g->hub->perm;
    s.pinv = g->hub->pinv;
    s.moved = g->hub->moved;
    s.hub_words = g->hub->vertices / 32u;
    s.hub_min_edges = g->hub_min_edges ? g->hub_min_edges
                                       : std::max<uint32_t>(kHubMinEdges, 2u * g->hub->vertices);
  }
  const bool graph_loop = o.loop == BFS_LOOP_GRAPH && !timer && o.record < 2;
  GraphEntry *ge = nullptr;
  bfs_status rc;
  if (graph_loop) {
    rc = get_loop_graph(g, arm, o.sm_factor, o.ipt, &ge);
    if (rc != BFS_OK) return rc;
    if (arm < 0) {  // scheduler fused into init and level generation
      const SchedGraphConst gc = sched_graph_const(g->n_cols, g->nnz);
      s.sched_w = g->sched->d_w;
      s.sched_min_conf = g->sched->min_conf;
      s.sched_diam = gc.diam;
      s.sched_avg_deg_x = gc.avg_deg_x;
    }
  }
  CK(cudaEventRecord(g->ev0, g->stream));
  CK(launch_seed_state(g->d_st, *g->h_st, g->stream));
  uint32_t launches = 0;
  if (graph_loop) {
    CK(cudaGraphLaunch(ge->exec, g->stream));
  } else {
    rc = host_loop(g, arm, o.sm_factor, o.ipt, timer);
    if (rc != BFS_OK) return rc;
    launches = g->host_launches;
  }
  CK(cudaEventRecord(g->ev1, g->stream));
  if (after_launch) {
    rc = (*after_launch)();
    if (rc != BFS_OK) {
      cudaStreamSynchronize(g->stream);
      return rc;
    }
  }
  rc = read_state(g);
  if (rc != BFS_OK) return rc;
  const BfsDevState &r = *g->h_st;
  if (r.error & BFS_DEVERR_LEVEL_LIMIT)
    return fail(BFS_ERR_LEVEL_LIMIT, "level loop exceeded n_cols + 1 levels");
  if (r.error) return fail(BFS_ERR_DEVICE, "device error flag " + std::to_string(r.error));
  if (stats) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    stats->edges_count = r.edges_count;
    stats->reached = r.reached;
    stats->num_levels = r.max_level + 1;
    stats->device_ms = ms;
    stats->launches = (launches ? launches : r.launches) + 1;  // + the seed kernel
    stats->recorded = 0;
    if (o.record < 2) {
      std::memset(stats->level_explore_ms, 0, sizeof(stats->level_explore_ms));
      std::memset(stats->level_gen_ms, 0, sizeof(stats->level_gen_ms));
    }
    if (o.record) {
      const uint32_t nrec = std::min<uint32_t>(r.lvl + 1, BFS_MAX_RECORDED_LEVELS);
      stats->recorded = nrec;
      CK(cudaMemcpy(stats->level_frontier, g->tmpl.rec_frontier, nrec * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(stats->level_edges, g->tmpl.rec_edges, nrec * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(stats->level_arm, g->tmpl.rec_arm, nrec * 4, cudaMemcpyDeviceToHost));
      std::vector<int32_t> ran(nrec);
      CK(cudaMemcpy(ran.data(), g->tmpl.rec_ran, nrec * 4, cudaMemcpyDeviceToHost));
      // level_arm = the explore kernel that ran; where a scheduler chose the
      // arm on the device, the kernel that ran must be its choice
      for (uint32_t i = 0; i < nrec; i++) {
        if (stats->level_frontier[i] == 0) {
          stats->level_arm[i] = -1;
          continue;
        }
        const int32_t chosen = stats->level_arm[i];
        if (chosen >= 0 && ran[i] != chosen)
          return fail(BFS_ERR_DEVICE, "level " + std::to_string(i) + ": explore arm " +
                                          std::to_string(ran[i]) + " ran, scheduler chose " +
                                          std::to_string(chosen));
        stats->level_arm[i] = ran[i];
      }
    }
  }
  g->prof_explore = g->prof_gen = nullptr;
  return BFS_OK;
}

}  // namespace bfsgb

using namespace bfsgb;

extern "C" {

int bfs_abi_version(void) { return BFS_GB300_ABI_VERSION; }

const char *bfs_status_string(bfs_status s) {
  switch (s) {
    case BFS_OK: return "ok";
    case BFS_ERR_INVALID_ARG: return "invalid argument";
    case BFS_ERR_ROOT: return "root out of range";
    case BFS_ERR_GRAPH: return "malformed graph";
    case BFS_ERR_CUDA: return "CUDA error";
    case BFS_ERR_OOM: return "out of memory";
    case BFS_ERR_IO: return "I/O error";
    case BFS_ERR_LEVEL_LIMIT: return "level limit exceeded";
    case BFS_ERR_NO_DEVICE: return "no CUDA device";
    case BFS_ERR_UNSUPPORTED: return "unsupported";
    case BFS_ERR_DEVICE: return "device error";
  }
  return "unknown status";
}

const char *bfs_last_error(void) { return g_last_error.c_str(); }

void bfs_options_default(bfs_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->lb = BFS_LB_LLB;
  o->block = 256;
  o->sm_factor = 0;
  o->loop = BFS_LOOP_GRAPH;
  o->l2_pin = 1;
  o->record = 0;
  o->ipt = 4;
}

static bfs_status require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(BFS_ERR_NO_DEVICE, "no CUDA device visible");
  }
  return BFS_OK;
}

bfs_status bfs_graph_upload(const uint32_t *indptr, const uint32_t *inds, uint32_t n_rows,
                            uint32_t n_cols, uint64_t nnz, int validate, bfs_graph **out) {
  if (!indptr || (!inds && nnz) || !out) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  *out = nullptr;
  bfs_status rc = check_dims(n_rows, n_cols, nnz);
  if (rc != BFS_OK) return rc;
  rc = require_device();
  if (rc != BFS_OK) return rc;
  uint32_t *d_indptr = nullptr, *d_inds = nullptr;
  cudaError_t e = dev_malloc(&d_indptr, sizeof(uint32_t) * ((size_t)n_cols + 1));
  if (e == cudaSuccess) e = dev_malloc(&d_inds, sizeof(uint32_t) * (nnz ? nnz : 1));
  if (e == cudaSuccess)
    e = cudaMemcpy(d_indptr, indptr, sizeof(uint32_t) * ((size_t)n_cols + 1),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nnz)
    e = cudaMemcpy(d_inds, inds, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d_indptr);
    cudaFree(d_inds);
    return fail(e == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,
                std::string("graph upload: ") + cudaGetErrorString(e));
  }
  return make_graph(d_indptr, d_inds, n_rows, n_cols, nnz, true, validate, out);
}

bfs_status bfs_graph_wrap_device(const uint32_t *d_indptr, const uint32_t *d_inds,
                                 uint32_t n_rows, uint32_t n_cols, uint64_t nnz, int validate,
                                 bfs_graph **out) {
  if (!d_indptr || (!d_inds && nnz) || !out) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  *out = nullptr;
  bfs_status rc = check_dims(n_rows, n_cols, nnz);
  if (rc != BFS_OK) return rc;
  rc = require_device();
  if (rc != BFS_OK) return rc;
  return make_graph(d_indptr, d_inds, n_rows, n_cols, nnz, false, validate, out);
}

bfs_status bfs_graph_free(bfs_graph *g) {
  if (!g) return BFS_OK;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  free_sched(g);
  free_msbfs(g);
  free_hub(g);
  free_workspace(g);
  if (g->owns_csc) {
    cudaFree(g->indptr);
    cudaFree(g->inds);
  }
  delete g;
  return BFS_OK;
}

bfs_status bfs_graph_info(const bfs_graph *g, uint32_t *n_rows, uint32_t *n_cols,
                          uint64_t *nnz) {
  if (!g) return fail(BFS_ERR_INVALID_ARG, "null graph");
  if (n_rows) *n_rows = g->n_rows;
  if (n_cols) *n_cols = g->n_cols;
  if (nnz) *nnz = g->nnz;
  return BFS_OK;
}

bfs_status bfs_graph_device_csc(const bfs_graph *g, const uint32_t **d_indptr,
                                const uint32_t **d_inds) {
  if (!g) return fail(BFS_ERR_INVALID_ARG, "null graph");
  if (d_indptr) *d_indptr = g->indptr;
  if (d_inds) *d_inds = g->inds;
  return BFS_OK;
}

bfs_status bfs_run_device(bfs_graph *g, uint32_t root, const bfs_options *opts,
                          int32_t *levels_dev, int32_t *parents_dev, bfs_stats *stats) {
  return run_device_impl(g, root, opts, levels_dev, parents_dev, stats, nullptr);
}

bfs_status bfs_run(bfs_graph *g, uint32_t root, const bfs_options *opts, int32_t *levels_host,
                   int32_t *parents_host, bfs_stats *stats) {
  if (!g || !levels_host) return fail(BFS_ERR_INVALID_ARG, "null graph or level buffer");
  CK(cudaSetDevice(g->device));
  const size_t bytes = sizeof(int32_t) * (size_t)g->n_cols;
  if (!g->d_out_levels) CK(dev_malloc(&g->d_out_levels, bytes));
  if (parents_host && !g->d_out_parents) CK(dev_malloc(&g->d_out_parents, bytes));
  bfs_status rc = run_device_impl(g, root, opts, g->d_out_levels,
                                  parents_host ? g->d_out_parents : nullptr, stats, nullptr);
  if (rc != BFS_OK) return rc;
  CK(cudaMemcpyAsync(levels_host, g->d_out_levels, bytes, cudaMemcpyDeviceToHost, g->stream));
  if (parents_host)
    CK(cudaMemcpyAsync(parents_host, g->d_out_parents, bytes, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return BFS_OK;
}

// Runs i and i + 1 write device buffers of alternating slots; run i's copy
// to the host is queued on the copy stream once run i + 1 is queued, so it
// overlaps run i + 1, and run i + 2 waits on the main stream for that copy
// before it overwrites the slot.  Device-to-host copies into pageable memory
// return only when done, so with pageable buffers the runs are serial.
static bfs_status run_roots_impl(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                                 const bfs_options *opts, int32_t *const *levels_host,
                                 int32_t *const *parents_host, bfs_stats *stats) {
  const size_t bytes = sizeof(int32_t) * (size_t)g->n_cols;
  const int kinds = parents_host ? 2 : 1;
  for (int slot = 0; slot < (n_roots > 1 ? 2 : 1); slot++)
    for (int k = 0; k < kinds; k++)
      if (!g->d_ring[slot][k]) CK(dev_malloc(&g->d_ring[slot][k], bytes));
  if (!g->copy_stream) CK(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
  if (!g->ev_ready) CK(cudaEventCreateWithFlags(&g->ev_ready, cudaEventDisableTiming));
  for (auto &e : g->ev_copied)
    if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // queues the copy of finished run j (its device buffers are slot j & 1)
  auto copy_out = [&](uint32_t j) -> bfs_status {
    const int slot = (int)(j & 1u);
    CK(cudaStreamWaitEvent(g->copy_stream, g->ev_ready, 0));
    CK(cudaMemcpyAsync(levels_host[j], g->d_ring[slot][0], bytes, cudaMemcpyDeviceToHost,
                       g->copy_stream));
    if (parents_host)
      CK(cudaMemcpyAsync(parents_host[j], g->d_ring[slot][1], bytes, cudaMemcpyDeviceToHost,
                         g->copy_stream));
    CK(cudaEventRecord(g->ev_copied[slot], g->copy_stream));
    return BFS_OK;
  };
  for (uint32_t i = 0; i < n_roots; i++) {
    const int slot = (int)(i & 1u);
    if (i >= 2) CK(cudaStreamWaitEvent(g->stream, g->ev_copied[slot], 0));
    // run i-1's copy is issued after run i is queued, so that it does not
    // hold up the start of run i, and before the wait for run i
    const std::function<bfs_status()> prev_copy = [&]() { return copy_out(i - 1); };
    // returns after the run has finished (it reads the device state back)
    bfs_status rc = run_device_impl(g, roots[i], opts, g->d_ring[slot][0],
                                    parents_host ? g->d_ring[slot][1] : nullptr,
                                    stats ? stats + i : nullptr, nullptr,
                                    i > 0 ? &prev_copy : nullptr);
    if (rc != BFS_OK) return rc;
    CK(cudaEventRecord(g->ev_ready, g->stream));  // run i has finished
  }
  return copy_out(n_roots - 1);
}

bfs_status bfs_run_roots(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                         const bfs_options *opts, int32_t *const *levels_host,
                         int32_t *const *parents_host, bfs_stats *stats) {
  if (!g || (n_roots && (!roots || !levels_host)))
    return fail(BFS_ERR_INVALID_ARG, "null graph, roots or level buffers");
  for (uint32_t i = 0; i < n_roots; i++) {
    if (!levels_host[i] || (parents_host && !parents_host[i]))
      return fail(BFS_ERR_INVALID_ARG, "null output buffer of run " + std::to_string(i));
    if (roots[i] >= g->n_cols) return fail(BFS_ERR_ROOT, "root out of range");
  }
  if (n_roots == 0) return BFS_OK;
  CK(cudaSetDevice(g->device));
  const bfs_status rc = run_roots_impl(g, roots, n_roots, opts, levels_host, parents_host, stats);
  // no copy into the caller's buffers is left in flight, also after an error
  if (g->copy_stream) {
    const cudaError_t e = cudaStreamSynchronize(g->copy_stream);
    if (rc == BFS_OK && e != cudaSuccess) return fail(BFS_ERR_CUDA, cudaGetErrorString(e));
  }
  return rc;
}

bfs_status bfs_validate_device(bfs_graph *g, uint32_t root, const int32_t *levels_dev,
                               const int32_t *parents_dev, uint64_t *bad) {
  if (!g || !levels_dev || !bad) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (root >= g->n_cols) return fail(BFS_ERR_ROOT, "root out of range");
  CK(cudaSetDevice(g->device));
  uint8_t *flags = nullptr;
  unsigned long long *d_bad = nullptr, h_bad = 0;
  cudaError_t e = dev_malloc(&flags, 2 * (size_t)g->n_cols);
  if (e == cudaSuccess) e = dev_malloc(&d_bad, sizeof(*d_bad));
  if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 2 * (size_t)g->n_cols, g->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(*d_bad), g->stream);
  if (e == cudaSuccess)
    e = launch_validate(g->indptr, g->inds, g->n_rows, g->n_cols, root, levels_dev, parents_dev,
                        flags, flags + g->n_cols, d_bad, g->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  cudaFree(flags);
  cudaFree(d_bad);
  if (e != cudaSuccess) return fail(BFS_ERR_CUDA, std::string("validate: ") + cudaGetErrorString(e));
  *bad = h_bad;
  return BFS_OK;
}

bfs_status bfs_hub_configure(bfs_graph *g, int64_t vertices, uint32_t min_edges) {
  if (!g) return fail(BFS_ERR_INVALID_ARG, "null graph");
  if (vertices < -1) return fail(BFS_ERR_INVALID_ARG, "hub vertices must be -1, 0 or positive");
  CK(cudaSetDevice(g->device));
  CK(cudaStreamSynchronize(g->stream));
  g->hub_request = vertices;
  g->hub_min_edges = min_edges;
  g->hub_tried = false;  // an explicit request is built again, even after a failure
  return ensure_hub(g);
}

bfs_status bfs_hub_info(bfs_graph *g, uint32_t *vertices, int32_t *relabelled,
                        uint32_t *max_vertices) {
  if (!g) return fail(BFS_ERR_INVALID_ARG, "null graph");
  CK(cudaSetDevice(g->device));
  bfs_status rc = ensure_hub(g);
  if (rc != BFS_OK) return rc;
  if (vertices) *vertices = g->hub ? g->hub->vertices : 0u;
  if (relabelled) *relabelled = g->hub && g->hub->relabelled ? 1 : 0;
  if (max_vertices) *max_vertices = g->hub_max;
  return BFS_OK;
}

bfs_status bfs_validate_host(bfs_graph *g, uint32_t root, const int32_t *levels_host,
                             uint64_t *bad) {
  if (!g || !levels_host || !bad) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  CK(cudaSetDevice(g->device));
  const size_t bytes = sizeof(int32_t) * (size_t)g->n_cols;
  if (!g->d_out_levels) CK(dev_malloc(&g->d_out_levels, bytes));
  CK(cudaMemcpy(g->d_out_levels, levels_host, bytes, cudaMemcpyHostToDevice));
  return bfs_validate_device(g, root, g->d_out_levels, nullptr, bad);
}

}  // extern "C"
