// multigraph.cu -- many small graphs, one root each, in one persistent launch.
//
// The reference launches two kernels per level of one graph and synchronises
// with the host after each level (src/run_bfs_gpu.hpp:682-727); for graphs of
// a few thousand vertices that overhead is the whole run time.  Here a batch
// of graphs is packed into one CSC in HBM and a single persistent kernel runs
// all of them: every block claims whole graphs from a work counter (largest
// edge count first) and runs a complete level-synchronous top-down BFS of the
// graph on its own, with the visited bitmap in shared memory and __syncthreads
// as the level barrier.  Within a level the block uses the LLB form: a block
// exclusive scan of a tile's degrees, the tile's edges split evenly over the
// warps, owners resolved per warp round (bfs_internal / device_util), IPT
// rounds in flight per lane.  A claim is an atomicOr on the shared bitmap; the
// claiming thread writes the level and appends the vertex to the next queue
// (vertices >= n_rows or without out-edges get a level but are not queued).
//
// Block size (128/256/512) and items per thread (1/2/4 rounds per lane) come
// from an autotuner that times every combination on the batch and caches the
// choice per GPU and batch shape.  The launch (work-counter reset, level fill,
// persistent kernel) is captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "bfs_internal.h"
#include "device_util.cuh"

namespace bfsgb {

constexpr uint32_t kMultiMaxVertices = 1u << 18;  // 32 KiB shared bitmap

struct MultiDesc {
  uint64_t vbase;      // offset of the graph's indptr in the packed indptr array
  uint64_t ebase;      // offset of the graph's edges in the packed inds array
  uint64_t lbase;      // offset of the graph's levels in the output
  uint32_t n_rows, n_cols;
  uint32_t root;
  uint32_t pad;
};

template <int B, int IPT>
__global__ void __launch_bounds__(B) multi_bfs_kernel(const MultiDesc *__restrict__ descs,
                                                      const uint32_t *__restrict__ order,
                                                      uint32_t n_graphs,
                                                      const uint32_t *__restrict__ indptr_all,
                                                      const uint32_t *__restrict__ inds_all,
                                                      uint32_t *work, uint32_t *queues,
                                                      uint32_t qcap, int32_t *levels,
                                                      unsigned long long *edges_out) {
  constexpr int NW = B / 32;
  extern __shared__ uint32_t s_bitmap[];
  __shared__ uint32_t s_off[B + 1];
  __shared__ uint32_t s_beg[B];
  __shared__ uint32_t s_wsum[NW];
  __shared__ uint32_t s_graph, s_next;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t *q0 = queues + (size_t)blockIdx.x * 2 * qcap;
  uint32_t *q1 = q0 + qcap;

  for (;;) {
    if (threadIdx.x == 0) s_graph = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t gi = s_graph;
    if (gi >= n_graphs) break;
    const MultiDesc d = descs[order[gi]];
    const uint32_t *__restrict__ ip = indptr_all + d.vbase;
    const uint32_t *__restrict__ ix = inds_all + d.ebase;
    int32_t *lv = levels + d.lbase;
    const uint32_t words = (d.n_cols + 31u) >> 5;
    for (uint32_t w = threadIdx.x; w < words; w += B) s_bitmap[w] = 0u;
    __syncthreads();
    unsigned long long edges = 0;  // sum of the degrees of every expanded tile
    uint32_t F = 0;
    if (threadIdx.x == 0) {
      const uint32_t r = d.root;
      s_bitmap[r >> 5] |= 1u << (r & 31u);
      lv[r] = 0;
      const uint32_t rdeg = r < d.n_rows ? ip[r + 1] - ip[r] : 0u;
      if (rdeg) q0[0] = r;
      s_next = rdeg ? 1u : 0u;
    }
    __syncthreads();
    F = s_next;
    uint32_t *qc = q0, *qn = q1;
    int32_t lvl = 0;
    while (F > 0) {
      __syncthreads();
      if (threadIdx.x == 0) s_next = 0;
      __syncthreads();
      for (uint32_t tile = 0; tile < F; tile += B) {
        const uint32_t slot = tile + threadIdx.x;
        uint32_t beg = 0, deg = 0;
        if (slot < F) {
          const uint32_t u = qc[slot];
          beg = ip[u];
          deg = ip[u + 1] - beg;
        }
        const uint32_t incl = warp_incl_scan(deg, lane);
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
          uint32_t w = lane < (uint32_t)NW ? s_wsum[lane] : 0u;
          w = warp_incl_scan(w, lane);
          if (lane < (uint32_t)NW) s_wsum[lane] = w;
        }
        __syncthreads();
        const uint32_t total = s_wsum[NW - 1];
        s_off[threadIdx.x] = (warp ? s_wsum[warp - 1] : 0u) + incl - deg;
        s_beg[threadIdx.x] = beg;
        if (threadIdx.x == 0) s_off[B] = total;
        __syncthreads();
        const uint32_t per_warp = ((total + NW - 1) / NW + 31u) & ~31u;
        const uint32_t w0 = warp * per_warp;
        if (w0 < total) {
          const uint32_t w1 = min(total, w0 + per_warp);
          uint32_t lo = 0, hi = B;
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_off[mid] <= w0) lo = mid; else hi = mid;
          }
          uint32_t cur = lo;
          for (uint32_t base = w0; base < w1; base += 32u * IPT) {
            uint32_t addr[IPT];
#pragma unroll
            for (int u = 0; u < IPT; u++) {
              const uint32_t rb = base + 32u * u;
              const uint32_t e = rb + lane;
              const uint32_t j = cur + 1u + lane;
              const uint32_t bnd = (j <= (uint32_t)B) ? s_off[j] : kFull;
              const uint32_t p = bnd - rb;
              const uint32_t starts = __reduce_or_sync(kFull, (p < 32u) ? (1u << p) : 0u);
              const uint32_t o = cur + __popc(starts & ((2u << lane) - 1u));
              addr[u] = (e < w1) ? s_beg[o] + (e - s_off[o]) : kFull;
              cur = __shfl_sync(kFull, o, 31);
              if (cur >= (uint32_t)B) cur = B - 1;
            }
            uint32_t nb[IPT];
#pragma unroll
            for (int u = 0; u < IPT; u++) nb[u] = addr[u] != kFull ? ix[addr[u]] : 0u;
#pragma unroll
            for (int u = 0; u < IPT; u++) {
              if (addr[u] == kFull) continue;
              const uint32_t v = nb[u], bit = 1u << (v & 31u);
              if (s_bitmap[v >> 5] & bit) continue;
              const uint32_t old = atomicOr(&s_bitmap[v >> 5], bit);
              if (old & bit) continue;
              lv[v] = lvl + 1;
              if (v < d.n_rows && ip[v + 1] > ip[v]) qn[atomicAdd(&s_next, 1u)] = v;
            }
          }
        }
        if (threadIdx.x == 0) edges += total;
        __syncthreads();
      }
      __syncthreads();
      F = s_next;
      uint32_t *t = qc;
      qc = qn;
      qn = t;
      lvl++;
    }
    if (threadIdx.x == 0) edges_out[order[gi]] = edges;
    __syncthreads();
  }
}

__global__ void multi_fill_kernel(int32_t *levels, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    levels[i] = -1;
}

using MultiKernel = void (*)(const MultiDesc *, const uint32_t *, uint32_t, const uint32_t *,
                             const uint32_t *, uint32_t *, uint32_t *, uint32_t, int32_t *,
                             unsigned long long *);

struct MultiConfig {
  int block, ipt;
  MultiKernel fn;
};

static const MultiConfig kMultiConfigs[] = {
    {128, 1, multi_bfs_kernel<128, 1>}, {128, 2, multi_bfs_kernel<128, 2>},
    {128, 4, multi_bfs_kernel<128, 4>}, {256, 1, multi_bfs_kernel<256, 1>},
    {256, 2, multi_bfs_kernel<256, 2>}, {256, 4, multi_bfs_kernel<256, 4>},
    {512, 1, multi_bfs_kernel<512, 1>}, {512, 2, multi_bfs_kernel<512, 2>},
    {512, 4, multi_bfs_kernel<512, 4>},
};
constexpr int kNumMultiConfigs = sizeof(kMultiConfigs) / sizeof(kMultiConfigs[0]);

}  // namespace bfsgb

using namespace bfsgb;

struct bfs_multi {
  int device = 0;
  int num_sms = 0;
  uint32_t n_graphs = 0;
  uint32_t max_cols = 0, max_rows = 0;
  uint64_t total_cols = 0, total_edges = 0;
  std::vector<MultiDesc> descs;
  uint32_t *d_indptr = nullptr, *d_inds = nullptr, *d_order = nullptr, *d_work = nullptr;
  uint32_t *d_queues = nullptr;
  MultiDesc *d_descs = nullptr;
  unsigned long long *d_edges = nullptr;
  size_t queue_blocks = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // captured launch for the current configuration and output buffer
  int cfg = -1;
  int32_t *graph_levels = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int grid = 0;
};

#define GK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(e_ == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,    \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

static int config_index(int block, int ipt) {
  for (int i = 0; i < kNumMultiConfigs; i++)
    if (kMultiConfigs[i].block == block && kMultiConfigs[i].ipt == ipt) return i;
  return -1;
}

static bfs_status multi_prepare(bfs_multi *m, int cfg, int32_t *levels_dev) {
  if (m->exec && m->cfg == cfg && m->graph_levels == levels_dev) return BFS_OK;
  if (m->exec) cudaGraphExecDestroy(m->exec);
  if (m->graph) cudaGraphDestroy(m->graph);
  m->exec = nullptr;
  m->graph = nullptr;
  const MultiConfig &c = kMultiConfigs[cfg];
  const size_t smem = (size_t)((m->max_cols + 31) / 32) * 4;
  GK(cudaFuncSetAttribute((const void *)c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)std::max<size_t>(smem, 1)));
  int occ = 0;
  GK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)c.fn, c.block, smem));
  int grid = m->num_sms * std::max(occ, 1);
  grid = (int)std::min<size_t>((size_t)grid, m->queue_blocks);
  grid = std::max(1, std::min<int>(grid, (int)m->n_graphs));
  m->grid = grid;
  // capture: reset work counter, fill levels with -1, persistent kernel
  GK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(m->d_work, 0, sizeof(uint32_t), m->stream);
  multi_fill_kernel<<<m->num_sms * 4, 256, 0, m->stream>>>(levels_dev, m->total_cols);
  c.fn<<<grid, c.block, smem, m->stream>>>(m->d_descs, m->d_order, m->n_graphs, m->d_indptr,
                                           m->d_inds, m->d_work, m->d_queues, m->max_rows,
                                           levels_dev, m->d_edges);
  cudaError_t ce = cudaStreamEndCapture(m->stream, &m->graph);
  if (ce != cudaSuccess)
    return fail(BFS_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
  GK(cudaGraphInstantiate(&m->exec, m->graph, 0));
  m->cfg = cfg;
  m->graph_levels = levels_dev;
  return BFS_OK;
}

extern "C" {

bfs_status bfs_multi_create(uint32_t n_graphs, const uint32_t *const *indptrs,
                            const uint32_t *const *inds, const uint32_t *n_rows,
                            const uint32_t *n_cols, const uint64_t *nnz, bfs_multi **out) {
  if (!out || !indptrs || !inds || !n_rows || !n_cols || !nnz || n_graphs == 0)
    return fail(BFS_ERR_INVALID_ARG, "bad arguments");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(BFS_ERR_NO_DEVICE, "no CUDA device visible");
  }
  bfs_multi *m = new bfs_multi();
  m->n_graphs = n_graphs;
  m->descs.resize(n_graphs);
  uint64_t vb = 0, eb = 0, lb = 0;
  for (uint32_t g = 0; g < n_graphs; g++) {
    if (!indptrs[g] || (!inds[g] && nnz[g]) || n_cols[g] == 0 || n_rows[g] > n_cols[g] ||
        n_cols[g] > kMultiMaxVertices || nnz[g] > BFS_MAX_EDGES || indptrs[g][n_cols[g]] != nnz[g]) {
      delete m;
      return fail(BFS_ERR_INVALID_ARG, "graph " + std::to_string(g) +
                                           ": bad sizes (at most 2^18 vertices per graph)");
    }
    MultiDesc &d = m->descs[g];
    d.vbase = vb;
    d.ebase = eb;
    d.lbase = lb;
    d.n_rows = n_rows[g];
    d.n_cols = n_cols[g];
    d.root = 0;
    vb += (uint64_t)n_cols[g] + 1;
    eb += nnz[g];
    lb += n_cols[g];
    m->max_cols = std::max(m->max_cols, n_cols[g]);
    m->max_rows = std::max(m->max_rows, std::max<uint32_t>(n_rows[g], 1));
  }
  m->total_cols = lb;
  m->total_edges = eb;
  // largest graphs first (longest-processing-time order)
  std::vector<uint32_t> order(n_graphs);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return nnz[a] > nnz[b]; });
  bfs_status rc = BFS_OK;
  std::vector<uint32_t> hip(vb), hix(eb ? eb : 1);
  for (uint32_t g = 0; g < n_graphs; g++) {
    std::memcpy(hip.data() + m->descs[g].vbase, indptrs[g], sizeof(uint32_t) * (n_cols[g] + 1));
    if (nnz[g]) std::memcpy(hix.data() + m->descs[g].ebase, inds[g], sizeof(uint32_t) * nnz[g]);
  }
  unsigned long long bad = 0;
  for (uint32_t g = 0; g < n_graphs && !bad; g++) {
    const uint32_t *ip = indptrs[g];
    if (ip[0] != 0) bad = 1;
    for (uint32_t v = 0; v < n_cols[g] && !bad; v++)
      if (ip[v + 1] < ip[v]) bad = 1;
    for (uint64_t k = 0; k < nnz[g] && !bad; k++)
      if (inds[g][k] >= n_cols[g]) bad = 1;
  }
  if (bad) {
    delete m;
    return fail(BFS_ERR_GRAPH, "malformed CSC in the batch");
  }
  auto cleanup = [&]() {
    cudaFree(m->d_indptr);
    cudaFree(m->d_inds);
    cudaFree(m->d_order);
    cudaFree(m->d_work);
    cudaFree(m->d_queues);
    cudaFree(m->d_descs);
    cudaFree(m->d_edges);
    if (m->stream) cudaStreamDestroy(m->stream);
    if (m->e0) cudaEventDestroy(m->e0);
    if (m->e1) cudaEventDestroy(m->e1);
    delete m;
  };
#define CK2(call)                                                                   \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      rc = fail(e_ == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,       \
                std::string(#call) + ": " + cudaGetErrorString(e_));                \
      cleanup();                                                                    \
      return rc;                                                                    \
    }                                                                               \
  } while (0)
  CK2(cudaGetDevice(&m->device));
  CK2(cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device));
  CK2(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  CK2(cudaEventCreate(&m->e0));
  CK2(cudaEventCreate(&m->e1));
  CK2(cudaMalloc(&m->d_indptr, sizeof(uint32_t) * vb));
  CK2(cudaMalloc(&m->d_inds, sizeof(uint32_t) * std::max<uint64_t>(eb, 1)));
  CK2(cudaMalloc(&m->d_order, sizeof(uint32_t) * n_graphs));
  CK2(cudaMalloc(&m->d_work, sizeof(uint32_t)));
  CK2(cudaMalloc(&m->d_descs, sizeof(MultiDesc) * n_graphs));
  CK2(cudaMalloc(&m->d_edges, sizeof(unsigned long long) * n_graphs));
  // queues: two of max_rows entries per resident block (bounded by the
  // largest occupancy of any configuration)
  m->queue_blocks = (size_t)m->num_sms * 16;
  CK2(cudaMalloc(&m->d_queues, sizeof(uint32_t) * 2 * (size_t)m->max_rows * m->queue_blocks));
  CK2(cudaMemcpy(m->d_indptr, hip.data(), sizeof(uint32_t) * vb, cudaMemcpyHostToDevice));
  CK2(cudaMemcpy(m->d_inds, hix.data(), sizeof(uint32_t) * std::max<uint64_t>(eb, 1),
                 cudaMemcpyHostToDevice));
  CK2(cudaMemcpy(m->d_order, order.data(), sizeof(uint32_t) * n_graphs, cudaMemcpyHostToDevice));
#undef CK2
  *out = m;
  return BFS_OK;
}

bfs_status bfs_multi_free(bfs_multi *m) {
  if (!m) return BFS_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  if (m->exec) cudaGraphExecDestroy(m->exec);
  if (m->graph) cudaGraphDestroy(m->graph);
  cudaFree(m->d_indptr);
  cudaFree(m->d_inds);
  cudaFree(m->d_order);
  cudaFree(m->d_work);
  cudaFree(m->d_queues);
  cudaFree(m->d_descs);
  cudaFree(m->d_edges);
  if (m->stream) cudaStreamDestroy(m->stream);
  if (m->e0) cudaEventDestroy(m->e0);
  if (m->e1) cudaEventDestroy(m->e1);
  delete m;
  return BFS_OK;
}

bfs_status bfs_multi_level_offset(const bfs_multi *m, uint32_t graph, uint64_t *offset) {
  if (!m || !offset || graph >= m->n_graphs) return fail(BFS_ERR_INVALID_ARG, "bad graph index");
  *offset = m->descs[graph].lbase;
  return BFS_OK;
}

bfs_status bfs_multi_run(bfs_multi *m, const uint32_t *roots, int32_t block, int32_t ipt,
                         int32_t *levels_dev, uint64_t *edges_count_out, double *device_ms) {
  if (!m || !roots || !levels_dev) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  const int cfg = config_index(block, ipt);
  if (cfg < 0) return fail(BFS_ERR_INVALID_ARG, "block must be 128/256/512 and ipt 1/2/4");
  for (uint32_t g = 0; g < m->n_graphs; g++)
    if (roots[g] >= m->descs[g].n_cols) return fail(BFS_ERR_ROOT, "root out of range");
  GK(cudaSetDevice(m->device));
  bool moved = false;
  for (uint32_t g = 0; g < m->n_graphs; g++) {
    if (m->descs[g].root != roots[g]) moved = true;
    m->descs[g].root = roots[g];
  }
  if (moved || m->cfg < 0)
    GK(cudaMemcpyAsync(m->d_descs, m->descs.data(), sizeof(MultiDesc) * m->n_graphs,
                       cudaMemcpyHostToDevice, m->stream));
  bfs_status rc = multi_prepare(m, cfg, levels_dev);
  if (rc != BFS_OK) return rc;
  GK(cudaEventRecord(m->e0, m->stream));
  GK(cudaGraphLaunch(m->exec, m->stream));
  GK(cudaEventRecord(m->e1, m->stream));
  if (edges_count_out)
    GK(cudaMemcpyAsync(edges_count_out, m->d_edges, sizeof(uint64_t) * m->n_graphs,
                       cudaMemcpyDeviceToHost, m->stream));
  GK(cudaStreamSynchronize(m->stream));
  float ms = 0.f;
  GK(cudaEventElapsedTime(&ms, m->e0, m->e1));
  if (device_ms) *device_ms = ms;
  return BFS_OK;
}

bfs_status bfs_multi_autotune(bfs_multi *m, const uint32_t *roots, int32_t *levels_dev,
                              int32_t reps, const char *cache_path, int32_t *best_block,
                              int32_t *best_ipt, float *times_ms) {
  if (!m || !roots || !levels_dev || !best_block || !best_ipt)
    return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (reps < 1) reps = 3;
  cudaDeviceProp prop;
  GK(cudaGetDeviceProperties(&prop, m->device));
  std::ostringstream key;
  key << prop.name << "|sm" << prop.multiProcessorCount << "|g" << m->n_graphs << "|v"
      << m->total_cols << "|e" << m->total_edges;
  if (cache_path && cache_path[0]) {
    std::ifstream in(cache_path);
    std::string line;
    while (std::getline(in, line)) {
      const size_t t1 = line.rfind('\t');
      if (t1 == std::string::npos) continue;
      const size_t t0 = line.rfind('\t', t1 - 1);
      if (t0 == std::string::npos || line.substr(0, t0) != key.str()) continue;
      const int b = std::atoi(line.c_str() + t0 + 1), p = std::atoi(line.c_str() + t1 + 1);
      if (config_index(b, p) >= 0) {
        *best_block = b;
        *best_ipt = p;
        if (times_ms)
          for (int i = 0; i < kNumMultiConfigs; i++) times_ms[i] = -1.f;
        return BFS_OK;
      }
    }
  }
  int best = 0;
  float best_ms = 1e30f;
  for (int i = 0; i < kNumMultiConfigs; i++) {
    double t = 0.0, mn = 1e30;
    bfs_status rc = bfs_multi_run(m, roots, kMultiConfigs[i].block, kMultiConfigs[i].ipt,
                                  levels_dev, nullptr, &t);  // warm-up + capture
    if (rc != BFS_OK) return rc;
    for (int r = 0; r < reps; r++) {
      rc = bfs_multi_run(m, roots, kMultiConfigs[i].block, kMultiConfigs[i].ipt, levels_dev,
                         nullptr, &t);
      if (rc != BFS_OK) return rc;
      mn = std::min(mn, t);
    }
    if (times_ms) times_ms[i] = (float)mn;
    if (mn < best_ms) {
      best_ms = (float)mn;
      best = i;
    }
  }
  *best_block = kMultiConfigs[best].block;
  *best_ipt = kMultiConfigs[best].ipt;
  if (cache_path && cache_path[0]) {
    std::ofstream outf(cache_path, std::ios::app);
    if (outf) outf << key.str() << '\t' << *best_block << '\t' << *best_ipt << '\n';
  }
  return BFS_OK;
}

}  // extern "C"
