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
#include <cooperative_groups.h>
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
#include "dev_alloc.h"
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

// Kernel parameters (passed by value).
struct MultiArgs {
  const MultiDesc *descs;
  const uint32_t *order;        // graphs, largest edge count first
  uint32_t n_graphs;
  uint32_t n_big;               // order[0, n_big): graphs run by a whole cluster
  const uint32_t *indptr_all;
  const uint32_t *inds_all;
  uint32_t *work;               // [0]: next small graph, [1]: next big graph
  uint32_t *queues;             // two queues of qcap entries per block
  uint32_t qcap;
  uint32_t *gbits;              // per cluster: the authoritative visited bitmap
  uint32_t gwords;              // words per cluster bitmap
  uint32_t *gcnt;               // per cluster: 3 queue counters + claimed graph
  int32_t *levels;
  unsigned long long *edges_out;
};

// One level of one graph over tiles tile0, tile0 + tstride, ... of B
// frontier entries (LLB form): block exclusive scan of the tile's degrees,
// the tile's edges split evenly over the warps, owners resolved per warp
// round, IPT rounds in flight per lane.  A claim is an atomicOr on the
// visited bitmap -- the block's own shared bitmap, or, for a graph shared by
// a cluster (CL), the cluster's bitmap in global memory, with the shared
// bitmap kept as a filter of already visited vertices.  The claiming thread
// writes the level; kept vertices are appended to qn through *ctr (a shared
// counter per vertex, or for CL a global counter per warp round).  Returns
// (in thread 0) the sum of the tiles' degrees.
template <int B, int IPT, bool CL>
__device__ __forceinline__ unsigned long long multi_level(
    const uint32_t *__restrict__ ip, const uint32_t *__restrict__ ix, int32_t *lv,
    uint32_t n_rows, const uint32_t *qc, uint32_t *qn, uint32_t F, int32_t lvl,
    uint32_t tile0, uint32_t tstride, uint32_t *s_bitmap, uint32_t *gb, uint32_t *ctr,
    uint32_t *s_off, uint32_t *s_beg, uint32_t *s_wsum) {
  constexpr int NW = B / 32;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  unsigned long long edges = 0;
  for (uint32_t tile = tile0; tile < F; tile += tstride) {
    const uint32_t slot = tile + threadIdx.x;
    uint32_t beg = 0, deg = 0;
    if (slot < F) {
      const uint32_t u = CL ? __ldcg(qc + slot) : qc[slot];
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
          bool push = false;
          const uint32_t v = nb[u];
          if (addr[u] != kFull) {
            const uint32_t w = v >> 5, bit = 1u << (v & 31u);
            if (!(s_bitmap[w] & bit)) {
              uint32_t old;
              if (CL) {
                old = atomicOr(gb + w, bit);
                atomicOr(s_bitmap + w, bit);
              } else {
                old = atomicOr(s_bitmap + w, bit);
              }
              if (!(old & bit)) {
                lv[v] = lvl + 1;
                push = v < n_rows && ip[v + 1] > ip[v];
                // a block's own queue: one shared-memory atomic per vertex
                if (!CL && push) qn[atomicAdd(ctr, 1u)] = v;
              }
            }
          }
          if (CL) {  // a cluster's queue in global memory: one atomic per warp round
            const uint32_t pm = __ballot_sync(kFull, push);
            if (pm) {
              const uint32_t leader = __ffs(pm) - 1u;
              uint32_t base0 = 0;
              if (lane == leader) base0 = atomicAdd(ctr, (uint32_t)__popc(pm));
              base0 = __shfl_sync(kFull, base0, leader);
              if (push) qn[base0 + __popc(pm & lt_mask)] = v;
            }
          }
        }
      }
    }
    if (threadIdx.x == 0) edges += total;
    __syncthreads();
  }
  return edges;
}

// A complete BFS of one graph by one block, the visited bitmap in shared
// memory and __syncthreads as the level barrier.
template <int B, int IPT>
__device__ __forceinline__ void multi_graph_block(const MultiArgs &a, uint32_t gi,
                                                  uint32_t *s_bitmap, uint32_t *s_off,
                                                  uint32_t *s_beg, uint32_t *s_wsum,
                                                  uint32_t *s_next) {
  const MultiDesc d = a.descs[a.order[gi]];
  const uint32_t *__restrict__ ip = a.indptr_all + d.vbase;
  const uint32_t *__restrict__ ix = a.inds_all + d.ebase;
  int32_t *lv = a.levels + d.lbase;
  uint32_t *q0 = a.queues + (size_t)blockIdx.x * 2 * a.qcap;
  uint32_t *q1 = q0 + a.qcap;
  const uint32_t words = (d.n_cols + 31u) >> 5;
  for (uint32_t w = threadIdx.x; w < words; w += B) s_bitmap[w] = 0u;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t r = d.root;
    s_bitmap[r >> 5] |= 1u << (r & 31u);
    lv[r] = 0;
    const uint32_t rdeg = r < d.n_rows ? ip[r + 1] - ip[r] : 0u;
    if (rdeg) q0[0] = r;
    s_next[0] = rdeg ? 1u : 0u;
  }
  __syncthreads();
  uint32_t F = s_next[0];
  uint32_t *qc = q0, *qn = q1;
  unsigned long long edges = 0;
  int32_t lvl = 0;
  while (F > 0) {
    __syncthreads();
    if (threadIdx.x == 0) s_next[0] = 0;
    __syncthreads();
    edges += multi_level<B, IPT, false>(ip, ix, lv, d.n_rows, qc, qn, F, lvl, 0u, B, s_bitmap,
                                        nullptr, s_next, s_off, s_beg, s_wsum);
    __syncthreads();
    F = s_next[0];
    uint32_t *t = qc;
    qc = qn;
    qn = t;
    lvl++;
  }
  if (threadIdx.x == 0) a.edges_out[a.order[gi]] = edges;
}

// Graphs claimed one per block from a work counter (largest first).
template <int B, int IPT>
__device__ __forceinline__ void multi_small_graphs(const MultiArgs &a, uint32_t *s_bitmap,
                                                   uint32_t *s_off, uint32_t *s_beg,
                                                   uint32_t *s_wsum, uint32_t *s_next,
                                                   uint32_t *s_graph) {
  for (;;) {
    if (threadIdx.x == 0) *s_graph = a.n_big + atomicAdd(&a.work[0], 1u);
    __syncthreads();
    const uint32_t gi = *s_graph;
    if (gi >= a.n_graphs) break;
    multi_graph_block<B, IPT>(a, gi, s_bitmap, s_off, s_beg, s_wsum, s_next);
    __syncthreads();
  }
}

template <int B, int IPT>
__global__ void __launch_bounds__(B, 2048 / B) multi_bfs_kernel(MultiArgs a) {
  extern __shared__ uint32_t s_bitmap[];
  __shared__ uint32_t s_off[B + 1];
  __shared__ uint32_t s_beg[B];
  __shared__ uint32_t s_wsum[B / 32];
  __shared__ uint32_t s_next[1], s_graph[1];
  multi_small_graphs<B, IPT>(a, s_bitmap, s_off, s_beg, s_wsum, s_next, s_graph);
}

// Clusters of C blocks first share the largest graphs (order[0, n_big)): a
// claimed graph's frontier tiles are dealt round-robin over the cluster's
// blocks, claims go to the cluster's bitmap in global memory (L2), every
// block keeps a shared-memory copy of the visited set as a filter (merged
// from the new frontier after every level), the level barrier is the
// cluster barrier, and the next frontier is one queue per cluster with
// counters in global memory.  Then every block takes small graphs on its
// own.  Each frontier entry is expanded by exactly one block, so the edge
// counts stay exact.
template <int B, int IPT, int C>
__global__ void __cluster_dims__(C, 1, 1) __launch_bounds__(B, 2048 / B)
    multi_bfs_cluster_kernel(MultiArgs a) {
  extern __shared__ uint32_t s_bitmap[];
  __shared__ uint32_t s_off[B + 1];
  __shared__ uint32_t s_beg[B];
  __shared__ uint32_t s_wsum[B / 32];
  __shared__ uint32_t s_next[1], s_graph[1];
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t rank = cl.block_rank();
  const uint32_t cid = blockIdx.x / C;
  uint32_t *gb = a.gbits + (size_t)cid * a.gwords;
  uint32_t *cnt = a.gcnt + (size_t)cid * 4;
  uint32_t *cq0 = a.queues + (size_t)(blockIdx.x - rank) * 2 * a.qcap;
  uint32_t *cq1 = cq0 + a.qcap;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) {
      cnt[3] = atomicAdd(&a.work[1], 1u);
      cnt[0] = cnt[1] = cnt[2] = 0;
    }
    cl.sync();
    const uint32_t gi = __ldcg(cnt + 3);
    if (gi >= a.n_big) break;  // uniform over the cluster
    const MultiDesc d = a.descs[a.order[gi]];
    const uint32_t *__restrict__ ip = a.indptr_all + d.vbase;
    const uint32_t *__restrict__ ix = a.inds_all + d.ebase;
    int32_t *lv = a.levels + d.lbase;
    const uint32_t words = (d.n_cols + 31u) >> 5;
    for (uint32_t w = rank * B + threadIdx.x; w < words; w += C * B) gb[w] = 0u;
    for (uint32_t w = threadIdx.x; w < words; w += B) s_bitmap[w] = 0u;
    cl.sync();
    const uint32_t r = d.root;
    if (threadIdx.x == 0) s_bitmap[r >> 5] |= 1u << (r & 31u);
    if (rank == 0 && threadIdx.x == 0) {
      gb[r >> 5] |= 1u << (r & 31u);
      lv[r] = 0;
      const uint32_t rdeg = r < d.n_rows ? ip[r + 1] - ip[r] : 0u;
      if (rdeg) cq0[0] = r;
      cnt[0] = rdeg ? 1u : 0u;
    }
    cl.sync();
    uint32_t F = __ldcg(cnt + 0);
    unsigned long long edges = 0;
    int32_t lvl = 0;
    while (F > 0) {
      // counter (lvl + 2) % 3 held a frontier size that everyone read
      // before the previous barrier; it takes the appends of level lvl + 1
      if (rank == 0 && threadIdx.x == 0) cnt[(lvl + 2) % 3] = 0;
      uint32_t *qc = (lvl & 1) ? cq1 : cq0;
      uint32_t *qn = (lvl & 1) ? cq0 : cq1;
      uint32_t *ctr = cnt + (lvl + 1) % 3;
      edges += multi_level<B, IPT, true>(ip, ix, lv, d.n_rows, qc, qn, F, lvl, rank * B, C * B,
                                         s_bitmap, gb, ctr, s_off, s_beg, s_wsum);
      cl.sync();
      const uint32_t fn = __ldcg(ctr);
      // vertices claimed by the other blocks join this block's filter
      for (uint32_t i = threadIdx.x; i < fn; i += B) {
        const uint32_t v = __ldcg(qn + i);
        atomicOr(s_bitmap + (v >> 5), 1u << (v & 31u));
      }
      __syncthreads();
      F = fn;
      lvl++;
    }
    if (threadIdx.x == 0 && edges) atomicAdd(&a.edges_out[a.order[gi]], edges);
    cl.sync();  // queues, counters and bitmap are free for the cluster's next graph
  }
  multi_small_graphs<B, IPT>(a, s_bitmap, s_off, s_beg, s_wsum, s_next, s_graph);
}

__global__ void multi_fill_kernel(int32_t *levels, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    levels[i] = -1;
}

using MultiKernel = void (*)(MultiArgs);

struct MultiConfig {
  int block, ipt, cluster;
  MultiKernel fn;
};

static const MultiConfig kMultiConfigs[] = {
    {128, 1, 1, multi_bfs_kernel<128, 1>}, {128, 2, 1, multi_bfs_kernel<128, 2>},
    {128, 4, 1, multi_bfs_kernel<128, 4>}, {256, 1, 1, multi_bfs_kernel<256, 1>},
    {256, 2, 1, multi_bfs_kernel<256, 2>}, {256, 4, 1, multi_bfs_kernel<256, 4>},
    {512, 1, 1, multi_bfs_kernel<512, 1>}, {512, 2, 1, multi_bfs_kernel<512, 2>},
    {512, 4, 1, multi_bfs_kernel<512, 4>},
    {256, 2, 2, multi_bfs_cluster_kernel<256, 2, 2>}, {256, 4, 2, multi_bfs_cluster_kernel<256, 4, 2>},
    {512, 2, 2, multi_bfs_cluster_kernel<512, 2, 2>}, {512, 4, 2, multi_bfs_cluster_kernel<512, 4, 2>},
    {256, 2, 4, multi_bfs_cluster_kernel<256, 2, 4>}, {256, 4, 4, multi_bfs_cluster_kernel<256, 4, 4>},
    {512, 2, 4, multi_bfs_cluster_kernel<512, 2, 4>}, {512, 4, 4, multi_bfs_cluster_kernel<512, 4, 4>},
    {256, 2, 8, multi_bfs_cluster_kernel<256, 2, 8>}, {256, 4, 8, multi_bfs_cluster_kernel<256, 4, 8>},
    {512, 2, 8, multi_bfs_cluster_kernel<512, 2, 8>}, {512, 4, 8, multi_bfs_cluster_kernel<512, 4, 8>},
};
constexpr int kNumMultiConfigs = sizeof(kMultiConfigs) / sizeof(kMultiConfigs[0]);
constexpr int kNumSingleConfigs = 9;  // the first 9: one block per graph

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
  uint32_t *d_gbits = nullptr, *d_gcnt = nullptr;  // cluster bitmaps and counters
  size_t gbits_words = 0, gcnt_words = 0;
  std::vector<uint64_t> order_nnz;                   // edge counts in claim order
  uint32_t n_big = 0;
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

static int config_index(int block, int ipt, int cluster) {
  for (int i = 0; i < kNumMultiConfigs; i++)
    if (kMultiConfigs[i].block == block && kMultiConfigs[i].ipt == ipt &&
        kMultiConfigs[i].cluster == cluster)
      return i;
  return -1;
}

static bfs_status multi_prepare(bfs_multi *m, int cfg, int32_t *levels_dev) {
  if (m->exec && m->cfg == cfg && m->graph_levels == levels_dev) return BFS_OK;
  if (m->exec) cudaGraphExecDestroy(m->exec);
  if (m->graph) cudaGraphDestroy(m->graph);
  m->exec = nullptr;
  m->graph = nullptr;
  const MultiConfig &c = kMultiConfigs[cfg];
  const uint32_t words = (m->max_cols + 31) / 32;
  const size_t smem = (size_t)words * 4;
  GK(cudaFuncSetAttribute((const void *)c.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)std::max<size_t>(smem, 1)));
  int occ = 0;
  GK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)c.fn, c.block, smem));
  int grid = m->num_sms * std::max(occ, 1);
  grid = (int)std::min<size_t>((size_t)grid, m->queue_blocks);
  uint32_t n_big = 0;
  if (c.cluster > 1) {
    grid = std::max(c.cluster, grid / c.cluster * c.cluster);
    // a graph is shared by a cluster when its edges exceed `cluster` blocks'
    // fair share of the batch's edges
    for (uint32_t i = 0; i < m->n_graphs; i++)
      if ((double)m->order_nnz[i] * grid >= (double)m->total_edges * c.cluster) n_big = i + 1;
    const size_t n_clusters = (size_t)grid / c.cluster;
    if (m->gbits_words < n_clusters * words) {
      cudaFree(m->d_gbits);
      m->d_gbits = nullptr;
      GK(dev_malloc(&m->d_gbits, sizeof(uint32_t) * n_clusters * words));
      m->gbits_words = n_clusters * words;
    }
    if (m->gcnt_words < n_clusters * 4) {
      cudaFree(m->d_gcnt);
      m->d_gcnt = nullptr;
      GK(dev_malloc(&m->d_gcnt, sizeof(uint32_t) * n_clusters * 4));
      m->gcnt_words = n_clusters * 4;
    }
  } else {
    grid = std::max(1, std::min<int>(grid, (int)m->n_graphs));
  }
  m->grid = grid;
  m->n_big = n_big;
  MultiArgs a;
  a.descs = m->d_descs;
  a.order = m->d_order;
  a.n_graphs = m->n_graphs;
  a.n_big = n_big;
  a.indptr_all = m->d_indptr;
  a.inds_all = m->d_inds;
  a.work = m->d_work;
  a.queues = m->d_queues;
  a.qcap = m->max_rows;
  a.gbits = m->d_gbits;
  a.gwords = words;
  a.gcnt = m->d_gcnt;
  a.levels = levels_dev;
  a.edges_out = m->d_edges;
  // capture: reset the work counters and edge counts, fill levels with -1,
  // persistent kernel
  GK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(m->d_work, 0, 2 * sizeof(uint32_t), m->stream);
  cudaMemsetAsync(m->d_edges, 0, sizeof(unsigned long long) * m->n_graphs, m->stream);
  multi_fill_kernel<<<m->num_sms * 4, 256, 0, m->stream>>>(levels_dev, m->total_cols);
  c.fn<<<grid, c.block, smem, m->stream>>>(a);
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
  m->order_nnz.resize(n_graphs);
  for (uint32_t i = 0; i < n_graphs; i++) m->order_nnz[i] = nnz[order[i]];
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
  CK2(dev_malloc(&m->d_indptr, sizeof(uint32_t) * vb));
  CK2(dev_malloc(&m->d_inds, sizeof(uint32_t) * std::max<uint64_t>(eb, 1)));
  CK2(dev_malloc(&m->d_order, sizeof(uint32_t) * n_graphs));
  CK2(dev_malloc(&m->d_work, 2 * sizeof(uint32_t)));
  CK2(dev_malloc(&m->d_descs, sizeof(MultiDesc) * n_graphs));
  CK2(dev_malloc(&m->d_edges, sizeof(unsigned long long) * n_graphs));
  // queues: two of max_rows entries per resident block (bounded by the
  // largest occupancy of any configuration)
  m->queue_blocks = (size_t)m->num_sms * 16;
  CK2(dev_malloc(&m->d_queues, sizeof(uint32_t) * 2 * (size_t)m->max_rows * m->queue_blocks));
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
  cudaFree(m->d_gbits);
  cudaFree(m->d_gcnt);
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
  return bfs_multi_run_ex(m, roots, block, ipt, 1, levels_dev, edges_count_out, device_ms);
}

bfs_status bfs_multi_run_ex(bfs_multi *m, const uint32_t *roots, int32_t block, int32_t ipt,
                            int32_t cluster, int32_t *levels_dev, uint64_t *edges_count_out,
                            double *device_ms) {
  if (!m || !roots || !levels_dev) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  const int cfg = config_index(block, ipt, cluster);
  if (cfg < 0)
    return fail(BFS_ERR_INVALID_ARG,
                "unsupported configuration: block 128/256/512 x ipt 1/2/4 (cluster 1), or "
                "block 256/512 x ipt 2/4 x cluster 2/4/8");
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

}  // extern "C"

// Times configurations [0, n_cfg) on the batch (best of reps after a warm-up
// run that also captures the launch) and returns the fastest; a cache file
// keeps the choice per GPU, batch shape and configuration set.
static bfs_status multi_autotune(bfs_multi *m, const uint32_t *roots, int32_t *levels_dev,
                                 int32_t reps, const char *cache_path, int n_cfg, int *best_out,
                                 float *times_ms) {
  if (!m || !roots || !levels_dev) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (reps < 1) reps = 3;
  cudaDeviceProp prop;
  GK(cudaGetDeviceProperties(&prop, m->device));
  std::ostringstream key;
  key << prop.name << "|sm" << prop.multiProcessorCount << "|g" << m->n_graphs << "|v"
      << m->total_cols << "|e" << m->total_edges << "|c" << n_cfg;
  if (cache_path && cache_path[0]) {
    std::ifstream in(cache_path);
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string k;
      int b = 0, p = 0, c = 0;
      if (!std::getline(ls, k, '\t') || k != key.str()) continue;
      if (!(ls >> b >> p >> c)) continue;
      const int i = config_index(b, p, c);
      if (i >= 0 && i < n_cfg) {
        *best_out = i;
        if (times_ms)
          for (int j = 0; j < n_cfg; j++) times_ms[j] = -1.f;
        return BFS_OK;
      }
    }
  }
  int best = 0;
  float best_ms = 1e30f;
  for (int i = 0; i < n_cfg; i++) {
    const MultiConfig &c = kMultiConfigs[i];
    double t = 0.0, mn = 1e30;
    bfs_status rc = bfs_multi_run_ex(m, roots, c.block, c.ipt, c.cluster, levels_dev, nullptr,
                                     &t);  // warm-up + capture
    if (rc != BFS_OK) return rc;
    for (int r = 0; r < reps; r++) {
      rc = bfs_multi_run_ex(m, roots, c.block, c.ipt, c.cluster, levels_dev, nullptr, &t);
      if (rc != BFS_OK) return rc;
      mn = std::min(mn, t);
    }
    if (times_ms) times_ms[i] = (float)mn;
    if (mn < best_ms) {
      best_ms = (float)mn;
      best = i;
    }
  }
  *best_out = best;
  if (cache_path && cache_path[0]) {
    std::ofstream outf(cache_path, std::ios::app);
    if (outf)
      outf << key.str() << '\t' << kMultiConfigs[best].block << ' ' << kMultiConfigs[best].ipt
           << ' ' << kMultiConfigs[best].cluster << '\n';
  }
  return BFS_OK;
}

extern "C" {

bfs_status bfs_multi_autotune(bfs_multi *m, const uint32_t *roots, int32_t *levels_dev,
                              int32_t reps, const char *cache_path, int32_t *best_block,
                              int32_t *best_ipt, float *times_ms) {
  if (!best_block || !best_ipt) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  int best = 0;
  bfs_status rc = multi_autotune(m, roots, levels_dev, reps, cache_path, kNumSingleConfigs,
                                 &best, times_ms);
  if (rc != BFS_OK) return rc;
  *best_block = kMultiConfigs[best].block;
  *best_ipt = kMultiConfigs[best].ipt;
  return BFS_OK;
}

bfs_status bfs_multi_autotune_ex(bfs_multi *m, const uint32_t *roots, int32_t *levels_dev,
                                 int32_t reps, const char *cache_path, int32_t *best_block,
                                 int32_t *best_ipt, int32_t *best_cluster, float *times_ms) {
  if (!best_block || !best_ipt || !best_cluster) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  int best = 0;
  bfs_status rc = multi_autotune(m, roots, levels_dev, reps, cache_path, kNumMultiConfigs,
                                 &best, times_ms);
  if (rc != BFS_OK) return rc;
  *best_block = kMultiConfigs[best].block;
  *best_ipt = kMultiConfigs[best].ipt;
  *best_cluster = kMultiConfigs[best].cluster;
  return BFS_OK;
}

int32_t bfs_multi_num_configs(int32_t *blocks, int32_t *ipts, int32_t *clusters, int32_t max) {
  for (int i = 0; i < kNumMultiConfigs && i < max; i++) {
    if (blocks) blocks[i] = kMultiConfigs[i].block;
    if (ipts) ipts[i] = kMultiConfigs[i].ipt;
    if (clusters) clusters[i] = kMultiConfigs[i].cluster;
  }
  return kNumMultiConfigs;
}

}  // extern "C"
