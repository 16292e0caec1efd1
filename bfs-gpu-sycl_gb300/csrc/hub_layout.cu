// hub_layout.cu -- the degree-ordered hub layout of a graph handle.
//
// In a top-down BFS every edge costs one probe of the visited bitmap, a
// random 4-byte gather over an n/8-byte bitmap, and on power-law graphs most
// of the edges of the large levels point at a few high in-degree vertices
// ("hubs") that were reached levels earlier.  The hub layout gives the
// explore kernel a cheap test for exactly those probes: the graph is
// relabelled so that internal ids 0 .. K-1 are the K vertices of highest
// in-degree, in that order, and the explore kernel keeps bits 0 .. K-1 of
// the visited bitmap in shared memory.  A probe of a hub already visited is
// then answered by shared memory; every other probe goes to the bitmap in
// global memory as before, so levels stay exact.
//
// Relabelling (a permutation perm: internal -> original, pinv its inverse):
//   internal i < K              -> the i-th vertex by in-degree (ties by id)
//   internal v >= K, original position of a hub
//                               -> a non-hub whose original id was < K
//                                  (the displaced and vacated ids are paired
//                                  in increasing order)
//   every other v               -> itself
// so outside the hub prefix almost every vertex keeps its id (and the
// locality of the original numbering).  The relabelled CSC lists, for
// internal vertex i, the out-neighbours of perm[i] mapped through pinv.
// Level and parent arrays are still written in original ids (the level
// generation kernel writes level[perm[v]]), so callers see no difference.
//
// A graph whose K highest in-degree vertices take less than a quarter of all
// edge endpoints (grids, uniform random graphs) gets no layout at all: the
// prefix would catch few probes, and the copy would cost memory and the
// shared-memory copy time for nothing.
//
// Graphs with n_cols <= K need no relabelling: the whole bitmap fits in
// shared memory and the layout is the identity (no copy).  Graphs with
// n_rows < n_cols keep the identity too (a relabelling could move a vertex
// across the n_rows boundary, which decides whether it is expanded); their
// shared-memory prefix is then simply the first K original ids.
#include <cuda_runtime.h>
#include <cub/cub.cuh>

#include <algorithm>
#include <string>

#include "bfs_internal.h"
#include "dev_alloc.h"
#include "engine.h"
#include "hub_layout.h"

namespace bfsgb {
namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;

__global__ void indeg_kernel(const uint32_t *__restrict__ inds, uint64_t nnz, uint32_t *indeg) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride)
    atomicAdd(indeg + inds[e], 1u);
}

__global__ void init_perm_kernel(uint32_t n, uint32_t *iota, uint32_t *perm, uint32_t *pinv) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    iota[v] = v;
    perm[v] = v;
    pinv[v] = kNone;
  }
}

// Sum of the K largest in-degrees (the edge endpoints the prefix covers).
__global__ void top_sum_kernel(const uint32_t *__restrict__ sorted_deg, uint32_t K,
                               unsigned long long *sum) {
  unsigned long long t = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x)
    t += sorted_deg[i];
  for (int d = 16; d > 0; d >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, d);
  if ((threadIdx.x & 31u) == 0 && t) atomicAdd(sum, t);
}

// internal i < K takes the i-th vertex by in-degree
__global__ void place_hubs_kernel(const uint32_t *__restrict__ by_degree, uint32_t K,
                                  uint32_t *perm, uint32_t *pinv) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += stride) {
    const uint32_t h = by_degree[i];
    perm[i] = h;
    pinv[h] = i;
  }
}

// displaced: non-hubs with original id < K; vacated: hub ids >= K
__global__ void flags_kernel(const uint32_t *__restrict__ pinv, uint32_t K, uint32_t n,
                             uint8_t *displaced, uint8_t *vacated) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += stride) {
    const bool hub = pinv[v] != kNone;
    displaced[v] = (v < K && !hub) ? 1 : 0;
    vacated[v] = (v >= K && hub) ? 1 : 0;
  }
}

__global__ void pair_kernel(const uint32_t *__restrict__ displaced,
                            const uint32_t *__restrict__ vacated, const uint32_t *count,
                            uint32_t *perm, uint32_t *pinv) {
  const uint32_t m = *count;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) {
    perm[vacated[j]] = displaced[j];
    pinv[displaced[j]] = vacated[j];
  }
}

__global__ void finish_pinv_kernel(uint32_t n, uint32_t *pinv, const uint32_t *__restrict__ indptr,
                                   const uint32_t *__restrict__ perm, uint32_t *deg) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += stride) {
    if (v < n && pinv[v] == kNone) pinv[v] = v;
    deg[v] = v < n ? indptr[perm[v] + 1] - indptr[perm[v]] : 0u;
  }
}

// Bit v of `moved` is set when perm[v] != v (one ballot per 32 vertices).
__global__ void moved_kernel(const uint32_t *__restrict__ perm, uint32_t n, uint32_t words,
                             uint32_t *moved) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < words * 32u; v += stride) {
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, v < n && perm[v] != v);
    if ((threadIdx.x & 31u) == 0) moved[v >> 5] = m;
  }
}

// One warp per internal vertex: its list is the original list of perm[i],
// every destination mapped through pinv.
__global__ void relabel_kernel(const uint32_t *__restrict__ indptr,
                               const uint32_t *__restrict__ inds,
                               const uint32_t *__restrict__ perm,
                               const uint32_t *__restrict__ pinv,
                               const uint32_t *__restrict__ indptr_h, uint32_t n,
                               uint32_t *inds_h) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint32_t src = perm[i];
    const uint32_t b = indptr[src], d = indptr[src + 1] - b, o = indptr_h[i];
    for (uint32_t j = lane; j < d; j += 32u) inds_h[o + j] = pinv[inds[b + j]];
  }
}

}  // namespace

void free_hub(bfs_graph *g) {
  HubLayout *h = g->hub;
  if (!h) return;
  if (h->relabelled) {
    cudaFree(h->indptr);
    cudaFree(h->inds);
    cudaFree(h->perm);
    cudaFree(h->pinv);
    cudaFree(h->moved);
  }
  delete h;
  g->hub = nullptr;
}

uint32_t hub_max_vertices(const bfs_graph *g, size_t static_bytes) {
  // dynamic shared memory of the explore kernel: what the device allows a
  // block beside the kernel's static arrays, in whole 16-byte rows
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, g->device) !=
          cudaSuccess ||
      optin <= 0 || (size_t)optin <= static_bytes + 1024) {
    cudaGetLastError();
    return 0;
  }
  const size_t bytes = (size_t)optin - static_bytes - 1024;
  return (uint32_t)(bytes * 8 / 128 * 128);
}

bfs_status build_hub(bfs_graph *g, uint32_t K) {
  free_hub(g);
  if (K == 0) return BFS_OK;
  const uint32_t n = g->n_cols;
  HubLayout *h = new (std::nothrow) HubLayout();
  if (!h) return fail(BFS_ERR_OOM, "host allocation failed");
  h->indptr = g->indptr;
  h->inds = g->inds;
  // identity for small graphs, graphs whose rows are not all expanded and
  // graphs of 2^31 vertices or more (level generation marks moved ids in
  // bit 31 of its vertex lists)
  if (n <= K || g->n_rows != n || n > 0x80000000u) {
    // identity: the prefix is the first min(K, all) original ids
    const uint32_t bits = (uint32_t)std::min<uint64_t>((uint64_t)K, (uint64_t)g->words * 32u);
    h->vertices = bits / 128u * 128u;
    h->relabelled = false;
    g->hub = h;
    return BFS_OK;
  }
  h->vertices = K;
  h->relabelled = true;  // from here on the arrays below are the layout's own
  h->indptr = h->inds = nullptr;
  cudaStream_t s = g->stream;
  uint32_t *indeg = nullptr, *iota = nullptr, *sorted_deg = nullptr, *by_degree = nullptr;
  uint32_t *list_d = nullptr, *list_v = nullptr, *count = nullptr, *deg = nullptr;
  unsigned long long *cover = nullptr, h_cover = 0;
  bool flat = false;
  uint8_t *flags = nullptr;
  void *tmp = nullptr;
  size_t tmp_bytes = 0, t_sort = 0, t_sel = 0, t_scan = 0;
  cudaError_t e = cudaSuccess;
  const int grid = g->num_sms * 8;
#define HUB_CK(x)                    \
  do {                               \
    e = (x);                         \
    if (e != cudaSuccess) goto done; \
  } while (0)
  HUB_CK(dev_malloc(&h->perm, sizeof(uint32_t) * (size_t)n));
  HUB_CK(dev_malloc(&h->pinv, sizeof(uint32_t) * (size_t)n));
  HUB_CK(dev_malloc(&h->moved, sizeof(uint32_t) * (size_t)g->words));
  HUB_CK(dev_malloc(&h->indptr, sizeof(uint32_t) * ((size_t)n + 1)));
  HUB_CK(dev_malloc(&h->inds, sizeof(uint32_t) * (g->nnz ? g->nnz : 1)));
  HUB_CK(dev_malloc(&indeg, sizeof(uint32_t) * (size_t)n));
  HUB_CK(dev_malloc(&iota, sizeof(uint32_t) * (size_t)n));
  HUB_CK(dev_malloc(&sorted_deg, sizeof(uint32_t) * (size_t)n));
  HUB_CK(dev_malloc(&by_degree, sizeof(uint32_t) * (size_t)n));
  HUB_CK(dev_malloc(&list_d, sizeof(uint32_t) * (size_t)K));
  HUB_CK(dev_malloc(&list_v, sizeof(uint32_t) * (size_t)K));
  HUB_CK(dev_malloc(&count, sizeof(uint32_t) * 2));
  HUB_CK(dev_malloc(&cover, sizeof(unsigned long long)));
  HUB_CK(dev_malloc(&deg, sizeof(uint32_t) * ((size_t)n + 1)));
  HUB_CK(dev_malloc(&flags, 2 * (size_t)n));
  HUB_CK(cub::DeviceRadixSort::SortPairsDescending(nullptr, t_sort, indeg, sorted_deg, iota,
                                                   by_degree, (int64_t)n, 0, 32, s));
  HUB_CK(cub::DeviceSelect::Flagged(nullptr, t_sel, iota, flags, list_d, count, (int64_t)n, s));
  HUB_CK(cub::DeviceScan::ExclusiveSum(nullptr, t_scan, deg, h->indptr, (int64_t)n + 1, s));
  tmp_bytes = std::max(t_sort, std::max(t_sel, t_scan));
  HUB_CK(dev_malloc(&tmp, tmp_bytes));

  HUB_CK(cudaMemsetAsync(indeg, 0, sizeof(uint32_t) * (size_t)n, s));
  indeg_kernel<<<grid, 256, 0, s>>>(g->inds, g->nnz, indeg);
  init_perm_kernel<<<grid, 256, 0, s>>>(n, iota, h->perm, h->pinv);
  HUB_CK(cudaGetLastError());
  // stable radix sort: equal in-degrees keep increasing ids
  {
    size_t t = tmp_bytes;
    HUB_CK(cub::DeviceRadixSort::SortPairsDescending(tmp, t, indeg, sorted_deg, iota, by_degree,
                                                     (int64_t)n, 0, 32, s));
  }
  HUB_CK(cudaMemsetAsync(cover, 0, sizeof(unsigned long long), s));
  top_sum_kernel<<<grid, 256, 0, s>>>(sorted_deg, K, cover);
  HUB_CK(cudaMemcpyAsync(&h_cover, cover, sizeof(h_cover), cudaMemcpyDeviceToHost, s));
  HUB_CK(cudaStreamSynchronize(s));
  if (h_cover * 4ull < g->nnz) {
    flat = true;  // no hubs to speak of: no layout
    goto done;
  }
  place_hubs_kernel<<<grid, 256, 0, s>>>(by_degree, K, h->perm, h->pinv);
  flags_kernel<<<grid, 256, 0, s>>>(h->pinv, K, n, flags, flags + n);
  HUB_CK(cudaGetLastError());
  {
    size_t t = tmp_bytes;
    HUB_CK(cub::DeviceSelect::Flagged(tmp, t, iota, flags, list_d, count, (int64_t)n, s));
    t = tmp_bytes;
    HUB_CK(cub::DeviceSelect::Flagged(tmp, t, iota, flags + n, list_v, count + 1, (int64_t)n, s));
  }
  pair_kernel<<<grid, 256, 0, s>>>(list_d, list_v, count, h->perm, h->pinv);
  finish_pinv_kernel<<<grid, 256, 0, s>>>(n, h->pinv, g->indptr, h->perm, deg);
  moved_kernel<<<grid, 256, 0, s>>>(h->perm, n, g->words, h->moved);
  HUB_CK(cudaGetLastError());
  {
    size_t t = tmp_bytes;
    HUB_CK(cub::DeviceScan::ExclusiveSum(tmp, t, deg, h->indptr, (int64_t)n + 1, s));
  }
  relabel_kernel<<<grid, 256, 0, s>>>(g->indptr, g->inds, h->perm, h->pinv, h->indptr, n, h->inds);
  HUB_CK(cudaGetLastError());
  {
    uint32_t hc[2] = {0, 0};
    HUB_CK(cudaMemcpyAsync(hc, count, sizeof(hc), cudaMemcpyDeviceToHost, s));
    HUB_CK(cudaStreamSynchronize(s));
    if (hc[0] != hc[1]) {
      e = cudaErrorUnknown;  // the two lists must pair up exactly
      goto done;
    }
  }
done:
#undef HUB_CK
  cudaStreamSynchronize(s);
  cudaFree(indeg);
  cudaFree(iota);
  cudaFree(sorted_deg);
  cudaFree(by_degree);
  cudaFree(list_d);
  cudaFree(list_v);
  cudaFree(count);
  cudaFree(cover);
  cudaFree(deg);
  cudaFree(flags);
  cudaFree(tmp);
  if (e != cudaSuccess || flat) {
    cudaGetLastError();
    g->hub = h;  // frees the layout's own arrays, never the graph's
    free_hub(g);
    if (flat) return BFS_OK;
    if (e == cudaErrorMemoryAllocation) return BFS_OK;  // no layout: plain kernels
    return fail(BFS_ERR_CUDA, std::string("hub layout: ") + cudaGetErrorString(e));
  }
  g->hub = h;
  return BFS_OK;
}

}  // namespace bfsgb
