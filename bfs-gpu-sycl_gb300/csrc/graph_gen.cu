// graph_gen.cu -- seeded synthetic graphs in the reference's CSC layout.
//
// The reference builds its datasets offline with networkit's R-MAT generator
// and scipy (scripts/genGraph.py:41-64, scripts/generator.py:211-245, :94-98).
// Those tools are not part of the hot path and their output is not seeded,
// so this engine generates its own graphs: every edge is a pure function of
// (seed, edge index) through a counter-based hash (bfs_internal.h), which
// makes the host builder and the device builder produce the same CSC bytes.
//
// CSC conventions match scripts/generator.py:115-147: uint32 indptr of
// n + 1 entries, uint32 destination ids sorted within each vertex, no
// duplicates (scipy's csr_matrix sums duplicates into one structural entry).
#include <cuda_runtime.h>
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "bfs_internal.h"
#include "dev_alloc.h"

namespace bfsgb {
bfs_status graph_from_owned_device(uint32_t *d_indptr, uint32_t *d_inds,
                                   uint32_t n_rows, uint32_t n_cols,
                                   uint64_t nnz, bfs_graph **out);
bfs_status graph_download_impl(const bfs_graph *g, bfs_csc_host *out);
}  // namespace bfsgb

using namespace bfsgb;

namespace {

int host_threads() {
  unsigned n = std::thread::hardware_concurrency();
  if (n == 0) n = 1;
  if (n > 64) n = 64;
  return (int)n;
}

template <typename F>
void parallel_for(uint64_t n, F &&fn) {
  int nt = host_threads();
  if (n < 4096 || nt == 1) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  uint64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    uint64_t b = (uint64_t)t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back([&fn, b, e] { fn(b, e); });
  }
  for (auto &x : th) x.join();
}

uint32_t to_fixed32(double p) {
  if (p <= 0.0) return 0;
  if (p >= 1.0) return 0xFFFFFFFFu;
  return (uint32_t)std::floor(p * 4294967296.0);
}

bool rmat_params(uint32_t scale, uint32_t edge_factor, double a, double b,
                 double c, uint64_t seed, RmatParams *p) {
  if (scale < 1 || scale > 30 || edge_factor < 1) return false;
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0 + 1e-12) return false;
  p->scale = scale;
  p->n_edges = (uint64_t)edge_factor << scale;
  p->seed_mixed = mix64(seed);
  p->t_a = to_fixed32(a);
  p->t_ab = to_fixed32(a + b);
  p->t_abc = to_fixed32(a + b + c);
  return true;
}

// Builds a de-duplicated CSC from a pure edge function: edge(i, &u, &v)
// returns false for a dropped edge.  Two passes over the edge stream
// (count, scatter), then every adjacency list is sorted and de-duplicated.
template <typename EdgeFn>
bfs_status build_csc(uint32_t n, uint64_t m, bool symmetrize, EdgeFn edge,
                     bfs_csc_host *out) {
  std::vector<uint64_t> deg(n + 1, 0);
  std::vector<uint32_t> cnt(n, 0);
  parallel_for(m, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; i++) {
      uint32_t u, v;
      if (!edge(i, &u, &v) || u == v) continue;
      __atomic_fetch_add(&cnt[u], 1u, __ATOMIC_RELAXED);
      if (symmetrize) __atomic_fetch_add(&cnt[v], 1u, __ATOMIC_RELAXED);
    }
  });
  for (uint32_t v = 0; v < n; v++) deg[v + 1] = deg[v] + cnt[v];
  uint64_t raw = deg[n];
  std::vector<uint32_t> buf;
  try {
    buf.resize(raw);
  } catch (...) {
    return fail(BFS_ERR_OOM, "host allocation failed while building CSC");
  }
  std::vector<uint64_t> cursor(deg.begin(), deg.end() - 1);
  parallel_for(m, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; i++) {
      uint32_t u, v;
      if (!edge(i, &u, &v) || u == v) continue;
      buf[__atomic_fetch_add(&cursor[u], 1ull, __ATOMIC_RELAXED)] = v;
      if (symmetrize)
        buf[__atomic_fetch_add(&cursor[v], 1ull, __ATOMIC_RELAXED)] = u;
    }
  });
  // sort + unique per row, record unique counts
  parallel_for(n, [&](uint64_t b, uint64_t e) {
    for (uint64_t v = b; v < e; v++) {
      uint32_t *s = buf.data() + deg[v], *t = buf.data() + deg[v + 1];
      std::sort(s, t);
      cnt[v] = (uint32_t)(std::unique(s, t) - s);
    }
  });
  uint64_t nnz = 0;
  for (uint32_t v = 0; v < n; v++) nnz += cnt[v];
  if (nnz > BFS_MAX_EDGES)
    return fail(BFS_ERR_UNSUPPORTED, "graph has more than BFS_MAX_EDGES edges");
  out->n_rows = out->n_cols = n;
  out->nnz = nnz;
  out->indptr = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  out->inds = (uint32_t *)malloc(sizeof(uint32_t) * (nnz ? nnz : 1));
  if (!out->indptr || !out->inds) {
    free(out->indptr);
    free(out->inds);
    out->indptr = out->inds = nullptr;
    return fail(BFS_ERR_OOM, "host allocation failed for CSC output");
  }
  out->indptr[0] = 0;
  for (uint32_t v = 0; v < n; v++) out->indptr[v + 1] = out->indptr[v] + cnt[v];
  parallel_for(n, [&](uint64_t b, uint64_t e) {
    for (uint64_t v = b; v < e; v++)
      std::memcpy(out->inds + out->indptr[v], buf.data() + deg[v],
                  sizeof(uint32_t) * cnt[v]);
  });
  return BFS_OK;
}

// ---- device R-MAT builder ---------------------------------------------------
__global__ void rmat_keys_kernel(RmatParams p, int symmetrize,
                                 unsigned long long *keys) {
  const uint64_t sent = (1ull << (2 * p.scale)) - 1ull;  // (n-1, n-1): a self-loop
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_edges;
       i += stride) {
    uint32_t u, v;
    rmat_edge(p, i, &u, &v);
    uint64_t k0 = sent, k1 = sent;
    if (u != v) {
      k0 = ((uint64_t)u << p.scale) | v;
      k1 = ((uint64_t)v << p.scale) | u;
    }
    if (symmetrize) {
      keys[2 * i] = k0;
      keys[2 * i + 1] = k1;
    } else {
      keys[i] = k0;
    }
  }
}

// indptr[v] = first key with source >= v; inds[k] = destination of key k.
__global__ void csc_from_keys_kernel(const unsigned long long *keys, uint64_t nnz,
                                     uint32_t scale, uint32_t n,
                                     uint32_t *indptr, uint32_t *inds) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t lo_mask = (1ull << scale) - 1ull;
  for (uint64_t k = tid; k < nnz; k += stride) inds[k] = (uint32_t)(keys[k] & lo_mask);
  for (uint64_t v = tid; v <= n; v += stride) {
    uint64_t target = (uint64_t)v << scale;
    uint64_t lo = 0, hi = nnz;
    while (lo < hi) {
      uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < target) lo = mid + 1; else hi = mid;
    }
    indptr[v] = (uint32_t)lo;
  }
}

}  // namespace

extern "C" {

void bfs_csc_host_free(bfs_csc_host *g) {
  if (!g) return;
  free(g->indptr);
  free(g->inds);
  g->indptr = g->inds = nullptr;
  g->nnz = 0;
  g->n_rows = g->n_cols = 0;
}

bfs_status bfs_gen_rmat_host(uint32_t scale, uint32_t edge_factor, double a,
                             double b, double c, uint64_t seed, int symmetrize,
                             bfs_csc_host *out) {
  RmatParams p;
  if (!out || !rmat_params(scale, edge_factor, a, b, c, seed, &p))
    return fail(BFS_ERR_INVALID_ARG, "bad R-MAT parameters");
  std::memset(out, 0, sizeof(*out));
  return build_csc(1u << scale, p.n_edges, symmetrize != 0,
                   [&](uint64_t i, uint32_t *u, uint32_t *v) {
                     rmat_edge(p, i, u, v);
                     return true;
                   },
                   out);
}

bfs_status bfs_gen_er_host(uint32_t n, double avg_degree, uint64_t seed,
                           bfs_csc_host *out) {
  if (!out || n < 2 || !(avg_degree > 0.0))
    return fail(BFS_ERR_INVALID_ARG, "bad Erdos-Renyi parameters");
  std::memset(out, 0, sizeof(*out));
  uint64_t m = (uint64_t)std::llround((double)n * avg_degree / 2.0);
  uint64_t sm = mix64(seed);
  return build_csc(n, m, true,
                   [&](uint64_t i, uint32_t *u, uint32_t *v) {
                     *u = hash_to_range(hash3(sm, i, 0), n);
                     *v = hash_to_range(hash3(sm, i, 1), n);
                     return true;
                   },
                   out);
}

bfs_status bfs_gen_grid_host(uint32_t width, uint32_t height, double delete_prob,
                             uint64_t seed, bfs_csc_host *out) {
  if (!out || width < 1 || height < 1 || delete_prob < 0.0 || delete_prob > 1.0)
    return fail(BFS_ERR_INVALID_ARG, "bad grid parameters");
  uint64_t n64 = (uint64_t)width * height;
  if (n64 > 0xFFFFFFFEull) return fail(BFS_ERR_INVALID_ARG, "grid too large");
  std::memset(out, 0, sizeof(*out));
  const uint32_t n = (uint32_t)n64;
  const uint64_t sm = mix64(seed);
  const uint32_t thr = to_fixed32(delete_prob);
  const uint64_t n_horiz = (uint64_t)(width - 1) * height;
  // Undirected edge ids: horizontal (x,y)-(x+1,y) -> y*(W-1)+x,
  // vertical (x,y)-(x,y+1) -> n_horiz + y*W + x.  Kept iff draw >= thr.
  auto keep = [&](uint64_t eid) {
    return (uint32_t)hash3(sm, eid, 0) >= thr;
  };
  std::vector<uint32_t> cnt(n, 0);
  auto nbrs = [&](uint32_t v, uint32_t *list) {
    uint32_t x = v % width, y = v / width, k = 0;
    if (y > 0 && keep(n_horiz + (uint64_t)(y - 1) * width + x)) list[k++] = v - width;
    if (x > 0 && keep((uint64_t)y * (width - 1) + x - 1)) list[k++] = v - 1;
    if (x + 1 < width && keep((uint64_t)y * (width - 1) + x)) list[k++] = v + 1;
    if (y + 1 < height && keep(n_horiz + (uint64_t)y * width + x)) list[k++] = v + width;
    return k;
  };
  parallel_for(n, [&](uint64_t b, uint64_t e) {
    uint32_t tmp[4];
    for (uint64_t v = b; v < e; v++) cnt[v] = nbrs((uint32_t)v, tmp);
  });
  out->n_rows = out->n_cols = n;
  out->indptr = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  if (!out->indptr) return fail(BFS_ERR_OOM, "host allocation failed");
  out->indptr[0] = 0;
  for (uint32_t v = 0; v < n; v++) out->indptr[v + 1] = out->indptr[v] + cnt[v];
  out->nnz = out->indptr[n];
  out->inds = (uint32_t *)malloc(sizeof(uint32_t) * (out->nnz ? out->nnz : 1));
  if (!out->inds) {
    bfs_csc_host_free(out);
    return fail(BFS_ERR_OOM, "host allocation failed");
  }
  parallel_for(n, [&](uint64_t b, uint64_t e) {
    for (uint64_t v = b; v < e; v++) nbrs((uint32_t)v, out->inds + out->indptr[v]);
  });
  return BFS_OK;
}

bfs_status bfs_gen_rmat_device(uint32_t scale, uint32_t edge_factor, double a,
                               double b, double c, uint64_t seed, int symmetrize,
                               bfs_graph **out) {
  RmatParams p;
  if (!out || !rmat_params(scale, edge_factor, a, b, c, seed, &p))
    return fail(BFS_ERR_INVALID_ARG, "bad R-MAT parameters");
  *out = nullptr;
  const uint64_t nk = symmetrize ? 2 * p.n_edges : p.n_edges;
  const uint32_t n = 1u << scale;
  unsigned long long *k0 = nullptr, *k1 = nullptr, *d_nsel = nullptr;
  void *tmp = nullptr;
  uint32_t *indptr = nullptr, *inds = nullptr;
  cudaStream_t st = nullptr;
  bfs_status rc = BFS_OK;
  size_t tmp_sort = 0, tmp_uniq = 0;
  uint64_t nsel = 0, nnz = 0;
  int bits = 2 * (int)scale;
#define GEN_CHECK(x, what)                                           \
  do {                                                               \
    cudaError_t e_ = (x);                                            \
    if (e_ != cudaSuccess) {                                         \
      rc = fail(e_ == cudaErrorMemoryAllocation ? BFS_ERR_OOM        \
                                                : BFS_ERR_CUDA,      \
                std::string(what) + ": " + cudaGetErrorString(e_)); \
      goto done;                                                     \
    }                                                                \
  } while (0)
  GEN_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
  GEN_CHECK(dev_malloc(&k0, nk * sizeof(unsigned long long)), "keys");
  GEN_CHECK(dev_malloc(&k1, nk * sizeof(unsigned long long)), "keys");
  GEN_CHECK(dev_malloc(&d_nsel, sizeof(unsigned long long)), "count");
  {
    cub::DoubleBuffer<unsigned long long> db(k0, k1);
    GEN_CHECK(cub::DeviceRadixSort::SortKeys(nullptr, tmp_sort, db, (int64_t)nk, 0,
                                             bits, st),
              "sort sizing");
    GEN_CHECK(cub::DeviceSelect::Unique(nullptr, tmp_uniq, k0, k1, d_nsel,
                                        (int64_t)nk, st),
              "unique sizing");
    GEN_CHECK(dev_malloc(&tmp, std::max(tmp_sort, tmp_uniq)), "cub temp");
    rmat_keys_kernel<<<2048, 256, 0, st>>>(p, symmetrize, k0);
    GEN_CHECK(cudaGetLastError(), "rmat keys");
    size_t ts = tmp_sort;
    GEN_CHECK(cub::DeviceRadixSort::SortKeys(tmp, ts, db, (int64_t)nk, 0, bits, st),
              "sort");
    unsigned long long *sorted = db.Current(), *uniq = db.Alternate();
    size_t tu = tmp_uniq;
    GEN_CHECK(cub::DeviceSelect::Unique(tmp, tu, sorted, uniq, d_nsel, (int64_t)nk, st),
              "unique");
    GEN_CHECK(cudaMemcpyAsync(&nsel, d_nsel, sizeof(nsel), cudaMemcpyDeviceToHost, st),
              "count copy");
    GEN_CHECK(cudaStreamSynchronize(st), "generate");
    // the self-loop sentinel sorts last; drop it if present
    nnz = nsel;
    if (nnz > 0) {
      unsigned long long last = 0;
      GEN_CHECK(cudaMemcpy(&last, uniq + nnz - 1, sizeof(last), cudaMemcpyDeviceToHost),
                "tail copy");
      if (last == (1ull << bits) - 1ull) nnz--;
    }
    if (nnz > BFS_MAX_EDGES) {
      rc = fail(BFS_ERR_UNSUPPORTED, "graph has more than BFS_MAX_EDGES edges");
      goto done;
    }
    GEN_CHECK(dev_malloc(&indptr, sizeof(uint32_t) * ((size_t)n + 1)), "indptr");
    GEN_CHECK(dev_malloc(&inds, sizeof(uint32_t) * (nnz ? nnz : 1)), "inds");
    csc_from_keys_kernel<<<4096, 256, 0, st>>>(uniq, nnz, scale, n, indptr, inds);
    GEN_CHECK(cudaGetLastError(), "csc build");
    GEN_CHECK(cudaStreamSynchronize(st), "csc build");
  }
  rc = graph_from_owned_device(indptr, inds, n, n, nnz, out);
  if (rc == BFS_OK) indptr = inds = nullptr;  // owned by the handle now
done:
#undef GEN_CHECK
  if (st) cudaStreamSynchronize(st);
  cudaFree(k0);
  cudaFree(k1);
  cudaFree(d_nsel);
  cudaFree(tmp);
  cudaFree(indptr);
  cudaFree(inds);
  if (st) cudaStreamDestroy(st);
  return rc;
}

bfs_status bfs_graph_download(const bfs_graph *g, bfs_csc_host *out) {
  return graph_download_impl(g, out);
}

bfs_status bfs_sample_roots(const uint32_t *indptr, uint32_t n_rows, uint32_t count,
                            uint64_t seed, uint32_t *roots_out) {
  if (!indptr || (!roots_out && count)) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (count == 0) return BFS_OK;
  uint64_t eligible = 0;
  for (uint32_t v = 0; v < n_rows; v++) eligible += indptr[v + 1] > indptr[v];
  if (eligible < count)
    return fail(BFS_ERR_GRAPH, "fewer vertices with out-degree > 0 than roots requested");
  const uint64_t sm = mix64(seed ^ 0x726F6F7473ull);  // "roots"
  std::vector<uint32_t> chosen;
  chosen.reserve(count);
  for (uint64_t j = 0; chosen.size() < count; j++) {
    uint32_t v = hash_to_range(hash3(sm, j, 0), n_rows);
    if (indptr[v + 1] == indptr[v]) continue;
    if (std::find(chosen.begin(), chosen.end(), v) != chosen.end()) continue;
    chosen.push_back(v);
  }
  std::memcpy(roots_out, chosen.data(), sizeof(uint32_t) * count);
  return BFS_OK;
}

}  // extern "C"
