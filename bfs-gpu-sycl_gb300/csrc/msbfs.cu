// msbfs.cu -- batched multi-source BFS, 64 roots per uint64 lane.
//
// The reference runs one root per invocation (src/host.cpp:72, :146-150) and
// re-uploads the graph every run (src/run_bfs_gpu.hpp:620-670).  Here up to 64
// roots share every level: each vertex carries a 64-bit visited mask (bit j =
// reached by root j) and the frontier queue carries, per entry, the mask of
// roots whose frontier contains it.  One traversal of an edge u->v serves every
// root whose frontier holds u:  visited[v] |= mask(u) & ~visited[v], the test
// reading the mask as the level is being explored, so that a root already
// given to v by another edge costs no atomic.
// Level generation compares visited[] with its copy as of the previous level
// (prev[]) to get the new frontier and records, per level, the mask of roots
// that reached each vertex; an expansion kernel
// writes each root's int32 level row once, coalesced, from those masks, and
// each root's edgesCount (sum of degrees of the vertices that root expands,
// run_bfs_cpu.hpp:36), so every row is exactly the single-root level array
// of its root.
//
//   explore   edge-balanced like the GLB form: a warp takes a chunk of the
//             frontier's edges, finds the owner of its first edge with a 32-ary
//             search of the degree prefix, then takes each owner's first edge
//             and root mask from shuffles of coalesced loads.
//   levelgen  one vertex per lane: new = visited[v] & ~prev[v], stored as
//             hist[L][v] for the first kHistLevels levels (one coalesced 8-byte
//             store per vertex; level rows written level by level would be
//             scattered partial-sector stores, which HBM turns into
//             read-modify-writes); kept vertices are compacted with
//             ballot/popc and one atomic per block.
//   expand    one warp per 32 vertices writes every root's 32 level entries
//             as one 128-byte segment (-1 where unreached), once per pass; if
//             the search goes past the history it runs at that point and the
//             deeper levels are stored into the rows directly.
//   loop      a CUDA graph with a conditional WHILE node, as for one root.
//
// With the graph handle's hub layout (hub_layout.cu) the batch runs on the
// relabelled graph, whose internal ids 0 .. K-1 are the K highest in-degree
// vertices: level generation also writes a bitmap of the first (at most
// kMsHubMax) hub ids every root of the pass has reached (hubfull), explore
// copies it into shared memory on large levels and skips the 8-byte mask
// probe of those targets -- on power-law graphs many edges of the later
// levels point at them, and the mask array is larger than L2, so each probe
// skipped is a DRAM sector saved.  Rows are written in original ids (expand reads the internal state
// through pinv).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "bfs_internal.h"
#include "dev_alloc.h"
#include "device_util.cuh"
#include "engine.h"
#include "hub_layout.h"
#include "kernels.h"

namespace bfsgb {

constexpr int kLanes = 64;
constexpr int kMsBlock = 256;
constexpr int kMsU = 4;
constexpr uint32_t kMsChunk = 32u * kMsU * 4u;
// Levels kept as per-vertex root masks before the rows are written.
constexpr uint32_t kHistLevels = 16;
// Largest hub prefix the batched explore filters on (vertices): six blocks per
// SM each hold a copy, and every byte of it is taken from the L1 capacity the
// mask and queue loads need (RMAT-25 64-root pass: 24.5 ms without a filter,
// 23.6 ms with 32 K, 36.6 ms with 256 K).  The layout is in degree order, so
// its first 32 K ids are the top hubs whatever its own size.
constexpr uint32_t kMsHubMax = 1u << 15;

struct MsState {
  const uint32_t *indptr;
  const uint32_t *inds;
  uint32_t n_rows, n_cols;
  unsigned long long *vis;
  unsigned long long *prev;  // vis as of the previous level
  unsigned long long *hist;  // kHistLevels arrays of n_cols masks
  uint32_t *qb[2];
  uint32_t *qp[2];
  unsigned long long *qm[2];
  int32_t *level;  // n_lanes rows of n_cols
  // hub layout (null: identity ids, no filter)
  const uint32_t *perm, *pinv, *moved;
  uint32_t *hubfull;       // bit v (v < 32 hub_words): every root has reached v
  uint32_t hub_words;      // words of hubfull (0: no filter)
  uint32_t hub_min_edges;  // frontier edges from which explore loads it
  uint32_t n_lanes;
  uint32_t roots[kLanes];
  unsigned long long next_packed;
  uint32_t cur, F, EF, lvl;
  uint32_t done_blocks, error, level_cap, max_level, any_new;
  uint32_t launches;
  unsigned long long edges[kLanes];
};

// One block of 64 threads: seeds every root and builds the first frontier
// (roots shared by several lanes become one entry with several mask bits).
__global__ void ms_init_kernel(MsState *st, unsigned long long cond, int use_cond) {
  const uint32_t j = threadIdx.x;
  const uint32_t *pinv = st->pinv;  // roots are original ids
  if (j < st->n_lanes) {
    const uint32_t r = pinv ? pinv[st->roots[j]] : st->roots[j];
    atomicOr(&st->vis[r], 1ull << j);
    atomicOr(&st->prev[r], 1ull << j);
    atomicOr(&st->hist[r], 1ull << j);  // level 0
  }
  if (j < kLanes) st->edges[j] = 0;
  __syncthreads();
  if (j == 0) {
    uint32_t F = 0, EF = 0;
    for (uint32_t l = 0; l < st->n_lanes; l++) {
      const uint32_t r = pinv ? pinv[st->roots[l]] : st->roots[l];
      if (r >= st->n_rows) continue;
      const uint32_t b = st->indptr[r], e = st->indptr[r + 1];
      if (e == b) continue;
      uint32_t k = 0;
      while (k < F && st->qb[0][k] != b) k++;  // same root -> same first edge
      if (k < F) {
        st->qm[0][k] |= 1ull << l;
        continue;
      }
      st->qb[0][F] = b;
      st->qp[0][F] = EF;
      st->qm[0][F] = 1ull << l;
      EF += e - b;
      F++;
    }
    st->qp[0][F] = EF;
    st->F = F;
    st->EF = EF;
    st->cur = 0;
    st->lvl = 0;
    st->next_packed = 0;
    st->done_blocks = 0;
    st->error = 0;
    st->max_level = 0;
    st->any_new = 0;
    st->launches = 2;  // memset, init
    if (use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, F > 0);
  }
}

// Explore: the single-root GLB walk (one difference per entry, a 32-entry
// window re-based only when a round could leave it) with a root mask per
// entry: vis[v] |= mask(u) & ~vis[v].  A lane keeps its edge's entry index
// and reads the entry's mask only when v is not yet reached by every root
// (no mask travels through shuffles).  The plain load may see a stale mask,
// which costs only a redundant reduction.
__global__ void __launch_bounds__(kMsBlock, 1536 / kMsBlock)
    ms_explore_kernel(MsState *__restrict__ st) {
  extern __shared__ __align__(16) uint32_t s_full[];  // hubfull, hub_words words
  constexpr int NW = kMsBlock / 32;
  constexpr int U = kMsU;
  constexpr uint32_t kRound = 32u * U;
  const uint32_t F = st->F;
  if (F == 0) return;
  const uint32_t EF = st->EF;
  const uint32_t hw = st->hub_words;  // a multiple of 4
  const bool use_hub = hw != 0 && EF >= st->hub_min_edges;  // uniform over the grid
  if (use_hub) {
    const uint4 *src = reinterpret_cast<const uint4 *>(st->hubfull);
    uint4 *dst = reinterpret_cast<uint4 *>(s_full);
    for (uint32_t i = threadIdx.x; i < (hw >> 2); i += kMsBlock) dst[i] = src[i];
    __syncthreads();
  }
  const uint32_t hub_lim = use_hub ? hw * 32u : 0u;
  const uint32_t cq = st->cur;
  const uint32_t *__restrict__ qb = st->qb[cq];
  const uint32_t *__restrict__ qp = st->qp[cq];
  const unsigned long long *__restrict__ qm = st->qm[cq];
  const uint32_t *__restrict__ inds = st->inds;
  unsigned long long *vis = st->vis;
  const unsigned long long all_roots = st->n_lanes >= 64u ? ~0ull : (1ull << st->n_lanes) - 1ull;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint64_t pol = evict_first_policy();
  const uint32_t total_warps = gridDim.x * NW;
  // about four chunks per warp, whole groups of kMsU rounds
  uint64_t ch = ((uint64_t)EF + 4ull * total_warps - 1) / (4ull * total_warps);
  ch = (ch + kRound - 1) / kRound * kRound;
  const uint32_t CHUNK = (uint32_t)(ch > kMsChunk ? ch : kMsChunk);
  const uint32_t n_chunks = (uint32_t)(((uint64_t)EF + CHUNK - 1) / CHUNK);

  for (uint32_t c = blockIdx.x * NW + warp; c < n_chunks; c += total_warps) {
    const uint32_t w0 = c * CHUNK;
    const uint32_t w1 = (uint32_t)min((uint64_t)EF, (uint64_t)w0 + CHUNK);
    uint32_t cur = warp_owner_search(qp, F, w0, lane);
    uint32_t cur_d = qb[cur] - qp[cur];
    uint32_t c0 = cur;
    uint32_t bnd = (c0 + 1u + lane <= F) ? qp[c0 + 1u + lane] : kFull;
    uint32_t dl = (c0 + 1u + lane < F) ? qb[c0 + 1u + lane] - bnd : 0u;
    uint32_t wlast = __shfl_sync(kFull, bnd, 31);
    for (uint32_t base = w0; base < w1; base += kRound) {
      uint32_t ad[U], nb[U], ent[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const uint32_t rb = base + 32u * u;
        const uint32_t e = rb + lane;
        if (wlast < rb || wlast - rb < 31u) {  // warp-uniform
          c0 = cur;
          const uint32_t j = c0 + 1u + lane;
          bnd = (j <= F) ? qp[j] : kFull;
          dl = (j < F) ? qb[j] - bnd : 0u;
          wlast = __shfl_sync(kFull, bnd, 31);
        }
        const uint32_t p = bnd - rb;
        const uint32_t starts = __reduce_or_sync(kFull, (p < 32u) ? (1u << p) : 0u);
        const uint32_t k = __popc(starts & ((2u << lane) - 1u));
        const uint32_t srcl = k ? cur + k - c0 - 1u : 0u;
        const uint32_t s_d = __shfl_sync(kFull, dl, srcl);
        ad[u] = kFull;
        ent[u] = cur + k;  // the edge's entry: its root mask is read only if needed
        if (e < w1) ad[u] = e + (k ? s_d : cur_d);
        const uint32_t k31 = __popc(starts);
        if (k31) {
          cur += k31;
          cur_d = __shfl_sync(kFull, dl, cur - c0 - 1u);
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) nb[u] = ad[u] != kFull ? ld_stream(inds + ad[u], pol) : kFull;
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (nb[u] == kFull) continue;
        // a hub every root had reached by the previous level needs no probe
        if (nb[u] < hub_lim && ((s_full[nb[u] >> 5] >> (nb[u] & 31u)) & 1u)) continue;
        // roots not yet in v's live mask (it holds the roots of earlier levels
        // and those other edges gave v in this level): only new roots cost a
        // reduction.  A target every root has reached needs no root mask.
        const unsigned long long vm = vis[nb[u]];
        if (vm == all_roots) continue;
        const unsigned long long bits = qm[ent[u]] & ~vm;
        if (bits) red_or(vis + nb[u], bits);
      }
    }
  }
}

__device__ void ms_finish(MsState *st, unsigned long long cond, int use_cond) {
  const unsigned long long packed = *(volatile unsigned long long *)&st->next_packed;
  const uint32_t f_new = (uint32_t)(packed >> 32), ef_new = (uint32_t)packed;
  const uint32_t lvl = st->lvl + 1;
  if (*(volatile uint32_t *)&st->any_new) st->max_level = lvl;
  st->any_new = 0;
  const uint32_t nq = st->cur ^ 1u;
  st->qp[nq][f_new] = ef_new;
  st->cur = nq;
  st->F = f_new;
  st->EF = ef_new;
  st->lvl = lvl;
  st->next_packed = 0;
  st->done_blocks = 0;
  st->launches += 3;  // explore, levelgen, expand check
  if (f_new > 0 && lvl >= st->level_cap) {
    st->error |= BFS_DEVERR_LEVEL_LIMIT;
    st->F = 0;
  }
  if (use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, st->F > 0);
}

// Level generation, one vertex per thread: new = vis[v] & ~prev[v] (then
// prev[v] = vis[v]).  Levels
// below kHistLevels are recorded as masks, hist[L][v] = new (written for
// every vertex, coalesced; ms_expand_kernel turns them into the level rows);
// deeper levels are written straight into the rows.  Kept vertices are
// compacted with ballot/popc and one atomic per block.
__global__ void __launch_bounds__(kMsBlock) ms_levelgen_kernel(MsState *__restrict__ st,
                                                               unsigned long long cond,
                                                               int use_cond) {
  constexpr int NW = kMsBlock / 32;
  __shared__ unsigned long long s_wtot[NW];
  __shared__ unsigned long long s_base;
  __shared__ int s_last;
  __shared__ uint32_t s_any;
  const uint32_t n_cols = st->n_cols, n_rows = st->n_rows;
  unsigned long long *__restrict__ vis = st->vis;
  unsigned long long *__restrict__ prev = st->prev;
  const uint32_t *__restrict__ indptr = st->indptr;
  int32_t *__restrict__ level = st->level;
  const uint32_t L = st->lvl + 1;
  unsigned long long *__restrict__ hist =
      L < kHistLevels ? st->hist + (size_t)L * n_cols : nullptr;
  const uint32_t nq = st->cur ^ 1u;
  uint32_t *__restrict__ qb = st->qb[nq];
  uint32_t *__restrict__ qp = st->qp[nq];
  unsigned long long *__restrict__ qm = st->qm[nq];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const unsigned long long all_roots =
      st->n_lanes >= 64u ? ~0ull : (1ull << st->n_lanes) - 1ull;
  uint32_t *__restrict__ hubfull = st->hubfull;
  const uint32_t hub_words = st->hub_words;
  const uint32_t *__restrict__ perm = st->perm;
  const uint32_t *__restrict__ moved = st->moved;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  bool any = false;
  const uint64_t span = (uint64_t)kMsBlock;
  for (uint64_t sb = (uint64_t)blockIdx.x * span; sb < n_cols; sb += (uint64_t)gridDim.x * span) {
    const uint32_t v = (uint32_t)(sb + threadIdx.x);
    unsigned long long nw = 0;
    uint32_t b = 0, e = 0;
    bool full = false;
    if (v < n_cols) {
      const unsigned long long vv = vis[v];
      full = vv == all_roots;
      nw = vv & ~prev[v];
      if (nw) {
        prev[v] = vv;
        if (v < n_rows) {
          b = indptr[v];
          e = indptr[v + 1];
        }
      }
      if (hist) hist[v] = nw;
    }
    any |= nw != 0;
    // hub ids every root has reached (warps cover 32 aligned ids)
    if (hub_words) {
      const uint32_t fm = __ballot_sync(kFull, full);
      if (lane == 0 && (v >> 5) < hub_words) hubfull[v >> 5] = fm;
    }
    if (!hist) {  // past the history: one root row at a time
      // rows are in original ids
      const uint32_t ov = (nw && moved && ((moved[v >> 5] >> (v & 31u)) & 1u)) ? perm[v] : v;
      const uint32_t u_lo = __reduce_or_sync(kFull, (uint32_t)nw);
      const uint32_t u_hi = __reduce_or_sync(kFull, (uint32_t)(nw >> 32));
      for (uint32_t m = u_lo; m; m &= m - 1u) {
        const uint32_t j = __ffs(m) - 1u;
        if ((nw >> j) & 1ull) level[(size_t)j * n_cols + ov] = (int32_t)L;
      }
      for (uint32_t m = u_hi; m; m &= m - 1u) {
        const uint32_t j = 32u + __ffs(m) - 1u;
        if ((nw >> j) & 1ull) level[(size_t)j * n_cols + ov] = (int32_t)L;
      }
    }
    const uint32_t deg = e - b;
    // compact the kept vertices: ballot/popc per warp, one atomic per block
    const uint32_t km = __ballot_sync(kFull, deg > 0u);
    const uint32_t dincl = warp_incl_scan(deg, lane);
    if (lane == 31) s_wtot[warp] = ((unsigned long long)__popc(km) << 32) | dincl;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long run = 0;
      for (int i = 0; i < NW; i++) {
        const unsigned long long t = s_wtot[i];
        s_wtot[i] = run;
        run += t;
      }
      s_base = run ? atomicAdd(&st->next_packed, run) : 0ull;
    }
    __syncthreads();
    if (deg) {
      const unsigned long long wb = s_base + s_wtot[warp];
      const uint32_t slot = (uint32_t)(wb >> 32) + __popc(km & lt_mask);
      qb[slot] = b;
      qp[slot] = (uint32_t)wb + dincl - deg;
      qm[slot] = nw;
    }
    __syncthreads();
  }
  if (any) s_any = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_any) atomicOr(&st->any_new, 1u);
    __threadfence();
    const uint32_t ticket = atomicAdd(&st->done_blocks, 1u);
    s_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    ms_finish(st, cond, use_cond);
  }
}

// Writes the level rows from the history and, after the last level, the
// per-root edge counts.  In the level loop (final == 0) it acts only once,
// right after the last history level when the search goes on: it then
// writes every row entry (level or -1) so that level generation can write
// the deeper levels directly.  After the loop (final != 0) it writes the rows
// unless that already happened (the search went past the history), then
// adds, per root, the degrees of the vertices < n_rows it reached
// (run_bfs_cpu.hpp:36).
//
// One warp per 32 consecutive vertices, lane = vertex.  History levels are
// < 16, so a lane ORs its vertex's masks into four bit planes (plane k holds
// the roots whose level has bit k set) and a reached mask; the level of root
// j is then four bit extracts, and the warp stores root j's 32 entries as one
// 128-byte segment.  The root loop is unrolled so that every shift is a
// constant.
// Spreads the 4 low bits of n (n < 16) to bit 0 of the 4 bytes: the shifted
// copies n, n << 7, n << 14, n << 21 do not overlap, so the product has no
// carries and byte i holds bit i of n.
__device__ __forceinline__ uint32_t nibble_to_bytes(uint32_t n) {
  return (n * 0x00204081u) & 0x01010101u;
}

// Byte i of x, sign-extended: one prmt whose selector copies byte i into the
// low byte and replicates its sign bit (selector value 8 + i) into the others.
__device__ __forceinline__ int32_t sext_byte(uint32_t x, int i) {
  const uint32_t sel = (uint32_t)i | ((8u + (uint32_t)i) * 0x1110u);
  uint32_t r;
  asm("prmt.b32 %0, %1, 0, %2;" : "=r"(r) : "r"(x), "r"(sel));
  return (int32_t)r;
}

template <int H>
__device__ __forceinline__ void ms_store_rows(int32_t *__restrict__ row, size_t n, uint32_t v,
                                              bool in, uint32_t nl, uint32_t r, uint32_t b0,
                                              uint32_t b1, uint32_t b2, uint32_t b3) {
  // four roots at a time: their levels as four bytes (0xFF = unreached)
#pragma unroll
  for (int j = 0; j < 32; j += 4) {
    if ((uint32_t)(H * 32 + j) >= nl) break;  // uniform
    const uint32_t lv4 = nibble_to_bytes((b0 >> j) & 15u) | (nibble_to_bytes((b1 >> j) & 15u) << 1) |
                         (nibble_to_bytes((b2 >> j) & 15u) << 2) |
                         (nibble_to_bytes((b3 >> j) & 15u) << 3);
    const uint32_t seen = nibble_to_bytes((r >> j) & 15u) * 0xFFu;
    const uint32_t packed = lv4 | ~seen;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if ((uint32_t)(H * 32 + j + i) >= nl) break;  // uniform
      if (in) row[v] = sext_byte(packed, i);
      row += n;
    }
  }
}

__global__ void __launch_bounds__(kMsBlock, 4) ms_expand_kernel(MsState *__restrict__ st,
                                                                int final) {
  static_assert(kHistLevels <= 16, "levels must fit four bit planes");
  __shared__ unsigned long long s_edges[kLanes];
  __shared__ unsigned long long s_common;
  const uint32_t lvl = st->lvl;
  const bool expand = final ? (lvl < kHistLevels) : (lvl + 1u == kHistLevels && st->F > 0);
  if (!final && !expand) return;  // uniform over the grid
  const uint32_t n = st->n_cols, n_rows = st->n_rows, nl = st->n_lanes;
  const uint32_t lmax = lvl < kHistLevels ? lvl : kHistLevels - 1u;
  const unsigned long long *__restrict__ hist = st->hist;
  const unsigned long long *__restrict__ vis = st->vis;
  const uint32_t *__restrict__ indptr = st->indptr;
  int32_t *__restrict__ level = st->level;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (final) {
    if (threadIdx.x < kLanes) s_edges[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_common = 0;
    __syncthreads();
  }
  const unsigned long long all_roots = nl >= 64u ? ~0ull : (1ull << nl) - 1ull;
  unsigned long long acc_lo = 0, acc_hi = 0;  // degree sums of roots lane, 32 + lane
  unsigned long long common = 0;              // degree sums of vertices every root reached
  const uint64_t stride = (uint64_t)gridDim.x * kMsBlock;
  const uint32_t *__restrict__ pinv = st->pinv;
  const uint32_t *__restrict__ moved = st->moved;
  for (uint64_t t0 = (uint64_t)blockIdx.x * kMsBlock + warp * 32u; t0 < n; t0 += stride) {
    const uint32_t ov = (uint32_t)t0 + lane;  // original id: the row entry written
    const bool in = ov < n;
    // internal id whose masks and degree belong to it (moved ids only differ)
    const uint32_t v = (in && moved && ((moved[ov >> 5] >> (ov & 31u)) & 1u)) ? pinv[ov] : ov;
    // this step's loads are issued together: the mask and degree for the
    // edge counts, and history levels 0 .. 7 (8 .. 15 after them, if the
    // search went that deep)
    unsigned long long vm = 0;
    uint32_t d = 0;
    if (final && in) {
      vm = vis[v];
      if (v < n_rows) d = indptr[v + 1] - indptr[v];
    }
    if (expand) {
      unsigned long long r = 0, p0 = 0, p1 = 0, p2 = 0, p3 = 0;
      if (in) {
        // within levels L0 .. L0 + 3 (L0 a multiple of 4) bits 0 and 1 of
        // the level are those of k, bits 2 and 3 those of L0
        for (uint32_t L0 = 0; L0 <= lmax; L0 += 8) {
          unsigned long long m[8];
#pragma unroll
          for (int k = 0; k < 8; k++)
            m[k] = (L0 + k <= lmax) ? hist[(size_t)(L0 + k) * n + v] : 0ull;
#pragma unroll
          for (int h = 0; h < 8; h += 4) {
            const unsigned long long all4 = m[h] | m[h + 1] | m[h + 2] | m[h + 3];
            r |= all4;
            p0 |= m[h + 1] | m[h + 3];
            p1 |= m[h + 2] | m[h + 3];
            if ((L0 + h) & 4u) p2 |= all4;
            if ((L0 + h) & 8u) p3 |= all4;
          }
        }
      }
      ms_store_rows<0>(level, n, ov, in, nl, (uint32_t)r, (uint32_t)p0, (uint32_t)p1,
                       (uint32_t)p2, (uint32_t)p3);
      if (nl > 32)
        ms_store_rows<1>(level + (size_t)32 * n, n, ov, in, nl, (uint32_t)(r >> 32),
                         (uint32_t)(p0 >> 32), (uint32_t)(p1 >> 32), (uint32_t)(p2 >> 32),
                         (uint32_t)(p3 >> 32));
    }
    if (final) {
      // per-root degree sums as a bit-matrix product: lane j takes the
      // vertex masks of roots j and 32 + j (32 ballots), and the degrees go
      // in bit planes (one ballot per degree bit)
      const uint32_t deg = vm ? d : 0u;
      const uint32_t dmax = __reduce_max_sync(kFull, deg);
      // the usual warp: every vertex with edges was reached by every root
      // (the giant component), so its degrees count once for all roots
      if (dmax && __all_sync(kFull, deg == 0u || vm == all_roots)) {
        common += __reduce_add_sync(kFull, deg);
      } else if (dmax) {
        const uint32_t lo = (uint32_t)vm, hi = (uint32_t)(vm >> 32);
        uint32_t mlo = 0, mhi = 0;
#pragma unroll
        for (int j = 0; j < 32; j++) {
          const uint32_t a = __ballot_sync(kFull, (lo >> j) & 1u);
          const uint32_t c = __ballot_sync(kFull, (hi >> j) & 1u);
          if (lane == (uint32_t)j) {
            mlo = a;
            mhi = c;
          }
        }
        const int nbits = 32 - __clz(dmax);
        for (int b = 0; b < nbits; b++) {
          const uint32_t plane = __ballot_sync(kFull, (deg >> b) & 1u);
          acc_lo += (unsigned long long)__popc(mlo & plane) << b;
          acc_hi += (unsigned long long)__popc(mhi & plane) << b;
        }
      }
    }
  }
  if (final) {
    if (acc_lo) atomicAdd(&s_edges[lane], acc_lo);
    if (acc_hi) atomicAdd(&s_edges[32 + lane], acc_hi);
    if (lane == 0 && common) atomicAdd(&s_common, common);
    __syncthreads();
    if (threadIdx.x < nl && s_edges[threadIdx.x] + s_common)
      atomicAdd(&st->edges[threadIdx.x], s_edges[threadIdx.x] + s_common);
    if (blockIdx.x == 0 && threadIdx.x == 0) st->launches += 1;
  }
}

}  // namespace bfsgb

// ---- host side ----------------------------------------------------------------
using namespace bfsgb;

struct MsWorkspace {
  void *mem = nullptr;
  MsState *d_st = nullptr;
  MsState *h_st = nullptr;  // pinned
  MsState tmpl{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int grid_ex = 0, grid_lg = 0, grid_xp = 0;
  int32_t *rows = nullptr;  // one pass of level rows for bfs_run_batch_host
  size_t clear_bytes = 0;  // visited and prev masks, history level 0
  uint32_t *hubfull = nullptr;  // g->words words
  size_t hub_bytes = 0;    // explore's dynamic shared memory (the hub layout's prefix)
  uint32_t hub_gen = 0;    // the handle's layout generation this workspace copied
};

namespace bfsgb {

void free_msbfs(bfs_graph *g) {
  MsWorkspace *w = g->ms;
  if (!w) return;
  if (w->exec) cudaGraphExecDestroy(w->exec);
  if (w->graph) cudaGraphDestroy(w->graph);
  if (w->e0) cudaEventDestroy(w->e0);
  if (w->e1) cudaEventDestroy(w->e1);
  cudaFree(w->mem);
  cudaFree(w->d_st);
  cudaFree(w->rows);
  cudaFree(w->hubfull);
  if (w->h_st) cudaFreeHost(w->h_st);
  delete w;
  g->ms = nullptr;
}

}  // namespace bfsgb

#define MK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(e_ == cudaErrorMemoryAllocation ? BFS_ERR_OOM : BFS_ERR_CUDA,    \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

static bfs_status ms_setup(bfs_graph *g) {
  bfs_status hrc = ensure_hub(g);
  if (hrc != BFS_OK) return hrc;
  // the template and the graph below copy the layout's arrays and bake in its
  // shared-memory size: a workspace built for another layout is rebuilt
  const uint32_t ms_hub = g->hub ? std::min<uint32_t>(g->hub->vertices, kMsHubMax) : 0u;
  const size_t hub_bytes = (size_t)ms_hub / 8;
  if (g->ms && g->ms->hub_gen != g->hub_gen) free_msbfs(g);
  if (g->ms) return BFS_OK;
  MsWorkspace *w = new MsWorkspace();
  g->ms = w;
  w->hub_bytes = hub_bytes;
  w->hub_gen = g->hub_gen;
  const size_t n = g->n_cols, nr = std::max<uint32_t>(g->n_rows, 1);
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t b64 = al(n * 8), q4 = al(nr * 4), qp4 = al((nr + 1) * 4), q8 = al(nr * 8);
  const size_t bytes = (2 + kHistLevels) * b64 + 2 * (q4 + qp4 + q8);
  MK(dev_malloc(&w->mem, bytes));
  MK(dev_malloc(&w->d_st, sizeof(MsState)));
  MK(cudaMallocHost(&w->h_st, sizeof(MsState)));
  MK(cudaEventCreate(&w->e0));
  MK(cudaEventCreate(&w->e1));
  char *p = (char *)w->mem;
  MsState &s = w->tmpl;
  std::memset(&s, 0, sizeof(s));
  s.indptr = g->indptr;
  s.inds = g->inds;
  s.n_rows = g->n_rows;
  s.n_cols = g->n_cols;
  if (g->hub) {
    MK(dev_malloc(&w->hubfull, sizeof(uint32_t) * (size_t)g->words));
    s.indptr = g->hub->indptr;
    s.inds = g->hub->inds;
    s.perm = g->hub->perm;
    s.pinv = g->hub->pinv;
    s.moved = g->hub->moved;
    s.hubfull = w->hubfull;
    s.hub_words = ms_hub / 32u;
    s.hub_min_edges = g->hub_min_edges ? g->hub_min_edges
                                       : std::max<uint32_t>(kHubMinEdges, 2u * ms_hub);
    if (hub_bytes > 48 * 1024)
      MK(cudaFuncSetAttribute((const void *)ms_explore_kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hub_bytes));
  }
  s.vis = (unsigned long long *)p; p += b64;
  s.prev = (unsigned long long *)p; p += b64;
  s.hist = (unsigned long long *)p; p += kHistLevels * b64;
  for (int b = 0; b < 2; b++) {
    s.qb[b] = (uint32_t *)p; p += q4;
    s.qp[b] = (uint32_t *)p; p += qp4;
    s.qm[b] = (unsigned long long *)p; p += q8;
  }
  s.level_cap = g->n_cols + 1u;
  w->clear_bytes = 3 * b64;  // vis, prev, hist[0] are contiguous
  int occ_ex = 0, occ_lg = 0, occ_xp = 0;
  MK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_ex, (const void *)ms_explore_kernel,
                                                   kMsBlock, hub_bytes));
  MK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_lg, (const void *)ms_levelgen_kernel,
                                                   kMsBlock, 0));
  MK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_xp, (const void *)ms_expand_kernel,
                                                   kMsBlock, 0));
  w->grid_ex = g->num_sms * std::max(occ_ex, 1);
  w->grid_lg = g->num_sms * std::max(occ_lg, 1);
  w->grid_xp = g->num_sms * std::max(occ_xp, 1);

  // graph: memset(vis, prev, hist[0]) -> init ->
  //   while(F > 0) { explore -> levelgen -> expand(in loop) } -> expand(final)
  MK(cudaGraphCreate(&w->graph, 0));
  cudaGraphConditionalHandle cond;
  MK(cudaGraphConditionalHandleCreate(&cond, w->graph, 0, cudaGraphCondAssignDefault));
  unsigned long long cond_arg = (unsigned long long)cond;
  int one = 1;
  MsState *st = w->d_st;
  cudaMemsetParams mp;
  std::memset(&mp, 0, sizeof(mp));
  mp.dst = w->mem;
  mp.elementSize = 4;
  mp.width = w->clear_bytes / 4;
  mp.height = 1;
  cudaGraphNode_t n_ms, n_init, n_while, n_ex, n_lg, n_xp, n_xf;
  MK(cudaGraphAddMemsetNode(&n_ms, w->graph, nullptr, 0, &mp));
  cudaGraphNode_t init_deps[2] = {n_ms, nullptr};
  size_t n_init_deps = 1;
  if (w->hubfull) {
    // a pass starts with no hub known to be reached by every root
    cudaMemsetParams hp = mp;
    hp.dst = w->hubfull;
    hp.width = g->words;
    MK(cudaGraphAddMemsetNode(&init_deps[1], w->graph, nullptr, 0, &hp));
    n_init_deps = 2;
  }
  cudaKernelNodeParams kp;
  std::memset(&kp, 0, sizeof(kp));
  void *init_args[] = {&st, &cond_arg, &one};
  kp.func = (void *)ms_init_kernel;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(kLanes);
  kp.kernelParams = init_args;
  MK(cudaGraphAddKernelNode(&n_init, w->graph, init_deps, n_init_deps, &kp));
  alignas(cudaGraphNodeParams) unsigned char wbuf[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams &wp = *reinterpret_cast<cudaGraphNodeParams *>(wbuf);
  wp.type = cudaGraphNodeTypeConditional;
  wp.conditional.handle = cond;
  wp.conditional.type = cudaGraphCondTypeWhile;
  wp.conditional.size = 1;
  MK(cudaGraphAddNode(&n_while, w->graph, &n_init, nullptr, 1, &wp));
  cudaGraph_t body = wp.conditional.phGraph_out[0];
  void *ex_args[] = {&st};
  kp.func = (void *)ms_explore_kernel;
  kp.gridDim = dim3(w->grid_ex);
  kp.blockDim = dim3(kMsBlock);
  kp.sharedMemBytes = (unsigned)hub_bytes;
  kp.kernelParams = ex_args;
  MK(cudaGraphAddKernelNode(&n_ex, body, nullptr, 0, &kp));
  kp.sharedMemBytes = 0;
  void *lg_args[] = {&st, &cond_arg, &one};
  kp.func = (void *)ms_levelgen_kernel;
  kp.gridDim = dim3(w->grid_lg);
  kp.blockDim = dim3(kMsBlock);
  kp.kernelParams = lg_args;
  MK(cudaGraphAddKernelNode(&n_lg, body, &n_ex, 1, &kp));
  int in_loop = 0, after = 1;
  void *xp_args[] = {&st, &in_loop};
  kp.func = (void *)ms_expand_kernel;
  kp.gridDim = dim3(w->grid_xp);
  kp.kernelParams = xp_args;
  MK(cudaGraphAddKernelNode(&n_xp, body, &n_lg, 1, &kp));
  void *xf_args[] = {&st, &after};
  kp.kernelParams = xf_args;
  MK(cudaGraphAddKernelNode(&n_xf, w->graph, &n_while, 1, &kp));
  MK(cudaGraphInstantiate(&w->exec, w->graph, 0));
  return BFS_OK;
}

// The same pass as the graph, driven from the host: one frontier-size read-back
// per level.  Every kernel is a separate launch, which profilers can capture
// (kernels inside a graph with a conditional node cannot be).
static bfs_status ms_pass_host(bfs_graph *g, MsWorkspace *w) {
  cudaStream_t s = g->stream;
  MsState *st = w->d_st;
  unsigned long long no_cond = 0;
  int zero = 0;
  MK(cudaMemsetAsync(w->mem, 0, w->clear_bytes, s));
  if (w->hubfull) MK(cudaMemsetAsync(w->hubfull, 0, sizeof(uint32_t) * g->words, s));
  ms_init_kernel<<<1, kLanes, 0, s>>>(st, no_cond, zero);
  MK(cudaGetLastError());
  uint32_t *h_F = &w->h_st->F;
  for (;;) {
    MK(cudaMemcpyAsync(h_F, &st->F, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    MK(cudaStreamSynchronize(s));
    if (*h_F == 0) break;
    ms_explore_kernel<<<w->grid_ex, kMsBlock, w->hub_bytes, s>>>(st);
    MK(cudaGetLastError());
    ms_levelgen_kernel<<<w->grid_lg, kMsBlock, 0, s>>>(st, no_cond, zero);
    MK(cudaGetLastError());
    ms_expand_kernel<<<w->grid_xp, kMsBlock, 0, s>>>(st, 0);
    MK(cudaGetLastError());
  }
  ms_expand_kernel<<<w->grid_xp, kMsBlock, 0, s>>>(st, 1);
  MK(cudaGetLastError());
  return BFS_OK;
}

extern "C" bfs_status bfs_run_batch(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                                    int32_t *levels_dev, uint64_t *edges_count_out,
                                    bfs_batch_stats *stats) {
  return bfs_run_batch_loop(g, roots, n_roots, levels_dev, edges_count_out, BFS_LOOP_GRAPH,
                            stats);
}

extern "C" bfs_status bfs_run_batch_loop(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                                         int32_t *levels_dev, uint64_t *edges_count_out,
                                         int32_t loop, bfs_batch_stats *stats) {
  if (!g || !roots || !levels_dev) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  if (loop != BFS_LOOP_GRAPH && loop != BFS_LOOP_HOST)
    return fail(BFS_ERR_INVALID_ARG, "loop must be BFS_LOOP_GRAPH or BFS_LOOP_HOST");
  for (uint32_t i = 0; i < n_roots; i++)
    if (roots[i] >= g->n_cols) return fail(BFS_ERR_ROOT, "root out of range");
  MK(cudaSetDevice(g->device));
  bfs_status rc = ms_setup(g);
  if (rc != BFS_OK) {
    free_msbfs(g);
    return rc;
  }
  MsWorkspace *w = g->ms;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  double total_ms = 0.0;
  for (uint32_t b0 = 0; b0 < n_roots; b0 += kLanes) {
    const uint32_t nl = std::min<uint32_t>(kLanes, n_roots - b0);
    MsState &s = *w->h_st;
    s = w->tmpl;
    s.level = levels_dev + (size_t)b0 * g->n_cols;
    s.n_lanes = nl;
    for (uint32_t j = 0; j < nl; j++) s.roots[j] = roots[b0 + j];
    MK(cudaEventRecord(w->e0, g->stream));
    MK(cudaMemcpyAsync(w->d_st, w->h_st, sizeof(MsState), cudaMemcpyHostToDevice, g->stream));
    if (loop == BFS_LOOP_HOST) {
      rc = ms_pass_host(g, w);
      if (rc != BFS_OK) return rc;
    } else {
      MK(cudaGraphLaunch(w->exec, g->stream));
    }
    MK(cudaEventRecord(w->e1, g->stream));
    MK(cudaMemcpyAsync(w->h_st, w->d_st, sizeof(MsState), cudaMemcpyDeviceToHost, g->stream));
    MK(cudaStreamSynchronize(g->stream));
    const MsState &r = *w->h_st;
    if (r.error & BFS_DEVERR_LEVEL_LIMIT)
      return fail(BFS_ERR_LEVEL_LIMIT, "level loop exceeded n_cols + 1 levels");
    if (r.error) return fail(BFS_ERR_DEVICE, "device error flag " + std::to_string(r.error));
    float ms = 0.f;
    MK(cudaEventElapsedTime(&ms, w->e0, w->e1));
    total_ms += ms;
    if (edges_count_out)
      for (uint32_t j = 0; j < nl; j++) edges_count_out[b0 + j] = r.edges[j];
    if (stats) {
      stats->batches++;
      stats->max_levels = std::max(stats->max_levels, r.max_level + 1);
      stats->launches += r.launches + 1;
    }
  }
  if (stats) stats->device_ms = total_ms;
  return BFS_OK;
}

extern "C" bfs_status bfs_run_batch_host(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                                         int32_t *levels_host, uint64_t *edges_count_out,
                                         bfs_batch_stats *stats) {
  if (!g || !roots) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  MK(cudaSetDevice(g->device));
  bfs_status rc = ms_setup(g);
  if (rc != BFS_OK) {
    free_msbfs(g);
    return rc;
  }
  MsWorkspace *w = g->ms;
  const size_t n = g->n_cols;
  if (!w->rows) MK(dev_malloc(&w->rows, sizeof(int32_t) * n * kLanes));
  bfs_batch_stats total;
  std::memset(&total, 0, sizeof(total));
  for (uint32_t b0 = 0; b0 < n_roots; b0 += kLanes) {
    const uint32_t nl = std::min<uint32_t>(kLanes, n_roots - b0);
    bfs_batch_stats st;
    rc = bfs_run_batch_loop(g, roots + b0, nl, w->rows,
                            edges_count_out ? edges_count_out + b0 : nullptr, BFS_LOOP_GRAPH,
                            &st);
    if (rc != BFS_OK) return rc;
    total.device_ms += st.device_ms;
    total.batches += st.batches;
    total.max_levels = std::max(total.max_levels, st.max_levels);
    total.launches += st.launches;
    if (levels_host)
      MK(cudaMemcpy(levels_host + (size_t)b0 * n, w->rows, sizeof(int32_t) * n * nl,
                    cudaMemcpyDeviceToHost));
  }
  if (stats) *stats = total;
  return BFS_OK;
}
