// kernels.cu -- sm_103a kernels of the level-synchronous top-down BFS.
//
// Per level the reference runs an explore kernel (src/run_bfs_gpu.hpp:388-477
// for LLB/SLB, :175-385 for GLB) that marks unvisited neighbours of the
// frontier in byte masks, then a level-generation kernel (:481-521) that scans
// every vertex, writes levels and appends the new frontier with one atomic per
// vertex.  The same two-step structure is kept here, redesigned for GB300:
//
//   explore   a frontier queue entry carries its first edge and the exclusive
//             prefix of degrees in queue order (plus its vertex id when
//             parents are recorded), so the per-level indptr gather moves out
//             of the edge loop.  Edges are processed in warp rounds of 32
//             consecutive edges (coalesced reads of the edge array, streamed
//             with an L2 evict-first policy and no L1 allocation).  The owner
//             entry of each edge is resolved with a warp OR-reduction of entry
//             boundaries plus popc instead of a per-edge binary search
//             (:448-464, :336-346).  Visiting tests one bit of a visited
//             bitmap (n/8 bytes, pinned in L2 through an access-policy window)
//             with a plain load and only then claims it with atomicOr, instead
//             of byte masks.
//   levelgen  scans the bitmap words (n/32, not n bytes): new = vis & ~prev.
//             Blocks claim spans of words from a counter, write the new
//             levels a bitmap word (one 32-byte sector of one-byte working
//             levels) at a time, and list each span's new vertices in shared
//             memory; warps take equal shares of the list and load degrees
//             32 at a time, and one atomic per block and span reserves the
//             queue tail (after levels with few edges, warps do the same on
//             their own, without block barriers).  The atomic adds
//             (count << 32 | chunk count), so every entry also receives the
//             exclusive prefix of its 16-byte edge chunks in queue order: the
//             grid-wide scan that GLB needs comes out of the same atomic.
//             Zero-degree vertices and vertices >= n_rows get their level
//             but are not queued (they would expand nothing;
//             run_bfs_cpu.hpp:31 never expands tid >= numRows).
//   finish    the last level-generation block swaps the queues, accumulates
//             edgesCount and, in the CUDA-graph loop, sets the while-node
//             condition, so no host round trip happens between levels.
//   output    after the last level one pass writes the int32 levels (original
//             ids, -1 for unvisited) from the working levels.
#include <cuda_runtime.h>
#include <cstdint>

#include "bfs_internal.h"
#include "device_util.cuh"
#include "kernels.h"
#include "bfs_sched_dev.cuh"

namespace bfsgb {

// Claim of bit n after a plain load saw it clear (the load may see a stale 0
// from an L1 copy; atomicOr's return value is authoritative, so exactly one
// thread claims n).  Parents are written in original ids (perm: internal ->
// original, null for the identity); `from` already is one.
__device__ __forceinline__ void claim(uint32_t *vis, uint32_t n, int32_t *parent, uint32_t from,
                                      const uint32_t *perm) {
  const uint32_t w = n >> 5, bit = 1u << (n & 31u);
  if (parent) {
    const uint32_t old = atomicOr(vis + w, bit);
    if (!(old & bit)) parent[perm ? perm[n] : n] = (int32_t)from;
  } else {
    red_or(vis + w, bit);  // result unused: a reduction, no round trip
  }
}

// Test-then-claim of bit n.
__device__ __forceinline__ void visit(uint32_t *vis, uint32_t n, int32_t *parent,
                                      uint32_t from, const uint32_t *perm) {
  if (vis[n >> 5] & (1u << (n & 31u))) return;
  claim(vis, n, parent, from, perm);
}

// Owner resolution for one warp round.  `cur` is an entry whose start is at
// or before the round base rb, `bnd` the start offset of entry cur + 1 + lane
// (all entries have degree >= 1, so starts are distinct).  Returns the entry
// owning edge rb + lane.
__device__ __forceinline__ uint32_t round_owner(uint32_t cur, uint32_t bnd,
                                                uint32_t rb, uint32_t lane) {
  const uint32_t p = bnd - rb;  // wraps to a large value when bnd < rb
  const uint32_t bits = (p < 32u) ? (1u << p) : 0u;
  const uint32_t starts = __reduce_or_sync(kFull, bits);
  return cur + __popc(starts & ((2u << lane) - 1u));
}

// ---- fill / init --------------------------------------------------------------

__global__ void fill_kernel(BfsDevState *st) {
  int32_t *parent = st->parent;
  const uint32_t n = st->n_cols;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  // parents to -1 (int4 stores for the body when the buffer is 16-byte
  // aligned); levels need no fill: level_out_kernel writes every entry
  if (parent) {
    const uint32_t n4 = (reinterpret_cast<uintptr_t>(parent) & 15u) == 0 ? (n >> 2) : 0u;
    const int4 neg = make_int4(-1, -1, -1, -1);
    for (uint32_t i = tid; i < n4; i += stride) reinterpret_cast<int4 *>(parent)[i] = neg;
    for (uint32_t i = (n4 << 2) + tid; i < n; i += stride) parent[i] = -1;
  }
  for (uint32_t i = tid; i < st->rec_cap; i += stride) st->rec_ran[i] = -1;
  // cleared bitmaps and unvisited working levels: kernel stores rather than
  // a memset, so that a BFS uses no copy engine between its start and its
  // final state read (words is a multiple of 32, the bitmaps and the
  // working levels -- 32 bytes per word -- are 16-byte aligned)
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  for (uint32_t i = tid; i < (st->words >> 2); i += stride) {
    reinterpret_cast<uint4 *>(st->vis)[i] = zero;
    reinterpret_cast<uint4 *>(st->prev)[i] = zero;
  }
  const uint4 unvisited = make_uint4(~0u, ~0u, ~0u, ~0u);
  for (uint32_t i = tid; i < st->words * 2u; i += stride)
    reinterpret_cast<uint4 *>(st->lv8)[i] = unvisited;
}

__device__ __forceinline__ int32_t output_level(uint32_t c, const int32_t *level, uint32_t u) {
  return c == kLv8Unvisited ? -1 : c == kLv8Deep ? level[u] : (int32_t)c;
}

__device__ __forceinline__ int4 output_levels4(uint32_t c4, const int32_t *level, uint32_t u) {
  return make_int4(output_level(c4 & 0xFFu, level, u), output_level((c4 >> 8) & 0xFFu, level, u + 1),
                   output_level((c4 >> 16) & 0xFFu, level, u + 2),
                   output_level(c4 >> 24, level, u + 3));
}

// Output levels, original id u from the working level of its internal id:
// every entry of `level` is written (-1 for unvisited), deep levels (written
// during the BFS) are kept.  Lane l of a warp step takes the 4-id groups
// g0 + 32 k (k < 4, g0 = 128 x warp + l): each store instruction writes 512
// contiguous bytes (whole sectors), and the four groups' loads are in flight
// together.  A relabelled id u is moved exactly when bit u of the moved
// bitmap is set (perm[u] != u iff pinv[u] != u); a group with moved ids
// gathers their working levels through pinv.
__global__ void level_out_kernel(BfsDevState *st) {
  int32_t *level = st->level;
  const uint8_t *lv8 = st->lv8;
  const uint32_t *moved = st->moved, *pinv = st->pinv;
  const uint32_t n = st->n_cols;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t step = gridDim.x * blockDim.x * 4u;  // groups per grid step
  const uint32_t n4 = (reinterpret_cast<uintptr_t>(level) & 15u) == 0 ? (n >> 2) : 0u;
  for (uint32_t g0 = gwarp * 128u + lane; g0 < n4; g0 += step) {
    uint32_t c[4], mb[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint32_t g = g0 + 32u * k, u = g << 2;
      c[k] = mb[k] = 0;
      if (g < n4) {
        c[k] = reinterpret_cast<const uint32_t *>(lv8)[g];
        if (moved) mb[k] = (moved[u >> 5] >> (u & 31u)) & 0xFu;
      }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint32_t g = g0 + 32u * k, u = g << 2;
      if (g < n4) {
        if (mb[k]) {
          uint32_t x = 0;
#pragma unroll
          for (uint32_t i = 0; i < 4; i++)
            x |= (uint32_t)lv8[((mb[k] >> i) & 1u) ? pinv[u + i] : u + i] << (8u * i);
          c[k] = x;
        }
        reinterpret_cast<int4 *>(level)[g] = output_levels4(c[k], level, u);
      }
    }
  }
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t u = (n4 << 2) + blockIdx.x * blockDim.x + threadIdx.x; u < n; u += stride) {
    const bool mv = moved && ((moved[u >> 5] >> (u & 31u)) & 1u);
    level[u] = output_level(lv8[mv ? pinv[u] : u], level, u);
  }
}

// The host template of the state, passed by value: seeding the state is a
// kernel rather than a host-to-device copy, for the same reason.
__global__ void seed_state_kernel(BfsDevState *st, BfsDevState s) {
  static_assert(sizeof(BfsDevState) % 4 == 0, "state is copied in words");
  const uint32_t *src = reinterpret_cast<const uint32_t *>(&s);
  uint32_t *dst = reinterpret_cast<uint32_t *>(st);
  for (uint32_t i = threadIdx.x; i < sizeof(BfsDevState) / 4; i += blockDim.x) dst[i] = src[i];
}

// Records, for the level being explored, which explore kernel ran.
template <int ARM>
__device__ __forceinline__ void note_arm(BfsDevState *st) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t l = st->lvl;
    if (l < st->rec_cap) st->rec_ran[l] = ARM;
  }
}
template <int B>
struct BlockIndex {
  static constexpr int value = B == 128 ? 0 : B == 256 ? 1 : 2;
};

// One warp: the learned scheduler's arm for the level with counters c, from
// the weights w (staged in shared memory by the caller) and the graph
// constants held in the state, stored in st->arm for explore_any.  Kept out
// of line so that the callers' register allocation is not affected.
__device__ __noinline__ void fused_sched_pick(BfsDevState *st, const LevelCounters &c,
                                               const float *w) {
  SchedGraphConst gc;
  gc.diam = st->sched_diam;
  gc.avg_deg_x = st->sched_avg_deg_x;
  sched_pick_warp<true>(st, c, w, st->sched_min_conf, gc);
}

// Copies the model to shared memory with all threads of the block: one
// round of parallel loads instead of the MLP's dependent ones; W2 and W3 are
// stored transposed there (sched_transposed_index), so that the warp reads
// them without bank conflicts.  The loads
// mark the model evict-last in L2, so that it stays there while each level's
// edge stream (evict-first) passes through.
// Threads first .. blockDim.x - 1 take part.
__device__ __forceinline__ void stage_weights(float *dst, const float *__restrict__ w,
                                              uint32_t first = 0) {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  for (uint32_t i = threadIdx.x - first; i < (uint32_t)kSchedParams; i += blockDim.x - first) {
    float x;
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(x) : "l"(w + i), "l"(pol));
    dst[sched_transposed_index((int)i)] = x;
  }
}

__device__ void init_state(BfsDevState *st, unsigned long long cond, int use_cond) {
  const uint32_t r = st->root;                     // original id
  const uint32_t ri = st->pinv ? st->pinv[r] : r;  // internal id
  st->vis[ri >> 5] |= 1u << (ri & 31u);
  st->prev[ri >> 5] |= 1u << (ri & 31u);
  st->lv8[ri] = 0;
  if (st->parent) st->parent[r] = (int32_t)r;
  const bool expanded = ri < st->n_rows;  // run_bfs_cpu.hpp:31
  uint32_t b = 0, e = 0;
  if (expanded) {
    b = st->indptr[ri];
    e = st->indptr[ri + 1];
  }
  if (expanded && e > b) {
    const uint32_t nch = edge_chunks(b, e - b, st->inds_off);
    st->qb[0][0] = b;
    st->qd[0][0] = e - b;
    st->qc[0][0] = 0;
    st->qc[0][1] = nch;
    st->qv[0][0] = r;
    st->F = 1;
    st->EF = e - b;
    st->EC = nch;
  } else {
    st->qc[0][0] = 0;
    st->F = 0;
    st->EF = 0;
    st->EC = 0;
  }
  st->edges_count = expanded ? (unsigned long long)(e - b) : 0ull;
  st->cur = 0;
  st->lvl = 0;
  st->reached = 1;
  st->reached_prev = 1;
  st->max_level = 0;
  st->next_packed = 0;
  st->next_edges = 0;
  st->done_blocks = 0;
  st->lg_cursor = 0;
  st->error = 0;
  st->launches = 3;  // fill, init and the level output after the loop
  st->arm = st->fixed_arm >= 0 ? st->fixed_arm : 0;
  if (st->rec_cap > 0) {
    st->rec_frontier[0] = st->F;
    st->rec_edges[0] = st->EF;
    st->rec_arm[0] = -1;
  }
  if (use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, st->F > 0);
}

// One warp: thread 0 seeds the root and the first frontier; with a fused
// scheduler the warp then picks level 0's arm.
__global__ void init_kernel(BfsDevState *st, unsigned long long cond, int use_cond) {
  __shared__ float s_w[kSchedParams];
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const float *w = st->sched_w;
  if (w != nullptr) stage_weights(s_w, w);
  if (threadIdx.x == 0) init_state(st, cond, use_cond);
  __syncwarp();
  if (w != nullptr) fused_sched_pick(st, level_counters(st), s_w);
}

// ---- explore: LLB / SLB -----------------------------------------------------
// A tile of B frontier entries per block iteration.  LLB takes entries
// tile*B .. tile*B+B-1; SLB takes tile, tile+T, tile+2T, ... with T the
// number of tiles, the strided mapping of run_bfs_gpu.hpp:416-420.  A block
// exclusive scan of the tile's degrees (shared memory) splits the tile's
// edges evenly over the block's warps (block-local balancing, :437-445).
// U warp rounds (U edges per lane) are resolved before their loads issue.
// Minimum resident blocks requested from the compiler (register budget).
// Measured on RMAT-25: 2048 resident threads per SM (32 registers) for 4
// rounds per lane make GLB and SLB faster despite a few spilled bytes; LLB's
// large-tile level is faster at 1536 threads (40 registers).  8 rounds per
// lane get 1024 threads (64 registers).
template <int B, int U, bool CONSTRAINED>
struct MinBlocks {
  static constexpr int value = (U <= 4 ? (CONSTRAINED ? 2048 : 1536) : 1024) / B;
};

// Barrier over the B threads of one (virtual) block: named barrier `id`.
template <int B>
__device__ __forceinline__ void vblock_sync(uint32_t id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(B) : "memory");
}

// LLB / SLB over one (virtual) block of B threads: thread tid of block vb out
// of nvb, shared arrays of B (+1) entries, barrier `bar`.  The explore kernels
// below run it either as a real block (tid = threadIdx.x, barrier 0) or as
// one of several B-thread slices of a 512-thread block.
template <int B, bool STRIDED, int U, bool PAR>
__device__ __forceinline__ void explore_local_body(const BfsDevState *__restrict__ st,
                                                   uint32_t F, uint32_t tid, uint32_t vb,
                                                   uint32_t nvb, uint32_t *s_off,
                                                   uint32_t *s_dif, uint32_t *s_vid,
                                                   uint32_t *s_wsum, uint32_t bar) {
  constexpr int NW = B / 32;
  const uint32_t cur_q = st->cur;
  const uint32_t *__restrict__ qb = st->qb[cur_q];
  const uint32_t *__restrict__ qd = st->qd[cur_q];
  const uint32_t *__restrict__ qv = st->qv[cur_q];
  const uint32_t *__restrict__ inds = st->inds;
  uint32_t *vis = st->vis;
  int32_t *parent = PAR ? st->parent : nullptr;
  const uint32_t *perm = PAR ? st->perm : nullptr;
  const uint32_t lane = tid & 31u, warp = tid >> 5;
  const uint32_t num_tiles = (F + B - 1) / B;
  const uint64_t pol = evict_first_policy();

  for (uint32_t tile = vb; tile < num_tiles; tile += nvb) {
    const uint32_t slot = STRIDED ? tile + tid * num_tiles : tile * B + tid;
    uint32_t beg = 0, deg = 0, vid = 0;
    if (slot < F) {
      beg = qb[slot];
      deg = qd[slot];
      if (PAR) vid = qv[slot];
    }
    const uint32_t incl = warp_incl_scan(deg, lane);
    if (lane == 31) s_wsum[warp] = incl;
    vblock_sync<B>(bar);
    if (warp == 0) {
      uint32_t w = lane < (uint32_t)NW ? s_wsum[lane] : 0u;
      w = warp_incl_scan(w, lane);
      if (lane < (uint32_t)NW) s_wsum[lane] = w;
    }
    vblock_sync<B>(bar);
    const uint32_t total = s_wsum[NW - 1];
    const uint32_t off = (warp ? s_wsum[warp - 1] : 0u) + incl - deg;
    s_off[tid] = off;
    s_dif[tid] = beg - off;
    if (PAR) s_vid[tid] = vid;
    if (tid == 0) s_off[B] = total;
    vblock_sync<B>(bar);

    // even split of the tile's edges over the warps, in whole warp rounds
    const uint64_t per_warp = (((uint64_t)total + NW - 1) / NW + 31u) & ~31ull;
    const uint64_t w0_64 = (uint64_t)warp * per_warp;
    if (w0_64 < total) {
      const uint32_t w0 = (uint32_t)w0_64;
      const uint32_t w1 = (uint32_t)((w0_64 + per_warp < total) ? w0_64 + per_warp : total);
      // owner of w0: last entry with s_off <= w0 (broadcast reads)
      uint32_t lo = 0, hi = B;
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_off[mid] <= w0) lo = mid; else hi = mid;
      }
      uint32_t cur = lo;
      for (uint32_t base = w0; base < w1; base += 32u * U) {
        uint32_t addr[U], from[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const uint32_t rb = base + 32u * u;
          const uint32_t e = rb + lane;
          const uint32_t j = cur + 1u + lane;
          const uint32_t bnd = (j <= (uint32_t)B) ? s_off[j] : kFull;
          const uint32_t o = round_owner(cur, bnd, rb, lane);
          addr[u] = kFull;
          from[u] = 0;
          if (e < w1) {
            addr[u] = e + s_dif[o];
            if (PAR) from[u] = s_vid[o];
          }
          cur = __shfl_sync(kFull, o, 31);
          if (cur >= (uint32_t)B) cur = B - 1;  // only reached past w1
        }
        uint32_t nb[U];
#pragma unroll
        for (int u = 0; u < U; u++) nb[u] = addr[u] != kFull ? ld_stream(inds + addr[u], pol) : 0u;
#pragma unroll
        for (int u = 0; u < U; u++)
          if (addr[u] != kFull) visit(vis, nb[u], parent, PAR ? from[u] : 0u, perm);
      }
    }
    vblock_sync<B>(bar);
  }
}

template <int B, bool STRIDED, int U, bool PAR>
__global__ void __launch_bounds__(B, (MinBlocks<B, U, STRIDED>::value))
    explore_local_kernel(BfsDevState *__restrict__ st) {
  __shared__ uint32_t s_off[B + 1];
  __shared__ uint32_t s_dif[B];  // first edge - tile offset, mod 2^32
  __shared__ uint32_t s_vid[B];
  __shared__ uint32_t s_wsum[B / 32];
  const uint32_t F = st->F;
  if (F == 0) return;
  note_arm<(STRIDED ? 2 : 0) * 3 + BlockIndex<B>::value>(st);
  explore_local_body<B, STRIDED, U, PAR>(st, F, threadIdx.x, blockIdx.x, gridDim.x, s_off, s_dif,
                                         s_vid, s_wsum, 0u);
}

// ---- explore: GLB over 16-byte chunks of the edge array --------------------
// Edge-balanced (run_bfs_gpu.hpp:318-366 deals single edges over
// SMs * SM_FACTOR work-groups after a grid-wide scan of the frontier's
// degrees, EN1-EN3 at :203-307).  Here the frontier's edges are walked in
// chunk space: counting 16-byte chunks from the 16-byte boundary at or
// below inds, an entry whose edges are inds[b, b + deg) owns the chunks
// (b + off)/4 .. (b + off + deg - 1)/4 (off = st->inds_off), and the queue's
// qc array, written by level generation, is the exclusive prefix of those
// counts in queue order: the grid-wide scan.  The chunk space [0, EC) is cut
// into equal warp chunks dealt over the grid; a warp finds the owner of its
// first chunk with a 32-ary search of qc, then walks forward in rounds of
// 32 chunks, one per lane: one 16-byte load and one owner resolution serve
// four edge slots.  Owners are resolved with a warp OR-reduction of the next
// 32 entry starts plus a popc (O(1) per chunk, instead of the reference's
// per-edge binary search, :336-346).  The slots outside [b, b + deg) -- only
// in an entry's first and last chunk -- are masked off, and a chunk that
// reaches outside inds (the first one when off > 0, the last one when the
// array does not fill it) is read with scalar loads of its valid slots
// only.  U chunks per lane (4 U edge slots) are loaded per group, and the
// next group's loads are issued before the current group's probes.
//
// HUB: probes of internal ids below hub_lim first test the block's
// shared-memory copy s_hub of those bits of the visited bitmap (the hub
// prefix under the hub layout); a set bit there means visited and no global
// probe is made.  A clear one says nothing about claims made since by other
// blocks, so the global test-then-claim follows, and a claimed hub's bit is
// then set in s_hub for the block's later probes (bits only ever go from 0
// to 1, so any snapshot is a valid "already visited" set).
// Chunks per lane and group of the chunk walk, whatever the ipt option: with
// the next group's loads in flight that is 16 edge slots per lane, at the
// 64 registers of a 1024-thread block (4 chunks per group spill).
constexpr int kChunkGroup = 2;

template <int U, bool PAR, bool HUB>
__device__ __forceinline__ void explore_chunk_body(const BfsDevState *__restrict__ st,
                                                   uint32_t F, uint32_t gw,
                                                   uint32_t total_warps, uint32_t *s_hub,
                                                   uint32_t hub_lim) {
  constexpr uint32_t kRound = 32u * U;
  constexpr uint32_t kMinChunk = kRound * kGlbGroups;
  const uint32_t EC = st->EC;
  const uint32_t cur_q = st->cur;
  const uint32_t *__restrict__ qb = st->qb[cur_q];
  const uint32_t *__restrict__ qd = st->qd[cur_q];
  const uint32_t *__restrict__ qc = st->qc[cur_q];
  const uint32_t *__restrict__ qv = st->qv[cur_q];
  const uint32_t off = st->inds_off;
  // chunk k is bytes [16 k, 16 k + 16) from the boundary at or below inds
  const uint32_t *__restrict__ inds0 = st->inds - off;
  const uint4 *__restrict__ inds4 = reinterpret_cast<const uint4 *>(inds0);
  // chunks lo4 .. hi4 - 1 lie wholly inside inds
  const uint32_t lo4 = off ? 1u : 0u;
  const uint32_t hi4 = (st->nnz + off) >> 2;
  uint32_t *vis = st->vis;
  const uint32_t *vis_c = vis;  // plain loads of the visited words
  const uint32_t s_hub_addr = HUB ? (uint32_t)__cvta_generic_to_shared(s_hub) : 0u;
  int32_t *parent = PAR ? st->parent : nullptr;
  const uint32_t *perm = PAR ? st->perm : nullptr;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t le_mask = (2u << lane) - 1u;  // lanes 0 .. lane (all for lane 31)
  const uint64_t pol = evict_first_policy();
  // about four warp chunks per warp, whole groups of U rounds
  uint64_t ch = ((uint64_t)EC + 4ull * total_warps - 1) / (4ull * total_warps);
  ch = (ch + kRound - 1) / kRound * kRound;
  const uint32_t CHUNK = (uint32_t)(ch > kMinChunk ? ch : kMinChunk);
  const uint32_t n_chunks = (uint32_t)(((uint64_t)EC + CHUNK - 1) / CHUNK);

  for (uint32_t c = gw; c < n_chunks; c += total_warps) {
    const uint32_t w0 = c * CHUNK;  // < EC
    const uint32_t w1 = (uint32_t)min((uint64_t)EC, (uint64_t)w0 + CHUNK);
    uint32_t cur = warp_owner_search(qc, F, w0, lane);
    // the current owner: chunk offset (b >> 2) - qc (mod 2^32), edge range
    // [cb, ce) counted from inds0 (edge p of inds is at p + off), vertex id
    uint32_t cb = qb[cur] + off;
    uint32_t ce = cb + qd[cur];
    uint32_t cd = (cb >> 2) - qc[cur];
    uint32_t cv = PAR ? qv[cur] : 0u;
    // window: entries c0 + 1 .. c0 + 32, one per lane (chunk start, offset,
    // edge range, id); re-based only when a round could leave it
    uint32_t c0 = cur, bnd, wd, wb, we, wv;
    auto load_window = [&]() {
      const uint32_t j = c0 + 1u + lane;
      bnd = (j <= F) ? qc[j] : kFull;  // qc[F] = EC
      wb = we = wd = wv = 0u;
      if (j < F) {
        wb = qb[j] + off;
        we = wb + qd[j];
        wd = (wb >> 2) - bnd;
        if (PAR) wv = qv[j];
      }
    };
    load_window();
    uint32_t wlast = __shfl_sync(kFull, bnd, 31);
    // Resolves the U rounds of chunks starting at chunk `base` and issues
    // their 16-byte loads: q (slots), m (valid-slot mask, bit i = slot i),
    // fr (source id, with parents).
    auto resolve = [&](uint32_t base, uint4 (&q)[U], uint32_t (&m)[U], uint32_t (&fr)[U]) {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const uint32_t rb = base + 32u * u;
        const uint32_t x = rb + lane;
        if (wlast < rb || wlast - rb < 31u) {  // warp-uniform
          c0 = cur;
          load_window();
          wlast = __shfl_sync(kFull, bnd, 31);
        }
        // entries at or before cur start before rb: their p wraps past 32
        const uint32_t starts = __reduce_or_sync(kFull, bit_or_zero(bnd - rb));
        const uint32_t k = __popc(starts & le_mask);
        const uint32_t srcl = k ? cur + k - c0 - 1u : 0u;
        const uint32_t sd = __shfl_sync(kFull, wd, srcl);
        const uint32_t sb = __shfl_sync(kFull, wb, srcl);
        const uint32_t se = __shfl_sync(kFull, we, srcl);
        const uint32_t sv = PAR ? __shfl_sync(kFull, wv, srcl) : 0u;
        const uint32_t d = k ? sd : cd, b = k ? sb : cb, e = k ? se : ce;
        fr[u] = PAR ? (k ? sv : cv) : 0u;
        m[u] = 0u;
        q[u] = make_uint4(0u, 0u, 0u, 0u);
        if (x < w1) {
          const uint32_t a4 = x + d;    // chunk index from inds0
          const uint32_t p0 = a4 << 2;  // position of its slot 0
          const uint32_t lo = b > p0 ? b - p0 : 0u;        // 0 .. 3
          const uint32_t hi = e - p0 < 4u ? e - p0 : 4u;   // 1 .. 4
          m[u] = (0xFu >> (4u - hi)) & (0xFu << lo);
          if (a4 >= lo4 && a4 < hi4) {
            q[u] = ld_stream4(inds4 + a4, pol);
          } else {  // a chunk that reaches outside inds: its valid slots only
            uint32_t t[4] = {0u, 0u, 0u, 0u};
#pragma unroll
            for (int i = 0; i < 4; i++)
              if ((m[u] >> i) & 1u) t[i] = ld_stream(inds0 + p0 + i, pol);
            q[u] = make_uint4(t[0], t[1], t[2], t[3]);
          }
        }
        // the owner of lane 31 is entry cur + popc(starts)
        const uint32_t k31 = __popc(starts);
        if (k31) {
          cur += k31;
          const uint32_t sl = cur - c0 - 1u;
          cd = __shfl_sync(kFull, wd, sl);
          cb = __shfl_sync(kFull, wb, sl);
          ce = __shfl_sync(kFull, we, sl);
          if (PAR) cv = __shfl_sync(kFull, wv, sl);
        }
      }
    };
    // Probes of the U chunks of a lane, branch-free: for every slot a
    // predicated shared load of the hub word (hub ids only), then a
    // predicated global load of the visited word (valid slots the hub word
    // did not show visited); a slot whose word shows its bit clear gets a
    // bit in need[u].  Only then, behind one branch per chunk, the claims --
    // a claim is an asm statement that orders memory, so no load may follow
    // it within the group.
    auto probe = [&](const uint4 (&q)[U], const uint32_t (&m)[U], const uint32_t (&fr)[U]) {
      uint32_t need[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const uint32_t n4[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
        need[u] = 0u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const uint32_t n = n4[i];
          const uint32_t bit = 1u << (n & 31u);
          uint32_t act = (m[u] >> i) & 1u;
          if (HUB) {
            uint32_t h = 0u;
            ld_shared_if(h, s_hub_addr + ((n >> 5) << 2), act & (n < hub_lim ? 1u : 0u));
            act &= (h & bit) ? 0u : 1u;
          }
          uint32_t word = bit;  // "visited" unless loaded
          ld_global_if(word, vis_c + (n >> 5), act);
          need[u] |= ((word & bit) ? 0u : 1u) << i;
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (need[u] == 0u) continue;
        const uint32_t n4[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (!((need[u] >> i) & 1u)) continue;
          const uint32_t n = n4[i];
          claim(vis, n, parent, fr[u], perm);
          if (HUB && n < hub_lim) atomicOr(s_hub + (n >> 5), 1u << (n & 31u));
        }
      }
    };
    // Software pipeline: the loads of the next U rounds are issued before
    // the probes of the current ones, so that they overlap.
    uint4 q[U], q2[U];
    uint32_t m[U], m2[U], fr[U], fr2[U];
    resolve(w0, q, m, fr);
    for (uint32_t base = w0; base < w1; base += kRound) {
      const bool more = base + kRound < w1;  // warp-uniform; no overflow: w1 < 2^32 - kRound
      if (more) resolve(base + kRound, q2, m2, fr2);
      probe(q, m, fr);
      if (!more) break;
#pragma unroll
      for (int u = 0; u < U; u++) {
        q[u] = q2[u];
        m[u] = m2[u];
        fr[u] = fr2[u];
      }
    }
  }
}

// The GLB arms' own kernel (the engine runs GLB levels in explore_any; the
// allocation-free entry point launches this one): 1024 threads per SM.
template <int B, int U, bool PAR>
__global__ void __launch_bounds__(B, 1024 / B)
    explore_global_kernel(BfsDevState *__restrict__ st) {
  const uint32_t F = st->F;
  if (F == 0) return;
  note_arm<1 * 3 + BlockIndex<B>::value>(st);
  explore_chunk_body<kChunkGroup, PAR, false>(st, F, blockIdx.x * (B / 32) + (threadIdx.x >> 5),
                                              gridDim.x * (B / 32), nullptr, 0u);
}

// ---- explore: any arm, chosen on the device ---------------------------------
// One kAnyBlock-thread kernel, one block per SM, that runs any arm: the arm
// passed in (arm_in >= 0; the GLB arms always run here, and so does every
// arm the per-level recorder times) or, with arm_in < 0, the arm the learned
// scheduler stored in st->arm (init or the last block of the previous level
// generation picked it), so the learned loop needs no switch node.
//   GLB  the 16-byte chunk walk, chunks dealt per warp over the grid (the
//        block size of the arm does not matter).  With a hub layout, levels
//        of at least hub_min_edges edges, once at least half as many
//        vertices as the prefix holds have been reached, first copy the hub
//        prefix of the visited bitmap into the block's dynamic shared memory
//        (s_hub) and probe through it.
//   LLB / SLB  tiles of 128, 256 or 512 entries on 8, 4 or 2 slices of the
//        block, each with its own shared arrays and named barrier.
template <int U, bool PAR>
__global__ void __launch_bounds__(kAnyBlock, 1)
    explore_any_kernel(BfsDevState *__restrict__ st, int arm_in) {
  extern __shared__ __align__(16) uint32_t s_hub[];
  __shared__ uint32_t s_off[kAnyBlock + 8];
  __shared__ uint32_t s_dif[kAnyBlock];
  __shared__ uint32_t s_vid[kAnyBlock];
  __shared__ uint32_t s_wsum[kAnyBlock / 32];
  const uint32_t F = st->F;
  if (F == 0) return;
  const int arm = arm_in >= 0 ? arm_in : st->arm;  // uniform over the grid
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t l = st->lvl;
    if (l < st->rec_cap) st->rec_ran[l] = arm;
  }
  const int form = arm / 3, bi = arm % 3;
  const uint32_t t = threadIdx.x;
  if (form == BFS_LB_GLB) {
    const uint32_t hw = st->hub_words;  // a multiple of 4
    // uniform over the grid; a level that reached fewer vertices than half
    // the prefix would find few hubs visited and skips the copy
    const bool use = hw != 0 && st->EF >= st->hub_min_edges && st->reached >= hw * 16u;
    if (use) {
      const uint4 *src = reinterpret_cast<const uint4 *>(st->vis);
      uint4 *dst = reinterpret_cast<uint4 *>(s_hub);
      for (uint32_t i = t; i < (hw >> 2); i += kAnyBlock) dst[i] = src[i];
      __syncthreads();
    }
    explore_chunk_body<kChunkGroup, PAR, true>(st, F, blockIdx.x * (kAnyBlock / 32) + (t >> 5),
                                               gridDim.x * (kAnyBlock / 32), s_hub,
                                               use ? hw * 32u : 0u);
  } else if (bi == 2) {
    const uint32_t v = t >> 9, o = v * 513u;
    if (form == BFS_LB_SLB)
      explore_local_body<512, true, U, PAR>(st, F, t & 511u, blockIdx.x * 2 + v, gridDim.x * 2,
                                            s_off + o, s_dif + v * 512, s_vid + v * 512,
                                            s_wsum + v * 16, 1u + v);
    else
      explore_local_body<512, false, U, PAR>(st, F, t & 511u, blockIdx.x * 2 + v, gridDim.x * 2,
                                             s_off + o, s_dif + v * 512, s_vid + v * 512,
                                             s_wsum + v * 16, 1u + v);
  } else if (bi == 1) {
    const uint32_t v = t >> 8, o = v * 257u;
    if (form == BFS_LB_SLB)
      explore_local_body<256, true, U, PAR>(st, F, t & 255u, blockIdx.x * 4 + v, gridDim.x * 4,
                                            s_off + o, s_dif + v * 256, s_vid + v * 256,
                                            s_wsum + v * 8, 1u + v);
    else
      explore_local_body<256, false, U, PAR>(st, F, t & 255u, blockIdx.x * 4 + v, gridDim.x * 4,
                                             s_off + o, s_dif + v * 256, s_vid + v * 256,
                                             s_wsum + v * 8, 1u + v);
  } else {
    const uint32_t v = t >> 7, o = v * 129u;
    if (form == BFS_LB_SLB)
      explore_local_body<128, true, U, PAR>(st, F, t & 127u, blockIdx.x * 8 + v, gridDim.x * 8,
                                            s_off + o, s_dif + v * 128, s_vid + v * 128,
                                            s_wsum + v * 4, 1u + v);
    else
      explore_local_body<128, false, U, PAR>(st, F, t & 127u, blockIdx.x * 8 + v, gridDim.x * 8,
                                             s_off + o, s_dif + v * 128, s_vid + v * 128,
                                             s_wsum + v * 4, 1u + v);
  }
}

// ---- level generation -----------------------------------------------------
// Returns the new level's counters (for the fused scheduler, without a
// round trip through global memory).
__device__ LevelCounters finish_level(BfsDevState *st, unsigned long long cond, int use_cond) {
  const unsigned long long packed = *(volatile unsigned long long *)&st->next_packed;
  const uint32_t f_new = (uint32_t)(packed >> 32);
  const uint32_t ec_new = (uint32_t)packed;
  const uint32_t ef_new = *(volatile uint32_t *)&st->next_edges;
  const uint32_t lvl = st->lvl + 1;
  const uint32_t reached = *(volatile uint32_t *)&st->reached;
  if (reached > st->reached_prev) st->max_level = lvl;
  st->reached_prev = reached;
  st->edges_count += ef_new;
  const uint32_t nq = st->cur ^ 1u;
  st->qc[nq][f_new] = ec_new;  // trailing total of the new queue's scan
  st->cur = nq;
  st->F = f_new;
  st->EF = ef_new;
  st->EC = ec_new;
  st->lvl = lvl;
  st->next_packed = 0;
  st->next_edges = 0;
  st->done_blocks = 0;
  st->lg_cursor = 0;
  st->launches += 2;
  if (lvl < st->rec_cap) {
    st->rec_frontier[lvl] = f_new;
    st->rec_edges[lvl] = ef_new;
    st->rec_arm[lvl] = -1;
  }
  if (f_new > 0 && lvl >= st->level_cap) {
    st->error |= BFS_DEVERR_LEVEL_LIMIT;
    st->F = 0;
  }
  if (use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, st->F > 0);
  return LevelCounters{st->F, ef_new, reached, lvl};
}

// Merges new-vertex bits into one 4-byte word of working levels (one byte
// per vertex): bytes whose bit in the low nibble of `bits` is set take the
// matching byte of `rep`.  The nibble is spread to bytes by one multiply (its
// shifted copies land on distinct bit positions, so no carries).
__device__ __forceinline__ uint32_t merge_levels(uint32_t word, uint32_t bits, uint32_t rep) {
  const uint32_t m = (((bits & 0xFu) * 0x00204081u) & 0x01010101u) * 0xFFu;
  return (word & ~m) | (rep & m);
}

// Level generation.  After a level that explored many edges, blocks claim
// spans of B bitmap words (one word per thread) from a counter -- the
// density of new vertices is uneven over the bitmap -- and load each span's
// words while working on the previous one.  The thread owning a word merges
// its new vertices' levels into the working levels: the word's 32 vertices
// are one 32-byte sector there, read when the word is seen and written back
// whole once the block's list is built.  The block lists the span's new
// vertices (vis & ~prev) in shared memory in vertex order (a block scan of
// the words' popcounts; each thread walks its word's set bits), then every
// warp takes an equal share of the list, whatever the bit layout.  Pass 1
// loads each entry's indptr pair (kLgUnroll rounds of loads in flight per
// lane), compacts the kept entries in place with their offset and degree,
// and counts them, their degrees and their 16-byte chunks; thread 0 reserves
// the block's queue slots and chunk offsets with one atomic -- slots and the
// chunk prefix must come from the same atomic, so that the prefix is in slot
// order; pass 2 writes the kept entries in 32-slot windows aligned to 128
// bytes, so that the queue stores fill whole sectors.  Four block barriers
// per span with new vertices, one per span without.  Degree and vertex
// totals go to the level's counters once per block, at the end.
//
// After a level that explored fewer than words / 8 edges (at most that many
// words hold new vertices, and on graphs of large diameter they are spread
// thinly over every span) the warps work on their own, without block
// barriers: warp g of the grid takes the 32-word groups g, g + G, g + 2G, ...
// (G warps), four groups' words in flight at a time, writes the new
// vertices' working levels as single bytes, lists them in its own slice of
// the list and runs pass 1, one queue reservation and pass 2 on the slice
// when the next group's entries would not fit in it, and at the end.
constexpr int kLgUnroll = 8;
constexpr int kLgMinBlocks = 3;  // 768 threads per SM: at most 80 registers
constexpr int kLgSparseGroups = 4;  // 32-word groups per warp step (sparse levels)

template <int B, bool PAR>
__global__ void __launch_bounds__(B, kLgMinBlocks) levelgen_kernel(BfsDevState *__restrict__ st,
                                                                   unsigned long long cond,
                                                                   int use_cond) {
  constexpr int NW = B / 32;
  constexpr uint32_t kSpan = B;         // words per block and step
  constexpr uint32_t kCap = kSpan * 32u;  // list capacity: every vertex of a span
  constexpr uint32_t kSlice = kCap / NW;  // a warp's slice: every vertex of 32 words
  static_assert((NW & (NW - 1)) == 0, "warps per block: a power of two");
  static_assert(kSlice == 1024u, "a warp's slice holds 32 words' vertices");
  static_assert(kSchedParams <= kCap, "the model must fit the list buffer");
  // list: entry (vertex id, bit 31 the moved flag), then its indptr offset;
  // degrees; original ids (parents only)
  extern __shared__ __align__(16) uint32_t s_dyn[];
  uint32_t *__restrict__ s_b = s_dyn;
  uint32_t *__restrict__ s_d = s_dyn + kCap;
  uint32_t *__restrict__ s_o = s_dyn + 2 * kCap;
  __shared__ uint32_t s_wc[2][NW];
  __shared__ unsigned long long s_wtot[NW];
  __shared__ uint32_t s_wdeg[NW];
  __shared__ uint32_t s_wreach[NW];
  __shared__ unsigned long long s_base;
  __shared__ uint32_t s_sb[2];
  __shared__ int s_last;
  __shared__ LevelCounters s_ctr;

  const uint32_t words = st->words;
  uint32_t *__restrict__ V = st->vis;
  uint32_t *__restrict__ P = st->prev;
  const uint32_t *__restrict__ indptr = st->indptr;
  const uint32_t n_rows = st->n_rows;
  const int32_t lvl_next = (int32_t)st->lvl + 1;
  int32_t *__restrict__ level = st->level;  // deep levels only
  uint8_t *__restrict__ lv8 = st->lv8;
  const uint32_t nq = st->cur ^ 1u;
  uint32_t *__restrict__ qb = st->qb[nq];
  uint32_t *__restrict__ qd = st->qd[nq];
  uint32_t *__restrict__ qc = st->qc[nq];
  uint32_t *__restrict__ qv = st->qv[nq];
  const uint32_t off = st->inds_off;
  const uint32_t *__restrict__ perm = st->perm;    // internal -> original (null: identity)
  const uint32_t *__restrict__ moved = st->moved;  // bit v: perm[v] != v
  // relabelled graphs have fewer than 2^31 vertices: bit 31 of a list entry
  // is then free for the moved flag
  const uint32_t id_mask = moved ? 0x7FFFFFFFu : 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t rep = (lvl_next < (int32_t)kLv8Deep ? (uint32_t)lvl_next : kLv8Deep) *
                       0x01010101u;  // the new level in every byte
  // new vertices and kept entries' degrees counted by this lane (summed over
  // the block at the end)
  uint32_t my_reached = 0, my_deg = 0;

  // the working levels of word w with new bits x: sector (l0, l1) merged and
  // written back; a deep level also goes to the output (original ids)
  auto write_levels = [&](uint32_t w, uint32_t x, uint32_t xm, uint4 l0, uint4 l1) {
    uint4 *__restrict__ sec = reinterpret_cast<uint4 *>(lv8) + 2u * (size_t)w;
    l0.x = merge_levels(l0.x, x, rep);
    l0.y = merge_levels(l0.y, x >> 4, rep);
    l0.z = merge_levels(l0.z, x >> 8, rep);
    l0.w = merge_levels(l0.w, x >> 12, rep);
    l1.x = merge_levels(l1.x, x >> 16, rep);
    l1.y = merge_levels(l1.y, x >> 20, rep);
    l1.z = merge_levels(l1.z, x >> 24, rep);
    l1.w = merge_levels(l1.w, x >> 28, rep);
    sec[0] = l0;
    sec[1] = l1;
    if (lvl_next >= (int32_t)kLv8Deep) {
      for (uint32_t y = x; y; y &= y - 1u) {
        const uint32_t bpos = (uint32_t)(__ffs(y) - 1);
        const uint32_t v = w * 32u + bpos;
        level[((xm >> bpos) & 1u) ? perm[v] : v] = lvl_next;
      }
    }
  };
  // Pass 1 over list entries [lo, hi) (one warp): every round's loads are
  // issued before their first use; kept entries (degree > 0) are compacted
  // in place, in list order, to [lo, lo + count) -- positions only move down
  // and an iteration's entries are already in registers.  Returns the warp's
  // kept count, degree and chunk sums (uniform over the warp).
  auto pass1 = [&](uint32_t lo, uint32_t hi, uint32_t &n_cnt, uint32_t &n_deg,
                   uint32_t &n_chk) {
    n_cnt = n_deg = n_chk = 0;
    for (uint32_t t0 = lo; t0 < hi; t0 += 32u * kLgUnroll) {
      uint32_t b[kLgUnroll], e[kLgUnroll], o[kLgUnroll];
#pragma unroll
      for (int r = 0; r < kLgUnroll; r++) {
        const uint32_t i = t0 + 32u * r + lane;
        b[r] = e[r] = 0;
        o[r] = 0;
        if (i < hi) {
          const uint32_t ent = s_b[i];
          const uint32_t v = ent & id_mask;
          if (PAR) o[r] = (ent & ~id_mask) ? perm[v] : v;
          if (v < n_rows) {
            b[r] = indptr[v];
            e[r] = indptr[v + 1];
          }
        }
      }
#pragma unroll
      for (int r = 0; r < kLgUnroll; r++) {
        const uint32_t deg = e[r] - b[r];  // 0 past hi
        const uint32_t km = __ballot_sync(kFull, deg > 0u);
        if (deg) {
          const uint32_t p = lo + n_cnt + __popc(km & lt_mask);
          s_b[p] = b[r];
          s_d[p] = deg;
          if (PAR) s_o[p] = o[r];
        }
        n_cnt += __popc(km);
        n_deg += deg;
        n_chk += edge_chunks(b[r], deg, off);
      }
    }
    n_deg = __reduce_add_sync(kFull, n_deg);
    n_chk = __reduce_add_sync(kFull, n_chk);
  };
  // Pass 2 (one warp): the n_cnt kept entries at [lo, lo + n_cnt) to queue
  // slots from wb (slot << 32 | chunk offset), in 32-slot windows aligned to
  // 128 bytes, two windows per step (their scans overlap).
  auto pass2 = [&](uint32_t lo, uint32_t n_cnt, unsigned long long wb) {
    const uint32_t slot0 = (uint32_t)(wb >> 32), end = slot0 + n_cnt;
    uint32_t prefc = (uint32_t)wb;
    for (uint32_t ws = slot0 & ~31u; ws < end; ws += 64u) {
      uint32_t b[2], deg[2], nch[2], cincl[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const uint32_t sl = ws + 32u * h + lane;
        b[h] = deg[h] = 0;
        if (sl >= slot0 && sl < end) {
          b[h] = s_b[lo + (sl - slot0)];
          deg[h] = s_d[lo + (sl - slot0)];
        }
        nch[h] = edge_chunks(b[h], deg[h], off);
        cincl[h] = warp_incl_scan(nch[h], lane);
      }
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const uint32_t sl = ws + 32u * h + lane;
        if (deg[h]) {  // exactly the slots in [slot0, end)
          qb[sl] = b[h];
          qd[sl] = deg[h];
          qc[sl] = prefc + cincl[h] - nch[h];
          if (PAR) qv[sl] = s_o[lo + (sl - slot0)];
        }
        prefc += __shfl_sync(kFull, cincl[h], 31);
      }
    }
  };

  if (st->EF >= (words >> 3)) {  // uniform over the grid: the block path
    if (threadIdx.x == 0) s_sb[0] = atomicAdd(&st->lg_cursor, kSpan);
    __syncthreads();
    uint32_t sb = s_sb[0];
    // this thread's word of the current span: vis, prev, moved
    uint32_t vw = 0, pw = 0, mw = 0;
    if (sb + threadIdx.x < words) {
      vw = V[sb + threadIdx.x];
      pw = P[sb + threadIdx.x];
      if (moved) mw = moved[sb + threadIdx.x];
    }
    for (uint32_t step = 0; sb < words; step ^= 1u) {
      const uint32_t w = sb + threadIdx.x;
      uint32_t x = vw & ~pw;
      const uint32_t xn = x, xm = mw;
      // the word's working levels, merged and written back after the list
      uint4 l0 = make_uint4(0u, 0u, 0u, 0u), l1 = l0;
      if (x) {  // x != 0 only for words < words
        P[w] = vw;
        const uint4 *sec = reinterpret_cast<const uint4 *>(lv8) + 2u * (size_t)w;
        l0 = sec[0];
        l1 = sec[1];
      }
      const uint32_t c = __popc(x);
      const uint32_t incl = warp_incl_scan(c, lane);
      if (lane == 31) s_wc[step][warp] = incl;
      if (threadIdx.x == 0) s_sb[step ^ 1u] = atomicAdd(&st->lg_cursor, kSpan);
      __syncthreads();
      uint32_t L = 0, woff = 0;
#pragma unroll
      for (int i = 0; i < NW; i++) {
        const uint32_t y = s_wc[step][i];
        woff += (uint32_t)i < warp ? y : 0u;
        L += y;
      }
      // the next span's words, in flight while this span is worked on
      sb = s_sb[step ^ 1u];
      vw = pw = mw = 0;
      if (sb + threadIdx.x < words) {
        vw = V[sb + threadIdx.x];
        pw = P[sb + threadIdx.x];
        if (moved) mw = moved[sb + threadIdx.x];
      }
      if (L == 0) continue;  // uniform over the block
      if (threadIdx.x == 0) my_reached += L;
      {
        uint32_t pos = woff + incl - c;
        const uint32_t vbase = w * 32u;
        while (x) {
          const uint32_t bpos = (uint32_t)(__ffs(x) - 1);
          s_b[pos++] = (vbase + bpos) | (((xm >> bpos) & 1u) << 31);
          x &= x - 1u;
        }
      }
      if (xn) write_levels(w, xn, xm, l0, l1);
      __syncthreads();
      // this warp's share of the list
      const uint32_t lo = (L * warp) / NW, hi = (L * (warp + 1u)) / NW;
      uint32_t n_cnt, n_deg, n_chk;
      pass1(lo, hi, n_cnt, n_deg, n_chk);
      if (lane == 0) {
        s_wtot[warp] = ((unsigned long long)n_cnt << 32) | n_chk;
        s_wdeg[warp] = n_deg;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int i = 0; i < NW; i++) {
          const unsigned long long y = s_wtot[i];
          s_wtot[i] = run;
          run += y;
          my_deg += s_wdeg[i];
        }
        s_base = run ? atomicAdd(&st->next_packed, run) : 0ull;
      }
      __syncthreads();
      if (n_cnt) pass2(lo, n_cnt, s_base + s_wtot[warp]);
      // the list is rewritten only after the next span's first barrier, so
      // pass 2 needs no trailing barrier
    }
  } else {  // the warp path (sparse levels)
    const uint32_t groups = words >> 5;  // words is a multiple of 32
    const uint32_t gwarp = blockIdx.x * NW + warp, nwarps = gridDim.x * NW;
    const uint32_t lo = warp * kSlice;  // this warp's slice of the list
    uint32_t size = 0;                  // entries in the slice
    auto flush = [&]() {
      uint32_t n_cnt, n_deg, n_chk;
      pass1(lo, lo + size, n_cnt, n_deg, n_chk);
      if (n_cnt) {
        unsigned long long wb = 0;
        if (lane == 0) {
          wb = atomicAdd(&st->next_packed, ((unsigned long long)n_cnt << 32) | n_chk);
          my_deg += n_deg;
        }
        pass2(lo, n_cnt, __shfl_sync(kFull, wb, 0));
      }
      size = 0;
      __syncwarp();  // pass 2's reads of the slice are done
    };
    for (uint32_t g0 = gwarp; g0 < groups; g0 += kLgSparseGroups * nwarps) {
      uint32_t vw[kLgSparseGroups], pw[kLgSparseGroups], mw[kLgSparseGroups];
#pragma unroll
      for (int k = 0; k < kLgSparseGroups; k++) {
        const uint32_t g = g0 + k * nwarps;
        vw[k] = pw[k] = mw[k] = 0;
        if (g < groups) {
          vw[k] = V[g * 32u + lane];
          pw[k] = P[g * 32u + lane];
          if (moved) mw[k] = moved[g * 32u + lane];
        }
      }
#pragma unroll
      for (int k = 0; k < kLgSparseGroups; k++) {
        uint32_t x = vw[k] & ~pw[k];
        if (!__any_sync(kFull, x != 0u)) continue;  // uniform over the warp
        const uint32_t w = (g0 + k * nwarps) * 32u + lane;
        if (x) P[w] = vw[k];
        const uint32_t c = __popc(x);
        const uint32_t incl = warp_incl_scan(c, lane);
        const uint32_t tot = __shfl_sync(kFull, incl, 31);
        my_reached += c;
        if (size + tot > kSlice) flush();
        uint32_t pos = lo + size + incl - c;
        const uint32_t vbase = w * 32u;
        // few new vertices per word here: their working levels are single
        // byte stores (the array is in L2), with no read of the sector
        while (x) {
          const uint32_t bpos = (uint32_t)(__ffs(x) - 1);
          const uint32_t mv = (mw[k] >> bpos) & 1u;
          s_b[pos++] = (vbase + bpos) | (mv << 31);
          lv8[vbase + bpos] = (uint8_t)rep;
          if (lvl_next >= (int32_t)kLv8Deep) {
            const uint32_t v = vbase + bpos;
            level[mv ? perm[v] : v] = lvl_next;
          }
          x &= x - 1u;
        }
        size += tot;
        __syncwarp();  // the slice's entries are written
      }
    }
    if (size) flush();
  }

  // Block totals, then the ticket.  Learned runs: every block copies the
  // model into its (now unused) list buffer while thread 0 takes the ticket,
  // so that the last block -- which picks the next level's arm -- holds it by
  // the time it knows it is last.  Thread 0 stays out of the copy: its fence
  // would otherwise wait for its share of the loads.
  my_reached = __reduce_add_sync(kFull, my_reached);
  if (lane == 0) {
    s_wreach[warp] = my_reached;
    s_wdeg[warp] = my_deg;
  }
  __syncthreads();  // also: every warp is done with the list
  const float *w = st->sched_w;
  float *s_w = reinterpret_cast<float *>(s_dyn);
  if (threadIdx.x == 0) {
    uint32_t reached = 0, deg_sum = 0;
#pragma unroll
    for (int i = 0; i < NW; i++) {
      reached += s_wreach[i];
      deg_sum += s_wdeg[i];
    }
    if (deg_sum) atomicAdd(&st->next_edges, deg_sum);  // a total: order does not matter
    if (reached) atomicAdd(&st->reached, reached);
    __threadfence();
    const uint32_t ticket = atomicAdd(&st->done_blocks, 1u);
    s_last = (ticket == gridDim.x - 1);
  } else if (w != nullptr) {
    stage_weights(s_w, w, 1u);
  }
  __syncthreads();
  if (s_last) {  // uniform over the block
    // the arm of the level just generated, for the explore_any launch of
    // the next loop iteration
    if (threadIdx.x == 0) {
      __threadfence();
      s_ctr = finish_level(st, cond, use_cond);
    }
    __syncthreads();
    if (w != nullptr && warp == 0) fused_sched_pick(st, s_ctr, s_w);
  }
}

// ---- validation (Graph500-style checks of a level array) --------------------
// Edge pass, edge-balanced: each thread takes kValEdges consecutive edges,
// finds the first one's source by binary search over indptr and walks on.
// For every expanded reached u and edge u->v: level[v] must be reached and
// <= level[u] + 1; v gets a witness if level[v] == level[u] + 1, and its
// parent is confirmed if parent[v] == u.
constexpr uint32_t kValEdges = 16;

__global__ void validate_edges_kernel(const uint32_t *__restrict__ indptr,
                                      const uint32_t *__restrict__ inds, uint32_t n_rows,
                                      const int32_t *__restrict__ level,
                                      const int32_t *__restrict__ parent,
                                      uint8_t *witness, uint8_t *parent_ok,
                                      unsigned long long *bad) {
  const uint32_t total = indptr[n_rows];  // edges of expandable vertices
  uint32_t nbad = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kValEdges;
  for (uint64_t e0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kValEdges;
       e0 < total; e0 += stride) {
    uint32_t lo = 0, hi = n_rows;  // last u with indptr[u] <= e0
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (indptr[mid] <= e0) lo = mid; else hi = mid;
    }
    uint32_t u = lo;
    const uint32_t e1 = (uint32_t)min((uint64_t)total, e0 + kValEdges);
    for (uint32_t e = (uint32_t)e0; e < e1; e++) {
      while (indptr[u + 1] <= e) u++;
      const int32_t lu = level[u];
      if (lu < 0) continue;
      const uint32_t v = inds[e];
      const int32_t lv = level[v];
      if (lv < 0 || lv > lu + 1) nbad++;
      if (lv == lu + 1) {
        witness[v] = 1;
        if (parent && parent[v] == (int32_t)u) parent_ok[v] = 1;
      }
    }
  }
  nbad = __reduce_add_sync(kFull, nbad);
  if ((threadIdx.x & 31u) == 0 && nbad) atomicAdd(bad, (unsigned long long)nbad);
}

// Vertex pass: root at level 0 (and its own parent); any other reached vertex
// needs a witness in-edge and, with parents, a confirmed parent.
__global__ void validate_vertices_kernel(uint32_t n_cols, uint32_t root,
                                         const int32_t *__restrict__ level,
                                         const int32_t *__restrict__ parent,
                                         const uint8_t *witness, const uint8_t *parent_ok,
                                         unsigned long long *bad) {
  uint32_t nbad = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n_cols;
       v += gridDim.x * blockDim.x) {
    const int32_t lv = level[v];
    if (v == root) {
      if (lv != 0) nbad++;
      if (parent && parent[v] != (int32_t)root) nbad++;
      continue;
    }
    if (lv == 0) nbad++;
    if (lv > 0 && !witness[v]) nbad++;
    if (parent) {
      if (lv > 0 && !parent_ok[v]) nbad++;
      if (lv < 0 && parent[v] != -1) nbad++;
    }
  }
  nbad = __reduce_add_sync(kFull, nbad);
  if ((threadIdx.x & 31u) == 0 && nbad) atomicAdd(bad, (unsigned long long)nbad);
}

// CSC check used at upload: indptr monotone, indptr[0] == 0, last == nnz,
// every destination < n_cols.
__global__ void check_csc_kernel(const uint32_t *__restrict__ indptr,
                                 const uint32_t *__restrict__ inds, uint32_t n_cols,
                                 uint64_t nnz, unsigned long long *bad) {
  uint32_t nbad = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (uint64_t v = tid; v < n_cols; v += stride)
    if (indptr[v + 1] < indptr[v]) nbad++;
  if (tid == 0 && (indptr[0] != 0 || (uint64_t)indptr[n_cols] != nnz)) nbad++;
  for (uint64_t k = tid; k < nnz; k += stride)
    if (inds[k] >= n_cols) nbad++;
  nbad = __reduce_add_sync(kFull, nbad);
  if ((threadIdx.x & 31u) == 0 && nbad) atomicAdd(bad, (unsigned long long)nbad);
}

// ---- kernel table ---------------------------------------------------------
template <int U, bool PAR>
static const void *explore_fn_u(int arm) {
  switch (arm) {
    case 0: return (const void *)explore_local_kernel<128, false, U, PAR>;
    case 1: return (const void *)explore_local_kernel<256, false, U, PAR>;
    case 2: return (const void *)explore_local_kernel<512, false, U, PAR>;
    case 3: return (const void *)explore_global_kernel<128, U, PAR>;
    case 4: return (const void *)explore_global_kernel<256, U, PAR>;
    case 5: return (const void *)explore_global_kernel<512, U, PAR>;
    case 6: return (const void *)explore_local_kernel<128, true, U, PAR>;
    case 7: return (const void *)explore_local_kernel<256, true, U, PAR>;
    case 8: return (const void *)explore_local_kernel<512, true, U, PAR>;
    default: return nullptr;
  }
}
const void *explore_kernel_fn(int arm, int ipt, bool parents) {
  if (parents) return ipt == 8 ? explore_fn_u<8, true>(arm) : explore_fn_u<4, true>(arm);
  return ipt == 8 ? explore_fn_u<8, false>(arm) : explore_fn_u<4, false>(arm);
}
const void *explore_any_kernel_fn(int ipt, bool parents) {
  if (parents)
    return ipt == 8 ? (const void *)explore_any_kernel<8, true> : (const void *)explore_any_kernel<4, true>;
  return ipt == 8 ? (const void *)explore_any_kernel<8, false> : (const void *)explore_any_kernel<4, false>;
}
const void *levelgen_kernel_fn(bool parents) {
  return parents ? (const void *)levelgen_kernel<kLevelgenBlock, true>
                 : (const void *)levelgen_kernel<kLevelgenBlock, false>;
}
size_t levelgen_smem(bool parents) {
  return (parents ? 3u : 2u) * kLevelgenBlock * 32u * sizeof(uint32_t);
}
const void *init_kernel_fn() { return (const void *)init_kernel; }
const void *fill_kernel_fn() { return (const void *)fill_kernel; }
const void *level_out_kernel_fn() { return (const void *)level_out_kernel; }

cudaError_t launch_validate(const uint32_t *indptr, const uint32_t *inds, uint32_t n_rows,
                            uint32_t n_cols, uint32_t root, const int32_t *level,
                            const int32_t *parent, uint8_t *witness, uint8_t *parent_ok,
                            unsigned long long *bad, cudaStream_t s) {
  validate_edges_kernel<<<2048, 256, 0, s>>>(indptr, inds, n_rows, level, parent, witness,
                                             parent_ok, bad);
  validate_vertices_kernel<<<1024, 256, 0, s>>>(n_cols, root, level, parent, witness,
                                                parent_ok, bad);
  return cudaGetLastError();
}

cudaError_t launch_seed_state(BfsDevState *st, const BfsDevState &s, cudaStream_t stream) {
  seed_state_kernel<<<1, 64, 0, stream>>>(st, s);
  return cudaGetLastError();
}

cudaError_t launch_check_csc(const uint32_t *indptr, const uint32_t *inds, uint32_t n_cols,
                             uint64_t nnz, unsigned long long *bad, cudaStream_t s) {
  check_csc_kernel<<<2048, 256, 0, s>>>(indptr, inds, n_cols, nnz, bad);
  return cudaGetLastError();
}

}  // namespace bfsgb
