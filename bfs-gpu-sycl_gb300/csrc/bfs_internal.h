// bfs_internal.h -- definitions shared by the engine's CUDA and C++ sources.
//
// Data layout in HBM for one graph handle (all arrays 256-byte aligned):
//   indptr  u32[n_cols + 1]   CSC offsets (reference format)
//   inds    u32[nnz]          destination ids
//   vis     u32[words]        visited bitmap, bit v = vertex v reached
//   prev    u32[words]        visited bitmap as of the previous level
//   qb[2]   u32[n_rows]       frontier queue: first edge (indptr[v]) of each entry
//   qd[2]   u32[n_rows]       degree of each entry
//   qc[2]   u32[n_rows + 1]   exclusive prefix of entry chunk counts (queue
//                             order): the 16-byte chunks of inds that hold an
//                             entry's edges; qc[F] holds the chunk total
//   qv[2]   u32[n_rows]       original vertex id of each entry (written only
//                             when parents are recorded)
//   state   BfsDevState       counters of the level loop (one struct)
// words = ceil(n_cols / 32) rounded up to a multiple of 32 (one warp reads
// 32 consecutive words in the level-generation kernel).
#pragma once
#include <cstdint>
#include <cstddef>
#include <string>

#include <vector_types.h>

#include "bfs_gb300.h"

#if defined(__CUDACC__)
#define BFS_HD __host__ __device__ __forceinline__
#else
#define BFS_HD inline
#endif

namespace bfsgb {

// ---- counter-based hashing -------------------------------------------------
// SplitMix64 output function (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014).  Pure function of its input,
// identical on host and device, so generated graphs do not depend on where
// or in which order they are built.
BFS_HD uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// Independent stream per (seed, counter, lane).
BFS_HD uint64_t hash3(uint64_t seed_mixed, uint64_t counter, uint32_t lane) {
  return mix64(seed_mixed + (counter << 8) + lane);
}

// R-MAT quadrant thresholds as 32-bit fixed point: a draw r (uniform u32)
// picks quadrant 0 if r < t_a, 1 if r < t_ab, 2 if r < t_abc, else 3.
struct RmatParams {
  uint32_t scale;
  uint64_t n_edges;     // generated (directed) edge count
  uint64_t seed_mixed;  // mix64(seed)
  uint32_t t_a, t_ab, t_abc;
};

// Edge i of the R-MAT stream: recursive quadrant descent, most significant
// bit first.  Quadrants: 0 -> (0,0), 1 -> (0,1), 2 -> (1,0), 3 -> (1,1).
BFS_HD void rmat_edge(const RmatParams &p, uint64_t i, uint32_t *u_out,
                      uint32_t *v_out) {
  uint32_t u = 0, v = 0;
  uint64_t h = 0;
  for (uint32_t l = 0; l < p.scale; l++) {
    if ((l & 1u) == 0) h = hash3(p.seed_mixed, i, l >> 1);
    uint32_t r = (l & 1u) ? (uint32_t)(h >> 32) : (uint32_t)h;
    uint32_t q = (r < p.t_a) ? 0u : (r < p.t_ab) ? 1u : (r < p.t_abc) ? 2u : 3u;
    u = (u << 1) | (q >> 1);
    v = (v << 1) | (q & 1u);
  }
  *u_out = u;
  *v_out = v;
}

// 16-byte chunks of the edge array (4 uint32 entries each) that hold the
// edges [b, b + deg) of one vertex, for an array starting off uint32 past a
// 16-byte boundary: chunks (b + off)/4 .. (b + off + deg - 1)/4.
BFS_HD uint32_t edge_chunks(uint32_t b, uint32_t deg, uint32_t off) {
  return deg ? ((b + off + deg + 3u) >> 2) - ((b + off) >> 2) : 0u;
}

// Maps a 64-bit hash to [0, n).
BFS_HD uint32_t hash_to_range(uint64_t h, uint32_t n) {
  return (uint32_t)(((h >> 32) * (uint64_t)n) >> 32);
}

// ---- device state of the level loop ---------------------------------------
constexpr uint8_t kLv8Unvisited = 0xFF;
constexpr uint8_t kLv8Deep = 0xFE;

struct BfsDevState {
  // graph
  const uint32_t *indptr;
  const uint32_t *inds;
  uint32_t nnz;          // entries of inds (< 2^32)
  uint32_t inds_off;     // inds' offset in uint32 from the 16-byte boundary
                         // below it (0..3): edge p lies in 16-byte chunk
                         // (p + inds_off) / 4 counted from that boundary
  uint32_t n_rows, n_cols;
  uint32_t words;        // bitmap words (padded)
  uint32_t root;
  // workspace
  uint32_t *vis;
  uint32_t *prev;
  uint32_t *qb[2];
  uint32_t *qd[2];
  uint32_t *qc[2];
  uint32_t *qv[2];
  int32_t *level;        // output, original ids; written at the end of the BFS
                         // (level_out_kernel), during it only for deep levels
  int32_t *parent;       // may be null
  // working levels, one byte per internal id (words * 32 bytes): kLv8Unvisited,
  // kLv8Deep (the level is >= kLv8Deep and already in `level`), else the
  // level.  Small enough to stay in L2, and written a whole 32-byte sector
  // (one bitmap word) at a time, where 4-byte stores into the output array
  // would each make L2 fetch the rest of their sector from DRAM.
  uint8_t *lv8;
  // hub layout (hub_layout.cu): with a relabelled graph, indptr/inds above are
  // the relabelled CSC and the kernels work on internal ids; levels and
  // parents are written in original ids.  Null: identity.
  const uint32_t *perm;  // internal id -> original id
  const uint32_t *pinv;  // original id -> internal id
  const uint32_t *moved; // bitmap: bit v set when perm[v] != v (null: identity)
  uint32_t hub_words;    // bitmap words of the hub prefix kept in shared memory
  uint32_t hub_min_edges;  // frontier edges from which explore loads them
  // level-loop counters (written by kernels)
  unsigned long long next_packed;  // (count << 32) | chunk sum, next frontier
  unsigned long long edges_count;  // sum of degrees of expanded vertices
  uint32_t next_edges;   // degree sum of the next frontier
  uint32_t cur;          // queue buffer holding the current frontier
  uint32_t F;            // current frontier entries
  uint32_t EF;           // current frontier edges
  uint32_t EC;           // current frontier 16-byte chunks of inds
  uint32_t lvl;          // level of the current frontier
  uint32_t reached;      // vertices with a level
  uint32_t reached_prev; // `reached` before the current level generation
  uint32_t max_level;    // deepest level that received a vertex
  uint32_t done_blocks;  // level-generation blocks finished this level
  uint32_t lg_cursor;    // next bitmap word to claim in level generation
  uint32_t error;        // non-zero: internal error flag
  uint32_t launches;     // kernels launched in the device loop
  int32_t arm;           // explore arm chosen for the current level
  int32_t fixed_arm;     // arm used when no scheduler runs (-1 = scheduler)
  uint32_t level_cap;    // levels allowed before BFS_ERR_LEVEL_LIMIT
  // learned scheduler run inside init and the last block of level
  // generation (CUDA-graph loop): it stores the next level's explore arm in
  // `arm`, which explore_any then runs
  const float *sched_w;      // model weights; null: the scheduler is not fused
  float sched_min_conf;      // below this top probability: the fallback arm
  float sched_diam;          // graph-level feature constants
  float sched_avg_deg_x;
  // per-level record (first BFS_MAX_RECORDED_LEVELS levels)
  uint32_t *rec_frontier;
  uint32_t *rec_edges;
  int32_t *rec_arm;          // arm chosen by a scheduler on the device, -1 if none
  int32_t *rec_ran;          // arm of the explore kernel that ran
  uint32_t rec_cap;
};

enum : uint32_t {
  BFS_DEVERR_LEVEL_LIMIT = 1u,
  BFS_DEVERR_QUEUE_OVERFLOW = 2u,
};

// Arms: lb * 3 + block index (0: 128, 1: 256, 2: 512).
constexpr int kNumArms = 9;
BFS_HD int arm_of(int lb, int block) {
  return lb * 3 + (block == 128 ? 0 : block == 512 ? 2 : 1);
}
BFS_HD int arm_lb(int arm) { return arm / 3; }
BFS_HD int arm_block(int arm) { return 128 << (arm % 3); }

// ---- error plumbing --------------------------------------------------------
void set_error(const std::string &msg);
bfs_status fail(bfs_status s, const std::string &msg);

}  // namespace bfsgb
