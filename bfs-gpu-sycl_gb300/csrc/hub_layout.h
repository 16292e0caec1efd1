// hub_layout.h -- the degree-ordered hub layout of a graph handle
// (hub_layout.cu).
#pragma once
#include <cstddef>
#include <cstdint>

#include "bfs_internal.h"

struct bfs_graph;

namespace bfsgb {

// Arrays the single-root level loop runs on when a layout exists.  With
// relabelled == false they are the graph's own CSC (not owned) and perm /
// pinv are null (identity).
struct HubLayout {
  uint32_t *indptr = nullptr;  // u32[n_cols + 1], relabelled CSC offsets
  uint32_t *inds = nullptr;    // u32[nnz], relabelled destinations
  uint32_t *perm = nullptr;    // internal id -> original id
  uint32_t *pinv = nullptr;    // original id -> internal id
  uint32_t *moved = nullptr;   // u32[words]: bit v set when perm[v] != v
  uint32_t vertices = 0;       // K: internal ids 0 .. K-1 are the hub prefix
  bool relabelled = false;
};

// Largest hub prefix (vertices) whose bitmap fits the explore kernel's
// dynamic shared memory on the handle's device, beside static_bytes of its
// own arrays.
uint32_t hub_max_vertices(const bfs_graph *g, size_t static_bytes);
// Builds the layout for a prefix of K vertices (K a multiple of 128; 0 frees
// it).  Out of device memory leaves the handle without a layout and returns
// BFS_OK: the kernels then run on the original CSC.
bfs_status build_hub(bfs_graph *g, uint32_t K);
void free_hub(bfs_graph *g);

}  // namespace bfsgb
