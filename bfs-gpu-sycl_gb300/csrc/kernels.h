// kernels.h -- host-visible entry points of kernels.cu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "bfs_internal.h"

namespace bfsgb {

constexpr int kLevelgenBlock = 256;
// Block size of the explore kernel that runs any arm (learned schedule and
// every GLB launch); one block per SM.
constexpr int kAnyBlock = 1024;
// Explore kernels keep U warp rounds (U edges per lane) in flight; U is the
// "items per thread" tunable (4 or 8).  A GLB warp chunk is at least
// kGlbGroups groups of U rounds (more when the level is large: about four
// chunks per warp of the grid).
constexpr int kGlbGroups = 4;
inline uint32_t glb_chunk_edges(int ipt) { return 32u * (uint32_t)ipt * kGlbGroups; }

// Kernel function pointers (for CUDA-graph kernel nodes and direct launches).
// Every kernel takes (BfsDevState*) first; levelgen and init also take
// (unsigned long long conditional_handle, int use_conditional).
// parents: the variant that also records BFS-tree parents.
const void *explore_kernel_fn(int arm, int ipt, bool parents);
// The explore kernel that runs any arm: arguments (BfsDevState*, int arm),
// arm < 0 = the arm stored in st->arm; kAnyBlock threads, one block per SM,
// dynamic shared memory of st->hub_words words for GLB levels behind the hub
// filter (the function's maximum dynamic shared memory must be raised first).
const void *explore_any_kernel_fn(int ipt, bool parents);
// Level generation: kLevelgenBlock threads, levelgen_smem(parents) bytes of
// dynamic shared memory (above the default limit: the function's maximum
// dynamic shared memory must be raised first).
const void *levelgen_kernel_fn(bool parents);
size_t levelgen_smem(bool parents);
const void *init_kernel_fn();
// fill clears the visited bitmaps (vis, prev: st->words words each), marks
// every working level unvisited and sets parents (when recorded) to -1.
const void *fill_kernel_fn();
// Writes the output levels (st->level, every entry) from the working levels;
// runs once after the level loop.  Arguments (BfsDevState*).
const void *level_out_kernel_fn();
// Writes the state st from a host copy with one small kernel.
cudaError_t launch_seed_state(BfsDevState *st, const BfsDevState &s, cudaStream_t stream);

cudaError_t launch_validate(const uint32_t *indptr, const uint32_t *inds, uint32_t n_rows,
                            uint32_t n_cols, uint32_t root, const int32_t *level,
                            const int32_t *parent, uint8_t *witness, uint8_t *parent_ok,
                            unsigned long long *bad, cudaStream_t s);
cudaError_t launch_check_csc(const uint32_t *indptr, const uint32_t *inds, uint32_t n_cols,
                             uint64_t nnz, unsigned long long *bad, cudaStream_t s);

}  // namespace bfsgb
