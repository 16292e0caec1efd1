// kernels.h -- host-visible entry points of kernels.cu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "bfs_internal.h"

namespace bfsgb {

constexpr int kLevelgenBlock = 256;
constexpr int kUnroll = 4;                          // warp rounds in flight per warp
constexpr uint32_t kGlbChunkEdges = 32u * kUnroll * 2u;  // GLB edges per warp chunk

// Kernel function pointers (for CUDA-graph kernel nodes and direct launches).
// Every kernel takes (BfsDevState*) first; levelgen and init also take
// (unsigned long long conditional_handle, int use_conditional).
const void *explore_kernel_fn(int arm);
const void *levelgen_kernel_fn();
const void *init_kernel_fn();
const void *fill_kernel_fn();

cudaError_t launch_validate(const uint32_t *indptr, const uint32_t *inds, uint32_t n_rows,
                            uint32_t n_cols, uint32_t root, const int32_t *level,
                            const int32_t *parent, uint8_t *witness, uint8_t *parent_ok,
                            unsigned long long *bad, cudaStream_t s);
cudaError_t launch_check_csc(const uint32_t *indptr, const uint32_t *inds, uint32_t n_cols,
                             uint64_t nnz, unsigned long long *bad, cudaStream_t s);

}  // namespace bfsgb
