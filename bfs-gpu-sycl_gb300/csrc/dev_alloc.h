// dev_alloc.h -- the engine's device allocations.
//
// Every device buffer of the engine is allocated through dev_malloc.  With
// the environment variable BFS_GB300_FAIL_ALLOC_BYTES=N set (a test hook,
// read on every call), each request of N bytes or more fails the way an
// exhausted device does (cudaErrorMemoryAllocation, reported as
// BFS_ERR_OOM), so tests reach the out-of-memory paths without filling the
// GPU.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdlib>

namespace bfsgb {

template <class T>
inline cudaError_t dev_malloc(T **p, size_t bytes) {
  if (const char *e = std::getenv("BFS_GB300_FAIL_ALLOC_BYTES")) {
    const unsigned long long limit = std::strtoull(e, nullptr, 10);
    if (limit != 0 && bytes >= limit) {
      *p = nullptr;
      return cudaErrorMemoryAllocation;
    }
  }
  return cudaMalloc(reinterpret_cast<void **>(p), bytes);
}

}  // namespace bfsgb
