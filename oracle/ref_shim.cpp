// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's own CPU BFS, `run_bfs_cpu` from
// src/run_bfs_cpu.hpp:5-85, unmodified and in place (the include path points
// at the reference tree; nothing is copied), behind a small C entry point so
// the oracle restatement in bfs_oracle.c can be checked against it.
//
// The header expects a few names from the reference's translation unit
// (src/host.cpp:1-21 and src/functions.hpp:165-169): NUM_GPU, VERBOSE, a
// DeviceInfo type and nlohmann::json.  Only `json["edgesCount"] = count` is
// used with VERBOSE == 0 (run_bfs_cpu.hpp:84), so a one-slot stand-in for the
// json type is enough and the vendored json library is not needed.
//
// Built once per partition count P by oracle/Makefile with -DNUM_GPU=P,
// exporting ref_bfs_p<P>.
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#ifndef NUM_GPU
#error "NUM_GPU must be defined"
#endif
#define VERBOSE 0

struct DeviceInfo {
  int gpuID;
  long long edgesProcessed;
  double percentage;
};

namespace nlohmann {
struct json {
  uint64_t edges_count = 0;
  uint64_t &operator[](const char *) { return edges_count; }
};
}  // namespace nlohmann

#include "run_bfs_cpu.hpp"

#define REF_CAT2(a, b) a##b
#define REF_CAT(a, b) REF_CAT2(a, b)
#define REF_FN REF_CAT(ref_bfs_p, NUM_GPU)

// Runs the reference BFS on n_parts == NUM_GPU partitions.  indptr[p] holds
// n_cols + 1 offsets; inds[p] holds nnz[p] global destination ids.
// level_out receives n_cols int32 levels (-1 unreached).
extern "C" int REF_FN(uint32_t n_rows, uint32_t n_cols,
                      const uint32_t *const *indptr,
                      const uint32_t *const *inds, const uint64_t *nnz,
                      uint32_t root, int32_t *level_out,
                      uint64_t *edges_count_out) {
  if (root >= n_cols || n_rows > n_cols) return 1;
  // host.cpp:161-169 initialisation
  std::vector<uint8_t> mask(n_cols, 0), upd(n_cols, 0), vis(n_cols, 0);
  std::vector<int> level(n_cols, -1);
  mask[root] = 1;
  vis[root] = 1;
  level[root] = 0;
  std::vector<uint32_t> offsets(NUM_GPU + 1, 0);
  offsets[NUM_GPU] = n_rows;
  std::vector<DeviceInfo> stats;
  nlohmann::json out;
#if NUM_GPU == 1
  std::vector<uint32_t> ip(indptr[0], indptr[0] + (size_t)n_cols + 1);
  std::vector<uint32_t> ix(inds[0], inds[0] + nnz[0]);
  run_bfs_cpu(n_rows, ip, ix, mask, upd, vis, level, out, offsets, stats);
#else
  std::vector<std::vector<uint32_t>> ip(NUM_GPU), ix(NUM_GPU);
  for (int p = 0; p < NUM_GPU; p++) {
    ip[p].assign(indptr[p], indptr[p] + (size_t)n_cols + 1);
    ix[p].assign(inds[p], inds[p] + nnz[p]);
  }
  run_bfs_cpu(n_rows, ip, ix, mask, upd, vis, level, out, offsets, stats);
#endif
  std::memcpy(level_out, level.data(), sizeof(int32_t) * (size_t)n_cols);
  if (edges_count_out) *edges_count_out = out.edges_count;
  return 0;
}
