// bfs_gpurun.hpp -- the reference's GPURun entry point, rebuilt on the C ABI.
//
// Drop-in for `template<typename vectorT> void GPURun(...)` of
// src/run_bfs_gpu.hpp:534-542 (called from src/host.cpp:147-150): same
// argument list and meaning, same JSON timing keys (run_bfs_gpu.hpp:784-790).
// Differences a caller may notice:
//   - the graph is uploaded once for all num_runs runs (the reference uploads
//     and frees it per run, :620-747);
//   - per-run time is the device time of one BFS (CUDA events around the
//     seeded level loop) instead of a host timer around the submits;
//   - no 1000-level cap (MAX_NUM_LEVELS, :13): every level is explored;
//   - errors throw std::runtime_error with the engine's message (the
//     reference prints SYCL exceptions and calls std::terminate, :794-807).
// The explore form follows the reference's build macros
// (USE_GLOBAL_LOAD_BALANCE -> GLB, USE_STRIDED_LOCAL_LOAD_BALANCE -> SLB,
// otherwise LLB) unless bfs::gpurun_config() selects another one, e.g. the
// learned per-level schedule.  JsonT is any JSON type with
// `json["key"] = value` (the reference's library, or bfs::Json).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "bfs_gb300.h"

namespace bfs {

struct GpuRunConfig {
  int lb = -1;            // -1: from the build macros; else bfs_lb
  int block = 256;
  int ipt = 4;
  int loop = BFS_LOOP_GRAPH;
  std::string weights;    // scheduler weights file (1545 float32) for BFS_LB_LEARNED
  float min_confidence = 0.f;
  bool validate_last = true;  // Graph500-style device check of the last run
  // outputs of the last GPURun call
  uint64_t edges_count = 0;
  uint32_t num_levels = 0;
  uint64_t validation_errors = 0;
  std::vector<double> run_ms;
};

inline GpuRunConfig &gpurun_config() {
  static GpuRunConfig cfg;
  return cfg;
}

inline int default_lb() {
#if defined(USE_GLOBAL_LOAD_BALANCE) && USE_GLOBAL_LOAD_BALANCE == 1
  return BFS_LB_GLB;
#elif defined(USE_STRIDED_LOCAL_LOAD_BALANCE) && USE_STRIDED_LOCAL_LOAD_BALANCE == 1
  return BFS_LB_SLB;
#else
  return BFS_LB_LLB;
#endif
}

// Timing statistics of the reference (src/functions.hpp:64-108): runs within
// `threshold` standard deviations of the mean, and the runs after the first
// 10 % (warm-up).
inline std::vector<double> filter_sigma(const std::vector<double> &d, double threshold) {
  const double mean = std::accumulate(d.begin(), d.end(), 0.0) / (double)d.size();
  double var = 0.0;
  for (double x : d) var += (x - mean) * (x - mean);
  const double sd = std::sqrt(var / (double)d.size());
  std::vector<double> out;
  for (double x : d)
    if (std::abs(x - mean) <= threshold * sd) out.push_back(x);
  return out;
}
inline std::vector<double> drop_warmup(const std::vector<double> &d) {
  const size_t skip = (size_t)((double)d.size() * 0.1);
  return std::vector<double>(d.begin() + (long)skip, d.end());
}

inline void check_status(bfs_status s, const char *what) {
  if (s != BFS_OK)
    throw std::runtime_error(std::string(what) + ": " + bfs_status_string(s) + " (" +
                             bfs_last_error() + ")");
}

// Merges P partitions (each with offsets over all columns and global
// destination ids) into one CSC, partition order kept per vertex -- the
// same BFS as run_bfs_cpu.hpp:47-62.
inline void merge_partitions(const std::vector<std::vector<uint32_t>> &indptr,
                             const std::vector<std::vector<uint32_t>> &inds, uint32_t n_cols,
                             std::vector<uint32_t> &ip, std::vector<uint32_t> &ix) {
  ip.assign((size_t)n_cols + 1, 0);
  ix.clear();
  for (uint32_t v = 0; v < n_cols; v++) {
    for (size_t p = 0; p < indptr.size(); p++) {
      if (v + 1 >= indptr[p].size()) continue;
      ix.insert(ix.end(), inds[p].begin() + indptr[p][v], inds[p].begin() + indptr[p][v + 1]);
    }
    ip[v + 1] = (uint32_t)ix.size();
  }
}

template <typename vectorT, typename JsonT>
void GPURun(uint32_t vertexCount, vectorT &IndexHost, vectorT &OffsetHost,
            std::vector<uint8_t> &h_visit_mask, std::vector<uint8_t> &h_visit,
            std::vector<std::vector<int>> &h_distance, int sourceNode, const int num_runs,
            JsonT &newJsonObj, std::vector<uint32_t> &h_visit_offsets) noexcept(false) {
  (void)h_visit_mask;
  (void)h_visit;
  (void)h_visit_offsets;
  GpuRunConfig &cfg = gpurun_config();
  if (num_runs < 1 || h_distance.size() < (size_t)num_runs)
    throw std::runtime_error("GPURun: h_distance must hold num_runs rows");
  const uint32_t n_cols = (uint32_t)h_distance[0].size();
  for (int i = 1; i < num_runs; i++)
    if (h_distance[(size_t)i].size() != (size_t)n_cols)
      throw std::runtime_error("GPURun: h_distance rows differ in length");
  std::vector<uint32_t> ip, ix;
  const std::vector<uint32_t> *pip = nullptr, *pix = nullptr;
  if constexpr (std::is_same_v<vectorT, std::vector<uint32_t>>) {
    if (OffsetHost.size() >= (size_t)n_cols + 1) {
      pip = &OffsetHost;
    } else {  // offsets of missing columns mean "no edges"
      ip = OffsetHost;
      ip.resize((size_t)n_cols + 1, OffsetHost.empty() ? 0u : OffsetHost.back());
      pip = &ip;
    }
    pix = &IndexHost;
  } else {
    merge_partitions(OffsetHost, IndexHost, n_cols, ip, ix);
    pip = &ip;
    pix = &ix;
  }
  const uint64_t nnz = (*pip)[n_cols];
  bfs_graph *g = nullptr;
  check_status(bfs_graph_upload(pip->data(), pix->empty() ? nullptr : pix->data(), vertexCount,
                                n_cols, nnz, 1, &g),
               "bfs_graph_upload");
  try {
    bfs_options o;
    bfs_options_default(&o);
    o.lb = cfg.lb >= 0 ? cfg.lb : default_lb();
    o.block = cfg.block;
    o.ipt = cfg.ipt;
    o.loop = cfg.loop;
    if (o.lb == BFS_LB_LEARNED && !cfg.weights.empty()) {
      std::vector<float> w(BFS_SCHED_PARAMS);
      std::ifstream f(cfg.weights, std::ios::binary);
      if (!f.read(reinterpret_cast<char *>(w.data()), (std::streamsize)(w.size() * 4)))
        throw std::runtime_error("cannot read scheduler weights " + cfg.weights);
      check_status(bfs_sched_attach(g, w.data(), cfg.min_confidence), "bfs_sched_attach");
    }
    std::vector<double> run_times((size_t)num_runs, 0.0);
    // the num_runs loop of run_bfs_gpu.hpp:682-730 as one bfs_run_roots call
    const std::vector<uint32_t> roots((size_t)num_runs, (uint32_t)sourceNode);
    std::vector<int32_t *> outs((size_t)num_runs);
    for (int i = 0; i < num_runs; i++) outs[(size_t)i] = h_distance[(size_t)i].data();
    std::vector<bfs_stats> stats((size_t)num_runs);
    check_status(bfs_run_roots(g, roots.data(), (uint32_t)num_runs, &o, outs.data(), nullptr,
                               stats.data()),
                 "bfs_run_roots");
    for (int i = 0; i < num_runs; i++) run_times[(size_t)i] = stats[(size_t)i].device_ms;
    const bfs_stats &st = stats.back();
    cfg.edges_count = st.edges_count;
    cfg.num_levels = st.num_levels;
    cfg.run_ms = run_times;
    cfg.validation_errors = 0;
    if (cfg.validate_last)
      check_status(bfs_validate_host(g, (uint32_t)sourceNode, h_distance[(size_t)num_runs - 1].data(),
                                     &cfg.validation_errors),
                   "bfs_validate_host");
    bfs_graph_free(g);
    g = nullptr;
    // run_bfs_gpu.hpp:756-790
    const std::vector<double> filtered = filter_sigma(run_times, 1.5);
    const std::vector<double> nof = drop_warmup(run_times);
    const double total = std::accumulate(run_times.begin(), run_times.end(), 0.0);
    newJsonObj["rawExecutionTimeAll"] = run_times;
    newJsonObj["avgExecutionTime"] = total / (double)run_times.size();
    newJsonObj["avgExecutionTimeFiltered"] =
        std::accumulate(filtered.begin(), filtered.end(), 0.0) / (double)filtered.size();
    newJsonObj["minExecutionTimeFiltered"] = *std::min_element(filtered.begin(), filtered.end());
    newJsonObj["avgExecutionTime90f"] =
        std::accumulate(nof.begin(), nof.end(), 0.0) / (double)nof.size();
    newJsonObj["minExecutionTime90f"] = *std::min_element(nof.begin(), nof.end());
    newJsonObj["totalExecutionTime"] = total;
  } catch (...) {
    if (g) bfs_graph_free(g);
    throw;
  }
}

}  // namespace bfs
