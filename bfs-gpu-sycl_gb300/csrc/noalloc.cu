// noalloc.cu -- single-root BFS that allocates no memory.
//
// Some callers cannot call cudaMalloc: code running inside an allocator or a
// memory-pool callback (a cudaMalloc there could re-enter it), processes that
// run under a hard device-memory budget fixed at start-up, and plugins whose
// host forbids device allocation after initialisation.  bfs_run_device_noalloc
// serves them: the caller passes the graph and the output level array (device
// memory it already owns), and the BFS workspace -- visited bitmaps, the two
// frontier queues and the level-loop state -- lives in the file-scope device
// array below.  It is sized for graphs of at most BFS_NOALLOC_MAX_VERTICES
// vertices (about 33 MiB), and every GPU that loads this library keeps it
// until the process exits.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address with cudaGetSymbolAddress (the name of the array in
// host code is a host-side stand-in, not a device address, so it is never
// passed to a kernel).  Make that first call before any stream capture.
//
// The first call is also when the array may come into existence.  Under
// CUDA's default lazy module loading (CUDA_MODULE_LOADING=LAZY) the library's
// device code and this array are loaded, and their device memory taken, when
// a device first uses them -- that is, inside the first call.  So make one
// warm-up call per device at start-up, outside any allocator callback and
// before a memory budget is fixed; every later call allocates nothing.
// Setting CUDA_MODULE_LOADING=EAGER instead loads the array when the context
// is created.  The address looked up at set-up is kept for the life of the
// process: after cudaDeviceReset, or with another context made current on
// the same device, it is stale, and such a process must not call this entry
// point again.
//
// Sharing: every call on a device uses the same array, and the array keeps the
// previous call's contents; each call clears the parts that must start at zero
// (both bitmaps and the loop counters).  Two calls that overlap on the GPU --
// from two host threads, or on two streams -- race on the array; serialise
// them.
//
// No cudaMalloc, cudaFree or other allocating routine is called: the launch
// geometry comes from an occupancy query, the state is written by a kernel
// from its by-value argument, and the per-level frontier size is read back
// with a small device-to-host copy.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "bfs_internal.h"
#include "kernels.h"

namespace bfsgb {
namespace {

constexpr uint32_t kMaxV = BFS_NOALLOC_MAX_VERTICES;
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
// layout of the scratch array
constexpr size_t kStateOff = 0;
constexpr size_t kBadOff = align256(sizeof(BfsDevState));
constexpr size_t kWordsMax = (((size_t)kMaxV + 31) / 32 + 31) / 32 * 32;
constexpr size_t kVisOff = kBadOff + 256;
constexpr size_t kPrevOff = kVisOff + align256(kWordsMax * 4);
constexpr size_t kQ4 = align256((size_t)kMaxV * 4);
constexpr size_t kQp4 = align256(((size_t)kMaxV + 1) * 4);
constexpr size_t kLv8Off = kPrevOff + align256(kWordsMax * 4);
constexpr size_t kQOff = kLv8Off + align256(kWordsMax * 32);
constexpr size_t kScratchBytes = kQOff + 2 * (3 * kQ4 + kQp4);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_dev[kMaxDevices] = {};
int g_grid[kMaxDevices][2] = {};  // explore, levelgen grid per device

constexpr int kArm = 4;  // GLB, 256 threads
constexpr int kIpt = 4;

// Writes the loop state from its by-value argument and clears the error
// counter (no host-to-device copy of a host buffer is needed).
__global__ void noalloc_state_kernel(BfsDevState s, BfsDevState *dst,
                                     unsigned long long *bad) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *dst = s;
    *bad = 0ull;
  }
}

bfs_status setup_device(int dev) {
  std::lock_guard<std::mutex> lk(g_setup_mutex);
  if (g_scratch_dev[dev]) return BFS_OK;
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(BFS_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                  cudaGetErrorString(e));
  int sms = 0, occ_ex = 0, occ_lg = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_ex, explore_kernel_fn(kArm, kIpt, false),
                                                      arm_block(kArm), 0);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(levelgen_kernel_fn(false), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)levelgen_smem(false));
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_lg, levelgen_kernel_fn(false),
                                                      kLevelgenBlock, levelgen_smem(false));
  if (e != cudaSuccess)
    return fail(BFS_ERR_CUDA, std::string("launch geometry: ") + cudaGetErrorString(e));
  g_grid[dev][0] = sms * (occ_ex > 0 ? occ_ex : 1);
  g_grid[dev][1] = sms * (occ_lg > 0 ? occ_lg : 1);
  g_scratch_dev[dev] = (unsigned char *)p;
  return BFS_OK;
}

}  // namespace
}  // namespace bfsgb

using namespace bfsgb;

#define NK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(BFS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

extern "C" bfs_status bfs_run_device_noalloc(const uint32_t *d_indptr, const uint32_t *d_inds,
                                             uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
                                             uint32_t root, int32_t *levels_dev,
                                             uint64_t *edges_count_out, void *stream) {
  if (!d_indptr || (!d_inds && nnz) || !levels_dev)
    return fail(BFS_ERR_INVALID_ARG, "null graph or level buffer");
  if (n_cols == 0 || n_rows > n_cols)
    return fail(BFS_ERR_INVALID_ARG, "need 0 < n_cols and n_rows <= n_cols");
  if (n_cols > kMaxV)
    return fail(BFS_ERR_INVALID_ARG,
                "bfs_run_device_noalloc supports at most " + std::to_string(kMaxV) +
                    " vertices (its fixed scratch size); use bfs_run_device for larger graphs");
  if (nnz > BFS_MAX_EDGES) return fail(BFS_ERR_INVALID_ARG, "nnz must be <= BFS_MAX_EDGES");
  if (root >= n_cols) return fail(BFS_ERR_ROOT, "root out of range");
  int dev = 0;
  NK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(BFS_ERR_UNSUPPORTED, "device index too large");
  bfs_status rc = setup_device(dev);
  if (rc != BFS_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char *base = g_scratch_dev[dev];

  BfsDevState h;
  std::memset(&h, 0, sizeof(h));
  h.indptr = d_indptr;
  h.inds = d_inds;
  h.nnz = (uint32_t)nnz;
  h.inds_off = (uint32_t)((reinterpret_cast<uintptr_t>(d_inds) & 15u) >> 2);
  h.n_rows = n_rows;
  h.n_cols = n_cols;
  h.words = (uint32_t)((((size_t)n_cols + 31) / 32 + 31) / 32 * 32);
  h.root = root;
  h.vis = (uint32_t *)(base + kVisOff);
  h.prev = (uint32_t *)(base + kPrevOff);
  h.lv8 = base + kLv8Off;
  for (int b = 0; b < 2; b++) {
    unsigned char *q = base + kQOff + (size_t)b * (3 * kQ4 + kQp4);
    h.qb[b] = (uint32_t *)q;
    h.qd[b] = (uint32_t *)(q + kQ4);
    h.qc[b] = (uint32_t *)(q + 2 * kQ4);
    h.qv[b] = (uint32_t *)(q + 2 * kQ4 + kQp4);
  }
  h.level = levels_dev;
  h.parent = nullptr;
  h.fixed_arm = kArm;
  h.level_cap = n_cols + 1u;
  h.rec_cap = 0;  // no per-level record in this entry point
  BfsDevState *st = (BfsDevState *)(base + kStateOff);
  unsigned long long *bad = (unsigned long long *)(base + kBadOff);

  // state + cleared counters, CSC check (fill clears the bitmaps)
  noalloc_state_kernel<<<1, 32, 0, s>>>(h, st, bad);
  NK(cudaGetLastError());
  NK(launch_check_csc(d_indptr, d_inds, n_cols, nnz, bad, s));
  unsigned long long h_bad = 0;
  NK(cudaMemcpyAsync(&h_bad, bad, sizeof(h_bad), cudaMemcpyDeviceToHost, s));
  NK(cudaStreamSynchronize(s));
  if (h_bad) return fail(BFS_ERR_GRAPH, "malformed CSC: " + std::to_string(h_bad) + " errors");

  unsigned long long no_cond = 0;
  int zero = 0;
  void *fill_args[] = {&st};
  NK(cudaLaunchKernel(fill_kernel_fn(), dim3(g_grid[dev][1]), dim3(256), fill_args, 0, s));
  void *init_args[] = {&st, &no_cond, &zero};
  NK(cudaLaunchKernel(init_kernel_fn(), dim3(1), dim3(32), init_args, 0, s));
  for (;;) {
    uint32_t F = 0;
    NK(cudaMemcpyAsync(&F, &st->F, sizeof(F), cudaMemcpyDeviceToHost, s));
    NK(cudaStreamSynchronize(s));
    if (F == 0) break;
    void *ex_args[] = {&st};
    NK(cudaLaunchKernel(explore_kernel_fn(kArm, kIpt, false), dim3(g_grid[dev][0]), dim3(arm_block(kArm)),
                        ex_args, 0, s));
    void *lg_args[] = {&st, &no_cond, &zero};
    NK(cudaLaunchKernel(levelgen_kernel_fn(false), dim3(g_grid[dev][1]), dim3(kLevelgenBlock),
                        lg_args, levelgen_smem(false), s));
  }
  NK(cudaLaunchKernel(level_out_kernel_fn(), dim3(g_grid[dev][1]), dim3(256), fill_args, 0, s));
  uint32_t err = 0;
  unsigned long long edges = 0;
  NK(cudaMemcpyAsync(&err, &st->error, sizeof(err), cudaMemcpyDeviceToHost, s));
  NK(cudaMemcpyAsync(&edges, &st->edges_count, sizeof(edges), cudaMemcpyDeviceToHost, s));
  NK(cudaStreamSynchronize(s));
  if (err & BFS_DEVERR_LEVEL_LIMIT)
    return fail(BFS_ERR_LEVEL_LIMIT, "level loop exceeded n_cols + 1 levels");
  if (err) return fail(BFS_ERR_DEVICE, "device error flag " + std::to_string(err));
  if (edges_count_out) *edges_count_out = edges;
  return BFS_OK;
}
