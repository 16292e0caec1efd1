/*
 * bfs_gb300.h -- C ABI of the GB300 (sm_103a) breadth-first-search engine.
 *
 * This is the drop-in boundary for the reference's single-partition GPU path.
 * The reference has no FFI: its boundary is the header-only C++ template
 *   GPURun(vertexCount, IndexHost, OffsetHost, h_visit_mask, h_visit,
 *          h_distance, sourceNode, num_runs, json, h_visit_offsets)
 * (src/run_bfs_gpu.hpp:534-542), called from src/host.cpp:149.  The entry
 * points below split that template into "upload the graph once" and "run one
 * BFS", with plain pointers and sizes, integer status codes and caller-owned
 * output buffers.  include/bfs_gpurun.hpp rebuilds the GPURun template on top
 * of them.
 *
 * Conventions
 *   - Graphs use the reference's single-partition CSC layout
 *     (src/graph_load.hpp:7-20, scripts/generator.py:115-185): `indptr` has
 *     n_cols + 1 uint32 offsets, `inds` has nnz uint32 destination ids.  The
 *     out-neighbours of vertex v are inds[indptr[v] .. indptr[v+1]).
 *   - Only vertices v < n_rows are expanded (n_rows <= n_cols), exactly as the
 *     reference's run_bfs_cpu loops tid < numRows (src/run_bfs_cpu.hpp:31).
 *   - Level arrays are int32[n_cols]: 0 at the root, -1 for unreached
 *     vertices, otherwise the hop distance (src/host.cpp:113-115).
 *   - No function throws; every one returns a bfs_status.  bfs_last_error()
 *     gives a message for the most recent failure on the calling thread.
 *   - Each graph handle owns its CUDA streams (one for the BFS kernels, one
 *     for bfs_run_roots' copies to the host); calls on one handle must not
 *     overlap from several host threads.
 */
#ifndef BFS_GB300_H
#define BFS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BFS_GB300_ABI_VERSION 1

typedef enum bfs_status {
  BFS_OK = 0,
  BFS_ERR_INVALID_ARG = 1,   /* null pointer, bad size or option */
  BFS_ERR_ROOT = 2,          /* root >= n_cols */
  BFS_ERR_GRAPH = 3,         /* malformed CSC: indptr not monotone, inds >= n_cols */
  BFS_ERR_CUDA = 4,          /* a CUDA runtime call failed */
  BFS_ERR_OOM = 5,           /* device or host allocation failed */
  BFS_ERR_IO = 6,            /* dataset file missing, empty or truncated */
  BFS_ERR_LEVEL_LIMIT = 7,   /* device level loop exceeded n_cols + 1 levels */
  BFS_ERR_NO_DEVICE = 8,     /* no CUDA device visible */
  BFS_ERR_UNSUPPORTED = 9,   /* option not supported for this graph */
  BFS_ERR_DEVICE = 10        /* a kernel reported an internal error flag */
} bfs_status;

/* Load-balancing form of the explore step (the reference picks one at compile
 * time with USE_GLOBAL_LOAD_BALANCE / USE_STRIDED_LOCAL_LOAD_BALANCE,
 * src/CMakeLists.txt:10-11). */
typedef enum bfs_lb {
  BFS_LB_LLB = 0,      /* local: block-level scan over a tile of the frontier */
  BFS_LB_GLB = 1,      /* global: grid-wide scan, edges dealt evenly to blocks */
  BFS_LB_SLB = 2,      /* strided local: frontier dealt round-robin to blocks */
  BFS_LB_LEARNED = 3   /* per-level choice by the learned scheduler */
} bfs_lb;

/* How the level loop is driven. */
typedef enum bfs_loop {
  BFS_LOOP_GRAPH = 0,  /* CUDA graph with a device-side while loop (default) */
  BFS_LOOP_HOST = 1    /* host loop, one frontier-size read-back per level,
                          like src/run_bfs_gpu.hpp:682-727 */
} bfs_loop;

typedef struct bfs_options {
  int32_t lb;          /* bfs_lb */
  int32_t block;       /* threads per block: 128, 256 or 512 (0 = 256) */
  int32_t sm_factor;   /* blocks per SM for the persistent grid (0 = auto) */
  int32_t loop;        /* bfs_loop */
  int32_t l2_pin;      /* 1 = pin the visited bitmaps in L2 (default on) */
  int32_t record;      /* 1 = fill bfs_stats per-level arrays; 2 = also time
                          every kernel with CUDA events (forces the host loop) */
  int32_t ipt;         /* edges per lane in flight in the explore kernels:
                          4 or 8 (0 = 4) */
} bfs_options;

#define BFS_MAX_RECORDED_LEVELS 4096
/* Largest edge count a device graph may have: the kernels walk edge offsets
 * in uint32 with whole 128-edge steps, which must not wrap. */
#define BFS_MAX_EDGES 0xFFFFF000u

typedef struct bfs_stats {
  uint64_t edges_count;   /* sum of out-degrees of expanded vertices; the
                             reference's json["edgesCount"] (run_bfs_cpu.hpp:36,84) */
  uint32_t num_levels;    /* levels with a non-empty frontier (max level + 1) */
  uint32_t reached;       /* vertices with level >= 0 */
  double device_ms;       /* seeded-root to last-level time, CUDA events */
  uint32_t launches;      /* kernels this engine launched for the run */
  uint32_t recorded;      /* entries filled in the arrays below */
  uint32_t level_frontier[BFS_MAX_RECORDED_LEVELS];  /* vertices expanded */
  uint32_t level_edges[BFS_MAX_RECORDED_LEVELS];     /* edges explored */
  int32_t level_arm[BFS_MAX_RECORDED_LEVELS];        /* lb*3 + block index */
  float level_explore_ms[BFS_MAX_RECORDED_LEVELS];   /* record == 2 only */
  float level_gen_ms[BFS_MAX_RECORDED_LEVELS];       /* record == 2 only */
} bfs_stats;

typedef struct bfs_graph bfs_graph;

/* ---- library ---------------------------------------------------------- */
int bfs_abi_version(void);
const char *bfs_status_string(bfs_status s);
const char *bfs_last_error(void);
/* Fills o with the defaults (LLB, 256 threads, graph loop, L2 pin on). */
void bfs_options_default(bfs_options *o);

/* ---- graph lifetime --------------------------------------------------- */
/* Copies a host CSC graph to the current CUDA device once (the reference
 * re-uploads it for every run, src/run_bfs_gpu.hpp:620-670).  validate = 1
 * checks monotone indptr and inds < n_cols on the device first. */
bfs_status bfs_graph_upload(const uint32_t *indptr, const uint32_t *inds,
                            uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
                            int validate, bfs_graph **out);
/* Wraps a CSC graph already in device memory (not copied, not freed by
 * bfs_graph_free; must outlive the handle). */
bfs_status bfs_graph_wrap_device(const uint32_t *d_indptr, const uint32_t *d_inds,
                                 uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
                                 int validate, bfs_graph **out);
bfs_status bfs_graph_free(bfs_graph *g);
bfs_status bfs_graph_info(const bfs_graph *g, uint32_t *n_rows, uint32_t *n_cols,
                          uint64_t *nnz);
/* Device pointers of the graph's CSC arrays (for callers that gather their
 * own statistics on the device). */
bfs_status bfs_graph_device_csc(const bfs_graph *g, const uint32_t **d_indptr,
                                const uint32_t **d_inds);

/* ---- hub layout of the single-root path -------------------------------- */
/* No counterpart in the reference.  On power-law graphs most edges of the
 * large levels point at a few high in-degree vertices reached levels
 * earlier; the GLB explore kernel answers those visited-bitmap probes from
 * shared memory.  For that the handle keeps a relabelled copy of the graph
 * whose internal ids 0 .. K-1 are its K highest in-degree vertices (graphs
 * of at most K vertices, and graphs with n_rows < n_cols, keep their own ids
 * and no copy).  The layout serves runs whose plan runs GLB levels (fixed
 * GLB arms and the learned schedule); fixed LLB and SLB runs keep the
 * original numbering, since their tile-local balancing suffers when the hubs
 * are consecutive ids.  Levels, parents and every other entry point still
 * use the caller's ids; results are identical with or without the layout.  The copy
 * costs nnz + 3 n_cols + 1 uint32 of device memory; if it cannot be
 * allocated the handle runs without it.
 * vertices: -1 = automatic (the default: K = 2^18, capped by the device's
 * shared memory), 0 = off, > 0 = K (rounded down to a multiple of 128).
 * min_edges: the smallest level (frontier edges) for which the explore
 * kernel loads the prefix into shared memory; 0 = automatic (max(2^21, 2K)).
 * The layout is built by this call, or by the first single-root run. */
bfs_status bfs_hub_configure(bfs_graph *g, int64_t vertices, uint32_t min_edges);
/* The current layout: *vertices = K (0: none), *relabelled = 1 if the
 * handle holds a relabelled copy, *max_vertices = the largest K the device
 * allows.  Any output may be NULL. */
bfs_status bfs_hub_info(bfs_graph *g, uint32_t *vertices, int32_t *relabelled,
                        uint32_t *max_vertices);

/* ---- single-root BFS -------------------------------------------------- */
/* One BFS from root.  levels_host (n_cols int32, required) and parents_host
 * (n_cols int32, optional: parent of each reached vertex, the root is its own
 * parent, -1 if unreached) are host buffers; the device-to-host copy is part
 * of the call.  stats may be NULL.  opts may be NULL (defaults). */
bfs_status bfs_run(bfs_graph *g, uint32_t root, const bfs_options *opts,
                   int32_t *levels_host, int32_t *parents_host, bfs_stats *stats);
/* n_roots BFS runs in one call, one per entry of roots, into host buffers:
 * run i writes its level array to levels_host[i] and, if parents_host is not
 * NULL, its parent array to parents_host[i] (n_cols int32 each).  This is the
 * reference's per-run loop (run_bfs_gpu.hpp:682-730, h_distance[i] per run).
 * The device-to-host copy of run i overlaps run i + 1 when the buffers are
 * pinned host memory; with pageable buffers the runs are serial.  stats, if
 * not NULL, receives n_roots entries.  Every root is checked before the
 * first run; on an error no copy is left in flight. */
bfs_status bfs_run_roots(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                         const bfs_options *opts, int32_t *const *levels_host,
                         int32_t *const *parents_host, bfs_stats *stats);
/* Same, with device output buffers (levels_dev required, parents_dev
 * optional); nothing is copied to the host except the small stats. */
bfs_status bfs_run_device(bfs_graph *g, uint32_t root, const bfs_options *opts,
                          int32_t *levels_dev, int32_t *parents_dev,
                          bfs_stats *stats);
/* Graph-validation helper (Graph500-style): checks on the device that
 * levels_dev is the exact BFS level array of root (root at 0, every edge
 * u->v from an expanded vertex has level[v] <= level[u] + 1, every reached
 * non-root vertex has an in-edge from level - 1) and, if parents_dev is not
 * NULL, that every parent is a level-1 in-neighbour.  *bad receives the
 * number of violations (0 = valid). */
bfs_status bfs_validate_device(bfs_graph *g, uint32_t root, const int32_t *levels_dev,
                               const int32_t *parents_dev, uint64_t *bad);
/* Same checks for a host level array (copied to the device first). */
bfs_status bfs_validate_host(bfs_graph *g, uint32_t root, const int32_t *levels_host,
                             uint64_t *bad);

/* ---- batched multi-source BFS ------------------------------------------ */
/* n_roots independent BFS runs on one graph, 64 roots per pass: each vertex
 * carries a 64-bit visited mask and one traversal of an edge serves every
 * root whose frontier holds its source.  Row i of levels_dev (n_roots x
 * n_cols int32, device) is exactly the level array of roots[i];
 * edges_count_out[i] (optional, host) its edgesCount.  The reference has one
 * root per invocation (src/host.cpp:72). */
typedef struct bfs_batch_stats {
  double device_ms;       /* CUDA-event time of all passes */
  uint32_t batches;       /* passes of up to 64 roots */
  uint32_t max_levels;    /* deepest level + 1 over all roots */
  uint32_t launches;      /* kernels launched */
} bfs_batch_stats;
bfs_status bfs_run_batch(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                         int32_t *levels_dev, uint64_t *edges_count_out,
                         bfs_batch_stats *stats);
/* bfs_run_batch for host callers: the level rows of each pass of 64 roots go
 * to a device buffer held by the graph handle and are copied to levels_host
 * (n_roots x n_cols int32, optional: NULL keeps only the edge counts and
 * stats); stats->device_ms covers the passes, not the copies. */
bfs_status bfs_run_batch_host(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                              int32_t *levels_host, uint64_t *edges_count_out,
                              bfs_batch_stats *stats);
/* bfs_run_batch with the level loop chosen by loop (bfs_loop): BFS_LOOP_HOST
 * launches every kernel separately (for profilers), BFS_LOOP_GRAPH is
 * bfs_run_batch.  Same results either way. */
bfs_status bfs_run_batch_loop(bfs_graph *g, const uint32_t *roots, uint32_t n_roots,
                              int32_t *levels_dev, uint64_t *edges_count_out, int32_t loop,
                              bfs_batch_stats *stats);

/* ---- many small graphs in one launch ----------------------------------- */
/* A batch of independent graphs (up to 2^18 vertices each) packed into one
 * CSC in HBM; bfs_multi_run runs one BFS per graph from roots[g] in a single
 * persistent kernel captured in a CUDA graph: each block claims whole graphs,
 * largest first, and runs their level loop on its own with the visited bitmap
 * in shared memory.  The reference needs one process run per graph and root
 * (src/host.cpp:57-276). */
typedef struct bfs_multi bfs_multi;
bfs_status bfs_multi_create(uint32_t n_graphs, const uint32_t *const *indptrs,
                            const uint32_t *const *inds, const uint32_t *n_rows,
                            const uint32_t *n_cols, const uint64_t *nnz, bfs_multi **out);
bfs_status bfs_multi_free(bfs_multi *m);
/* Offset of graph g's level array inside the packed output (sum of the
 * n_cols of the graphs before it). */
bfs_status bfs_multi_level_offset(const bfs_multi *m, uint32_t graph, uint64_t *offset);
/* levels_dev: sum of n_cols int32 (device).  block 128/256/512, ipt 1/2/4
 * (warp rounds in flight per lane).  edges_count_out: n_graphs (host,
 * optional); device_ms: CUDA-event time of the launch (optional). */
bfs_status bfs_multi_run(bfs_multi *m, const uint32_t *roots, int32_t block, int32_t ipt,
                         int32_t *levels_dev, uint64_t *edges_count_out, double *device_ms);
/* Times every (block, ipt) combination on this batch (best of reps) and
 * returns the fastest.  With cache_path, a previous result for the same GPU
 * and batch shape is reused and a new one is appended.  times_ms (optional)
 * receives the 9 timings, block-major (-1 when taken from the cache). */
bfs_status bfs_multi_autotune(bfs_multi *m, const uint32_t *roots, int32_t *levels_dev,
                              int32_t reps, const char *cache_path, int32_t *best_block,
                              int32_t *best_ipt, float *times_ms);
/* bfs_multi_run with cluster > 1: the batch's largest graphs (edge count at
 * least `cluster` blocks' fair share of the batch) are each run by a cluster
 * of `cluster` thread blocks (tiles of the frontier dealt over the cluster,
 * claims on a per-cluster bitmap in L2, the cluster barrier as the level
 * barrier); the other graphs run one per block as above.  Configurations:
 * cluster 1 with block 128/256/512 and ipt 1/2/4; cluster 2/4/8 with block
 * 256/512 and ipt 2/4.  No counterpart in the reference. */
bfs_status bfs_multi_run_ex(bfs_multi *m, const uint32_t *roots, int32_t block, int32_t ipt,
                            int32_t cluster, int32_t *levels_dev, uint64_t *edges_count_out,
                            double *device_ms);
/* bfs_multi_autotune over every configuration, clusters included; times_ms
 * (optional) receives bfs_multi_num_configs() timings in that order. */
bfs_status bfs_multi_autotune_ex(bfs_multi *m, const uint32_t *roots, int32_t *levels_dev,
                                 int32_t reps, const char *cache_path, int32_t *best_block,
                                 int32_t *best_ipt, int32_t *best_cluster, float *times_ms);
/* The configurations of bfs_multi_autotune_ex (up to max of them into the
 * optional arrays); returns their number. */
int32_t bfs_multi_num_configs(int32_t *blocks, int32_t *ipts, int32_t *clusters, int32_t max);

/* ---- BFS without device allocation ------------------------------------ */
/* No counterpart in the reference (its GPURun allocates per run).  For
 * callers that cannot allocate device memory -- code inside an allocator or
 * memory-pool callback, processes under a device-memory budget fixed at
 * start-up, plugins whose host forbids allocation after initialisation.
 * One BFS from root over a CSC graph already on the current device, into
 * levels_dev (n_cols int32, caller-owned); *edges_count_out (optional, host)
 * receives the reference's edgesCount.  The workspace is a fixed device array
 * inside the library (about 33 MiB per GPU that loads it, held until exit),
 * so graphs are limited to BFS_NOALLOC_MAX_VERTICES vertices and larger ones
 * are rejected with BFS_ERR_INVALID_ARG.  The first call on a device looks
 * up that array's address (make it before any stream capture), and under
 * CUDA's default lazy module loading it is also the call that loads the
 * library's device code and the array, taking their device memory: make one
 * warm-up call per device at start-up, outside any allocator callback and
 * before a memory budget is fixed (or set CUDA_MODULE_LOADING=EAGER).  Later
 * calls allocate nothing.  The address is kept for the life of the process,
 * so a process that resets the device (cudaDeviceReset) or makes another
 * context current on it must not call this entry point again.  All calls on
 * a device share the array: calls that overlap on the GPU race, so serialise
 * them.  stream may be NULL (default stream); the call returns when the BFS
 * has finished. */
#define BFS_NOALLOC_MAX_VERTICES (1u << 20)
bfs_status bfs_run_device_noalloc(const uint32_t *d_indptr, const uint32_t *d_inds,
                                  uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
                                  uint32_t root, int32_t *levels_dev,
                                  uint64_t *edges_count_out, void *stream);

/* ---- learned per-level scheduler -------------------------------------- */
/* The reference fixes the load-balancing form and work-group size at compile
 * time (src/CMakeLists.txt:10-11; run_bfs_gpu.hpp:195, 403, 493).  Here a
 * small FP32 MLP picks the explore arm (lb * 3 + block index, 9 arms) for
 * every level from 5 features of the level:
 *   x0 = log2(1 + frontier vertices) / 32
 *   x1 = log2(1 + frontier edges) / 32
 *   x2 = unvisited fraction (1 - reached / n_cols)
 *   x3 = min(level / diameter estimate, 8) / 8, with the estimate
 *        max(2, ln(n_cols) / ln(max(average degree, 2)))
 *   x4 = log2(1 + average degree nnz / n_cols) / 8
 * Layers 5 -> 32 (ReLU) -> 32 (ReLU) -> 9, softmax; weights are 1545 floats
 * laid out W1[32][5], b1[32], W2[32][32], b2[32], W3[9][32], b3[9].
 * Inference runs on the device inside the level loop; the choice never
 * changes the levels, only the time. */
#define BFS_SCHED_INPUTS 5
#define BFS_SCHED_ARMS 9
#define BFS_SCHED_PARAMS 1545

typedef struct bfs_level_sample {
  float features[BFS_SCHED_INPUTS];
  float arm_ms[BFS_SCHED_ARMS];   /* explore time of every arm on this level */
  uint32_t level, frontier, edges;
} bfs_level_sample;

typedef struct bfs_sched_train_opts {
  uint32_t epochs;      /* full-batch Adam steps (0 = 1500) */
  float lr;             /* Adam step size (0 = 3e-3) */
  uint64_t seed;        /* weight initialisation seed */
} bfs_sched_train_opts;

/* Runs one BFS from root in the host loop and, on every level, times the
 * explore step of all 9 arms (state restored between arms, best of `reps`
 * repetitions) before advancing.  Fills out[0 .. *n_out). */
bfs_status bfs_sched_record(bfs_graph *g, uint32_t root, int32_t ipt, int32_t reps,
                            bfs_level_sample *out, uint32_t max_levels, uint32_t *n_out);
/* Trains the MLP on the current CUDA device (hand-written forward/backward
 * and Adam kernels).  The loss is the expected excess explore time
 * sum_a softmax(z)_a * (t_a - t_best), in units of the mean best time, so
 * the fit minimises per-level regret.  weights_out receives 1545 floats. */
bfs_status bfs_sched_train(const bfs_level_sample *samples, uint32_t n,
                           const bfs_sched_train_opts *opts, float *weights_out,
                           float *final_loss);
/* Device inference on n feature vectors (n x 5): arms_out[i] = argmax arm,
 * conf_out[i] = its softmax probability (either output may be NULL). */
bfs_status bfs_sched_predict(const float *weights, const float *features, uint32_t n,
                             int32_t *arms_out, float *conf_out);
/* Attaches a model to a graph handle for bfs_options.lb = BFS_LB_LEARNED.
 * Levels whose top probability is below min_confidence fall back to the
 * fixed LLB/256 arm; with no model attached every level uses LLB/256.
 * weights == NULL detaches. */
bfs_status bfs_sched_attach(bfs_graph *g, const float *weights, float min_confidence);

/* ---- synthetic graphs and roots --------------------------------------- */
/* Seeded generators.  Every edge is a pure function of (seed, index) through
 * a counter-based hash, so the host and device builders produce identical
 * graphs.  Self-loops and duplicates are removed; symmetrize = 1 adds the
 * reverse of every edge.  Output CSC has n_rows == n_cols. */
typedef struct bfs_csc_host {
  uint32_t n_rows, n_cols;
  uint64_t nnz;
  uint32_t *indptr;   /* n_cols + 1, malloc'ed by the library */
  uint32_t *inds;     /* nnz, malloc'ed by the library */
} bfs_csc_host;
void bfs_csc_host_free(bfs_csc_host *g);

/* R-MAT (a, b, c; d = 1 - a - b - c) with 2^scale vertices and
 * edge_factor * 2^scale generated edges. */
bfs_status bfs_gen_rmat_host(uint32_t scale, uint32_t edge_factor, double a,
                             double b, double c, uint64_t seed, int symmetrize,
                             bfs_csc_host *out);
/* Same graph built on the current device and kept there as an engine handle
 * (no host copy); used for graphs too large to build quickly on the host. */
bfs_status bfs_gen_rmat_device(uint32_t scale, uint32_t edge_factor, double a,
                               double b, double c, uint64_t seed, int symmetrize,
                               bfs_graph **out);
/* width x height 4-neighbour grid; each undirected edge is deleted with
 * probability delete_prob. */
bfs_status bfs_gen_grid_host(uint32_t width, uint32_t height, double delete_prob,
                             uint64_t seed, bfs_csc_host *out);
/* Erdos-Renyi style graph: n vertices, n * avg_degree / 2 uniform random
 * undirected pairs before de-duplication. */
bfs_status bfs_gen_er_host(uint32_t n, double avg_degree, uint64_t seed,
                           bfs_csc_host *out);
/* Copies a device-built graph back to the host (for oracle checks). */
bfs_status bfs_graph_download(const bfs_graph *g, bfs_csc_host *out);
/* Draws count distinct roots with out-degree > 0 among vertices < n_rows,
 * seeded.  Fails with BFS_ERR_GRAPH if fewer than count such vertices exist. */
bfs_status bfs_sample_roots(const uint32_t *indptr, uint32_t n_rows, uint32_t count,
                            uint64_t seed, uint32_t *roots_out);

/* ---- reference dataset files ------------------------------------------ */
/* Reads <dir>/<name>-csc-<P>/<name>-csc-meta.bin plus the partition files,
 * the layout of src/graph_load.hpp:93-132 (P > 1 partitions are merged into
 * one CSC in partition order, which gives the same BFS levels and edge
 * counts as the reference's multi-partition CPU BFS).  dir == NULL means
 * "$PWD/dataset".  n_rows is the sum of partition rows and n_cols the first
 * record's cols, as src/host.cpp:86-92 derives them. */
bfs_status bfs_dataset_load(const char *dir, const char *name, uint32_t partitions,
                            bfs_csc_host *out);
/* Writes a single- or multi-partition dataset in the same layout (the
 * inverse of the above; in-degree balanced destination-row split for P > 1,
 * exact row counts: bfs_dataset_write_split with BFS_SPLIT_BALANCED). */
bfs_status bfs_dataset_write(const char *dir, const char *name, uint32_t partitions,
                             const bfs_csc_host *g);
/* Destination-row split of bfs_dataset_write_split. */
typedef enum bfs_split {
  BFS_SPLIT_BALANCED = 0, /* in-degree balanced, exact rows, all edges kept at P = 1 */
  BFS_SPLIT_REF_NNZ = 1,  /* scripts/generator.py nnzSplit + round8 (:11-40) */
  BFS_SPLIT_REF_ROW = 2   /* scripts/generator.py rowSplit + round8 (:11-12, :42-54) */
} bfs_split;
/* bfs_dataset_write with the split chosen by split (bfs_split).  The two
 * reference modes write the files scripts/generator.py writes for the same
 * (square, duplicate-free, column-sorted) matrix byte for byte, quirks
 * included: round8 of the last break drops the last rows when it rounds
 * down, partitions can be empty, and the row split can write fewer than P
 * partitions (the folder is still named -csc-<P>). */
bfs_status bfs_dataset_write_split(const char *dir, const char *name, uint32_t partitions,
                                   const bfs_csc_host *g, int32_t split);
/* Reads only the meta records (20 bytes each: u32 rows, u32 cols, u64 nnz,
 * u32 startRow; src/graph_load.hpp:49-92).  Returns the record count in
 * *count (at most max_records are stored). */
bfs_status bfs_dataset_read_meta(const char *meta_path, uint32_t *rows, uint32_t *cols,
                                 uint64_t *nnz, uint32_t *start_row,
                                 uint32_t max_records, uint32_t *count);

#ifdef __cplusplus
}
#endif
#endif /* BFS_GB300_H */
