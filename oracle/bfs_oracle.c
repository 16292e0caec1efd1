/*
 * bfs_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's level-synchronous top-down BFS,
 * `run_bfs_cpu` (src/run_bfs_cpu.hpp:5-85), used as the parity checker for
 * the CUDA engine.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library; the product never links it.
 *
 * Parity pin: tests/test_oracle.py checks this restatement against
 *   (a) oracle/_ref/libref_bfs.so, the reference's own run_bfs_cpu compiled
 *       from its header by oracle/Makefile (when the reference tree exists), and
 *   (b) the golden fixtures in tests/golden/, which were produced by (a) with
 *       tests/golden/make_golden.py.
 *
 * Semantics kept from the reference (and relied upon by the parity tests):
 *   - masks are byte arrays of length n_cols; the level array has n_cols
 *     entries, -1 for unreached, 0 for the root (src/host.cpp:161-169);
 *   - only vertices tid < n_rows are ever expanded (run_bfs_cpu.hpp:31,67),
 *     so a root >= n_rows yields a level array with only the root at 0;
 *   - edgesCount = sum of out-degrees of every expanded vertex
 *     (run_bfs_cpu.hpp:36), accumulated in 64 bits;
 *   - multi-partition graphs (NUM_GPU > 1) expand each partition's slice of a
 *     vertex in partition order (run_bfs_cpu.hpp:47-62).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define ORACLE_OK 0
#define ORACLE_ERR_ARG 1
#define ORACLE_ERR_OOM 5

/* One BFS over P partitions.  indptr[p] has n_cols+1 entries, inds[p] the
 * partition's destination ids (global).  Follows run_bfs_cpu.hpp:24-75. */
static int bfs_partitioned(uint32_t n_rows, uint32_t n_cols, int n_parts,
                           const uint32_t *const *indptr,
                           const uint32_t *const *inds, uint32_t root,
                           int32_t *level, uint64_t *edges_out) {
  if (n_cols == 0 || root >= n_cols || n_rows > n_cols) return ORACLE_ERR_ARG;
  uint8_t *mask = (uint8_t *)calloc(n_cols, 1);
  uint8_t *upd = (uint8_t *)calloc(n_cols, 1);
  uint8_t *vis = (uint8_t *)calloc(n_cols, 1);
  if (!mask || !upd || !vis) {
    free(mask); free(upd); free(vis);
    return ORACLE_ERR_OOM;
  }
  for (uint32_t i = 0; i < n_cols; i++) level[i] = -1;
  /* host.cpp:167-169: seed the root */
  mask[root] = 1;
  vis[root] = 1;
  level[root] = 0;

  uint64_t explored = 0;
  int cur = 0;
  int again;
  do {
    again = 0;
    /* expansion pass over every row (run_bfs_cpu.hpp:31-64) */
    for (uint32_t tid = 0; tid < n_rows; tid++) {
      if (mask[tid] != 1) continue;
      mask[tid] = 0;
      for (int p = 0; p < n_parts; p++) {
        uint32_t b = indptr[p][tid], e = indptr[p][tid + 1];
        explored += (uint64_t)(e - b);
        for (uint32_t k = b; k < e; k++) {
          uint32_t id = inds[p][k];
          if (!vis[id]) {
            level[id] = cur + 1;
            upd[id] = 1;
            vis[id] = 1;
          }
        }
      }
    }
    /* promotion pass (run_bfs_cpu.hpp:67-73) */
    for (uint32_t tid = 0; tid < n_rows; tid++) {
      if (upd[tid] == 1) {
        mask[tid] = 1;
        again = 1;
        upd[tid] = 0;
      }
    }
    cur++;
  } while (again);

  free(mask); free(upd); free(vis);
  if (edges_out) *edges_out = explored;
  return ORACLE_OK;
}

/* Range check the graph so the oracle never reads out of bounds. */
static int check_graph(uint32_t n_cols, uint64_t nnz, const uint32_t *indptr,
                       const uint32_t *inds) {
  if (indptr[0] != 0) return ORACLE_ERR_ARG;
  for (uint32_t i = 0; i < n_cols; i++)
    if (indptr[i + 1] < indptr[i]) return ORACLE_ERR_ARG;
  if ((uint64_t)indptr[n_cols] != nnz) return ORACLE_ERR_ARG;
  for (uint64_t k = 0; k < nnz; k++)
    if (inds[k] >= n_cols) return ORACLE_ERR_ARG;
  return ORACLE_OK;
}

/* Single-partition BFS: the path the engine replaces. */
int oracle_bfs(uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
               const uint32_t *indptr, const uint32_t *inds, uint32_t root,
               int32_t *level_out, uint64_t *edges_count_out) {
  if (!indptr || !level_out || (nnz && !inds)) return ORACLE_ERR_ARG;
  if (check_graph(n_cols, nnz, indptr, inds) != ORACLE_OK) return ORACLE_ERR_ARG;
  const uint32_t *ip[1] = {indptr};
  const uint32_t *ix[1] = {inds};
  return bfs_partitioned(n_rows, n_cols, 1, ip, ix, root, level_out,
                         edges_count_out);
}

/* Queue form of the same BFS, O(n + nnz) instead of O(n * levels + nnz).
 * Levels are unique hop distances, so this gives the same level array and the
 * same edgesCount (sum of out-degrees of expanded vertices, i.e. reached
 * vertices < n_rows) as run_bfs_cpu; tests/test_oracle.py pins it to
 * oracle_bfs on every golden case.  Used for high-diameter graphs, where the
 * level-synchronous restatement would scan all n vertices per level. */
static int bfs_queue(uint32_t n_rows, uint32_t n_cols, const uint32_t *indptr,
                     const uint32_t *inds, uint32_t root, int32_t *level_out,
                     uint64_t *edges_count_out) {
  if (n_cols == 0 || root >= n_cols || n_rows > n_cols) return ORACLE_ERR_ARG;
  uint32_t *queue = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n_cols);
  if (!queue) return ORACLE_ERR_OOM;
  for (uint32_t i = 0; i < n_cols; i++) level_out[i] = -1;
  level_out[root] = 0;
  uint64_t explored = 0;
  size_t head = 0, tail = 0;
  queue[tail++] = root;
  while (head < tail) {
    uint32_t u = queue[head++];
    if (u >= n_rows) continue; /* never expanded (run_bfs_cpu.hpp:31) */
    uint32_t b = indptr[u], e = indptr[u + 1];
    explored += (uint64_t)(e - b);
    for (uint32_t k = b; k < e; k++) {
      uint32_t v = inds[k];
      if (level_out[v] < 0) {
        level_out[v] = level_out[u] + 1;
        queue[tail++] = v;
      }
    }
  }
  free(queue);
  if (edges_count_out) *edges_count_out = explored;
  return ORACLE_OK;
}

int oracle_bfs_queue(uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
                     const uint32_t *indptr, const uint32_t *inds, uint32_t root,
                     int32_t *level_out, uint64_t *edges_count_out) {
  if (!indptr || !level_out || (nnz && !inds)) return ORACLE_ERR_ARG;
  if (n_cols == 0 || check_graph(n_cols, nnz, indptr, inds) != ORACLE_OK)
    return ORACLE_ERR_ARG;
  return bfs_queue(n_rows, n_cols, indptr, inds, root, level_out, edges_count_out);
}

/* Multi-partition BFS (run_bfs_cpu.hpp:47-62): partition p holds indptr of
 * n_cols+1 entries and global destination ids. */
int oracle_bfs_multi(uint32_t n_rows, uint32_t n_cols, int n_parts,
                     const uint32_t *const *indptr, const uint32_t *const *inds,
                     const uint64_t *nnz, uint32_t root, int32_t *level_out,
                     uint64_t *edges_count_out) {
  if (n_parts < 1 || !indptr || !inds || !level_out) return ORACLE_ERR_ARG;
  for (int p = 0; p < n_parts; p++)
    if (check_graph(n_cols, nnz[p], indptr[p], inds[p]) != ORACLE_OK)
      return ORACLE_ERR_ARG;
  return bfs_partitioned(n_rows, n_cols, n_parts, indptr, inds, root, level_out,
                         edges_count_out);
}

/* ---- multi-root driver: independent single-threaded BFS runs, one root per
 * worker at a time.  Used to time the reference algorithm on every host
 * core, and to produce many oracle level arrays quickly in tests. ---- */
typedef struct {
  uint32_t n_rows, n_cols;
  uint64_t nnz;
  const uint32_t *indptr, *inds;
  const uint32_t *roots;
  uint32_t n_roots;
  int32_t *levels;         /* n_roots x n_cols, or NULL */
  uint64_t *edges;         /* n_roots */
  int queue_form;          /* 1: oracle_bfs_queue */
  volatile uint32_t next;  /* shared work counter */
  pthread_mutex_t lock;
  int status;
} many_job;

static void *many_worker(void *arg) {
  many_job *job = (many_job *)arg;
  int32_t *scratch = NULL;
  if (!job->levels) {
    scratch = (int32_t *)malloc(sizeof(int32_t) * (size_t)job->n_cols);
    if (!scratch) {
      pthread_mutex_lock(&job->lock);
      job->status = ORACLE_ERR_OOM;
      pthread_mutex_unlock(&job->lock);
      return NULL;
    }
  }
  for (;;) {
    pthread_mutex_lock(&job->lock);
    uint32_t r = job->next++;
    pthread_mutex_unlock(&job->lock);
    if (r >= job->n_roots) break;
    int32_t *lv = job->levels ? job->levels + (size_t)r * job->n_cols : scratch;
    const uint32_t *ip[1] = {job->indptr};
    const uint32_t *ix[1] = {job->inds};
    int st = job->queue_form
                 ? bfs_queue(job->n_rows, job->n_cols, job->indptr, job->inds,
                             job->roots[r], lv, &job->edges[r])
                 : bfs_partitioned(job->n_rows, job->n_cols, 1, ip, ix, job->roots[r],
                                   lv, &job->edges[r]);
    if (st != ORACLE_OK) {
      pthread_mutex_lock(&job->lock);
      job->status = st;
      pthread_mutex_unlock(&job->lock);
    }
  }
  free(scratch);
  return NULL;
}

int oracle_bfs_many(uint32_t n_rows, uint32_t n_cols, uint64_t nnz,
                    const uint32_t *indptr, const uint32_t *inds,
                    const uint32_t *roots, uint32_t n_roots, int n_threads,
                    int queue_form, int32_t *levels_out, uint64_t *edges_out) {
  if (!indptr || !roots || !edges_out || n_threads < 1) return ORACLE_ERR_ARG;
  if (check_graph(n_cols, nnz, indptr, inds) != ORACLE_OK) return ORACLE_ERR_ARG;
  many_job job;
  memset(&job, 0, sizeof(job));
  job.n_rows = n_rows; job.n_cols = n_cols; job.nnz = nnz;
  job.indptr = indptr; job.inds = inds;
  job.roots = roots; job.n_roots = n_roots;
  job.levels = levels_out; job.edges = edges_out;
  job.queue_form = queue_form;
  pthread_mutex_init(&job.lock, NULL);
  if (n_threads > (int)n_roots) n_threads = (int)n_roots;
  if (n_threads < 1) n_threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
  if (!th) return ORACLE_ERR_OOM;
  int started = 0;
  for (int t = 0; t < n_threads; t++) {
    if (pthread_create(&th[t], NULL, many_worker, &job) != 0) break;
    started++;
  }
  if (started == 0) many_worker(&job);
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&job.lock);
  return job.status;
}
