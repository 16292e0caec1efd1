/*
 * graph_gen_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Independent CPU restatement of the engine's seeded R-MAT generator and root
 * sampler, so that bench.py's reference arm (the CPU BFS of the reference,
 * src/run_bfs_cpu.hpp:5-85) builds its graph and roots without loading the
 * engine library.  tests/test_oracle_gen.py pins both functions to the
 * engine's bfs_gen_rmat_host / bfs_sample_roots outputs byte for byte.
 *
 * The published algorithms restated here:
 *   - SplitMix64's output function (Steele, Lea, Flood, "Fast splittable
 *     pseudorandom number generators", OOPSLA 2014) as a counter-based hash:
 *     draw(counter, lane) = mix64(mix64(seed) + (counter << 8) + lane);
 *   - R-MAT (Chakrabarti, Zhan, Faloutsos, SDM 2004): edge i descends `scale`
 *     quadrant levels, most significant bit first; level l uses the low
 *     (l even) or high (l odd) 32 bits of draw(i, l / 2) compared with the
 *     fixed-point thresholds floor(p * 2^32) of a, a+b, a+b+c; quadrant q
 *     appends q >> 1 to the source and q & 1 to the destination.  The
 *     quadrant probabilities .57/.19/.19/.05 are Graph500's, the ones the
 *     reference's scripts/genGraph.py:48-52 passes to networkit;
 *   - the CSC conventions of the reference's scripts/generator.py:115-147:
 *     uint32 offsets, destinations sorted within each vertex, duplicates
 *     merged, self-loops dropped; symmetrize adds the reverse of each edge.
 *   - roots: draw j maps to a vertex by the high 32 bits times n >> 32;
 *     vertices with no out-edges and repeats are skipped.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <unistd.h>

#define GEN_OK 0
#define GEN_ERR_ARG 1
#define GEN_ERR_GRAPH 3
#define GEN_ERR_OOM 5

static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t draw(uint64_t seed_mixed, uint64_t counter, uint32_t lane) {
  return mix64(seed_mixed + (counter << 8) + lane);
}

static uint32_t threshold(double p) {
  if (p <= 0.0) return 0;
  if (p >= 1.0) return 0xFFFFFFFFu;
  return (uint32_t)(p * 4294967296.0); /* floor for p in (0, 1) */
}

static uint32_t to_range(uint64_t h, uint32_t n) {
  return (uint32_t)(((h >> 32) * (uint64_t)n) >> 32);
}

typedef struct {
  uint32_t scale;
  uint64_t n_edges;
  uint64_t seed_mixed;
  uint32_t t_a, t_ab, t_abc;
} rmat_t;

static void rmat_pair(const rmat_t *p, uint64_t i, uint32_t *src, uint32_t *dst) {
  uint32_t u = 0, v = 0;
  uint64_t h = 0;
  for (uint32_t l = 0; l < p->scale; l++) {
    if ((l & 1u) == 0) h = draw(p->seed_mixed, i, l >> 1);
    const uint32_t r = (l & 1u) ? (uint32_t)(h >> 32) : (uint32_t)h;
    const uint32_t q = r < p->t_a ? 0u : r < p->t_ab ? 1u : r < p->t_abc ? 2u : 3u;
    u = (u << 1) | (q >> 1);
    v = (v << 1) | (q & 1u);
  }
  *src = u;
  *dst = v;
}

/* ---- sorting of one adjacency list (quicksort, insertion sort below 24) -- */
static void isort(uint32_t *a, int64_t n) {
  for (int64_t i = 1; i < n; i++) {
    uint32_t x = a[i];
    int64_t j = i - 1;
    while (j >= 0 && a[j] > x) {
      a[j + 1] = a[j];
      j--;
    }
    a[j + 1] = x;
  }
}

static void qsort_u32(uint32_t *a, int64_t n) {
  while (n > 24) {
    uint32_t x = a[0], y = a[n / 2], z = a[n - 1]; /* median of three */
    uint32_t piv = x < y ? (y < z ? y : (x < z ? z : x)) : (x < z ? x : (y < z ? z : y));
    int64_t i = 0, j = n - 1;
    for (;;) {
      while (a[i] < piv) i++;
      while (a[j] > piv) j--;
      if (i >= j) break;
      uint32_t t = a[i];
      a[i] = a[j];
      a[j] = t;
      i++;
      j--;
    }
    /* recurse on the smaller side, loop on the larger */
    int64_t left = j + 1;
    if (left < n - left) {
      qsort_u32(a, left);
      a += left;
      n -= left;
    } else {
      qsort_u32(a + left, n - left);
      n = left;
    }
  }
  isort(a, n);
}

/* ---- threaded passes ------------------------------------------------------ */
typedef struct {
  const rmat_t *p;
  int symmetrize;
  uint64_t begin, end;
  uint32_t *cnt;          /* count pass */
  uint64_t *cursor;       /* scatter pass */
  uint32_t *buf;
  const uint64_t *off;    /* sort pass */
  int pass;
} job_t;

static void *work(void *arg) {
  job_t *j = (job_t *)arg;
  if (j->pass == 0 || j->pass == 1) {
    for (uint64_t i = j->begin; i < j->end; i++) {
      uint32_t u, v;
      rmat_pair(j->p, i, &u, &v);
      if (u == v) continue;
      if (j->pass == 0) {
        __atomic_fetch_add(&j->cnt[u], 1u, __ATOMIC_RELAXED);
        if (j->symmetrize) __atomic_fetch_add(&j->cnt[v], 1u, __ATOMIC_RELAXED);
      } else {
        j->buf[__atomic_fetch_add(&j->cursor[u], 1ull, __ATOMIC_RELAXED)] = v;
        if (j->symmetrize) j->buf[__atomic_fetch_add(&j->cursor[v], 1ull, __ATOMIC_RELAXED)] = u;
      }
    }
  } else {
    /* sort + merge duplicates per vertex; cnt[v] becomes the unique count */
    for (uint64_t v = j->begin; v < j->end; v++) {
      uint32_t *s = j->buf + j->off[v];
      int64_t n = (int64_t)(j->off[v + 1] - j->off[v]);
      qsort_u32(s, n);
      int64_t k = 0;
      for (int64_t i = 0; i < n; i++)
        if (k == 0 || s[i] != s[k - 1]) s[k++] = s[i];
      j->cnt[v] = (uint32_t)k;
    }
  }
  return NULL;
}

static int run_threads(job_t *proto, uint64_t n, int nt) {
  pthread_t th[64];
  job_t jobs[64];
  if (nt < 1) nt = 1;
  if (nt > 64) nt = 64;
  if (n < 4096) nt = 1;
  uint64_t chunk = (n + nt - 1) / nt;
  int created[64] = {0};
  for (int t = 0; t < nt; t++) {
    jobs[t] = *proto;
    jobs[t].begin = (uint64_t)t * chunk;
    jobs[t].end = jobs[t].begin + chunk < n ? jobs[t].begin + chunk : n;
    if (jobs[t].begin >= jobs[t].end) continue;
    if (pthread_create(&th[t], NULL, work, &jobs[t]) == 0)
      created[t] = 1;
    else
      work(&jobs[t]); /* no thread: run this share here */
  }
  for (int t = 0; t < nt; t++)
    if (created[t]) pthread_join(th[t], NULL);
  return 0;
}

void oracle_free(void *p) { free(p); }

/* R-MAT graph with 2^scale vertices and edge_factor * 2^scale generated edges
 * as a CSC (indptr: n + 1 offsets, inds: *nnz_out destinations, both
 * malloc'ed; release with oracle_free).  threads <= 0: one per online CPU. */
int oracle_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                    uint64_t seed, int symmetrize, int threads, uint32_t **indptr_out,
                    uint32_t **inds_out, uint64_t *nnz_out) {
  if (!indptr_out || !inds_out || !nnz_out) return GEN_ERR_ARG;
  if (scale < 1 || scale > 30 || edge_factor < 1) return GEN_ERR_ARG;
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0 + 1e-12) return GEN_ERR_ARG;
  if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
  rmat_t p;
  p.scale = scale;
  p.n_edges = (uint64_t)edge_factor << scale;
  p.seed_mixed = mix64(seed);
  p.t_a = threshold(a);
  p.t_ab = threshold(a + b);
  p.t_abc = threshold(a + b + c);
  const uint32_t n = 1u << scale;

  uint32_t *cnt = (uint32_t *)calloc(n, sizeof(uint32_t));
  uint64_t *off = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)n + 1));
  if (!cnt || !off) {
    free(cnt);
    free(off);
    return GEN_ERR_OOM;
  }
  job_t proto;
  memset(&proto, 0, sizeof(proto));
  proto.p = &p;
  proto.symmetrize = symmetrize != 0;
  proto.cnt = cnt;
  proto.pass = 0;
  run_threads(&proto, p.n_edges, threads);
  off[0] = 0;
  for (uint32_t v = 0; v < n; v++) off[v + 1] = off[v] + cnt[v];
  uint32_t *buf = (uint32_t *)malloc(sizeof(uint32_t) * (off[n] ? off[n] : 1));
  uint64_t *cursor = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
  if (!buf || !cursor) {
    free(cnt);
    free(off);
    free(buf);
    free(cursor);
    return GEN_ERR_OOM;
  }
  memcpy(cursor, off, sizeof(uint64_t) * (size_t)n);
  proto.cursor = cursor;
  proto.buf = buf;
  proto.pass = 1;
  run_threads(&proto, p.n_edges, threads);
  free(cursor);
  proto.off = off;
  proto.pass = 2;
  run_threads(&proto, n, threads);

  uint32_t *indptr = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n + 1));
  uint64_t nnz = 0;
  for (uint32_t v = 0; v < n; v++) nnz += cnt[v];
  if (!indptr || nnz > 0xFFFFFFFFull) {
    free(cnt);
    free(off);
    free(buf);
    free(indptr);
    return indptr ? GEN_ERR_GRAPH : GEN_ERR_OOM;
  }
  /* compact the unique prefixes of every list in place (left to right) */
  indptr[0] = 0;
  for (uint32_t v = 0; v < n; v++) {
    indptr[v + 1] = indptr[v] + cnt[v];
    if (off[v] != indptr[v]) memmove(buf + indptr[v], buf + off[v], sizeof(uint32_t) * cnt[v]);
  }
  free(cnt);
  free(off);
  uint32_t *inds = (uint32_t *)realloc(buf, sizeof(uint32_t) * (nnz ? nnz : 1));
  if (!inds) inds = buf;
  *indptr_out = indptr;
  *inds_out = inds;
  *nnz_out = nnz;
  return GEN_OK;
}

/* count distinct roots with out-degree > 0 among vertices < n_rows. */
int oracle_sample_roots(const uint32_t *indptr, uint32_t n_rows, uint32_t count, uint64_t seed,
                        uint32_t *roots_out) {
  if (!indptr || (!roots_out && count)) return GEN_ERR_ARG;
  if (count == 0) return GEN_OK;
  uint64_t eligible = 0;
  for (uint32_t v = 0; v < n_rows; v++) eligible += indptr[v + 1] > indptr[v];
  if (eligible < count) return GEN_ERR_GRAPH;
  const uint64_t sm = mix64(seed ^ 0x726F6F7473ull); /* the bytes of "roots" */
  uint32_t got = 0;
  for (uint64_t j = 0; got < count; j++) {
    const uint32_t v = to_range(draw(sm, j, 0), n_rows);
    if (indptr[v + 1] == indptr[v]) continue;
    int seen = 0;
    for (uint32_t k = 0; k < got && !seen; k++) seen = roots_out[k] == v;
    if (!seen) roots_out[got++] = v;
  }
  return GEN_OK;
}
