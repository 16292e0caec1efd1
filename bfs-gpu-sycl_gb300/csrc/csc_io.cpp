// csc_io.cpp -- the reference's binary CSC dataset layout.
//
// Layout (src/graph_load.hpp:93-132, scripts/generator.py:115-195):
//   <dir>/<name>-csc-<P>/<name>-csc-meta.bin       P records of 20 bytes:
//        u32 rows, u32 cols, u64 nnz, u32 startRow   (little-endian, packed)
//   <dir>/<name>-csc-<P>/<name>-csc-<i>-indptr.bin u32[cols + 1]
//   <dir>/<name>-csc-<P>/<name>-csc-<i>-inds.bin   u32[nnz], global ids
// Partition i holds the edges whose destination lies in its row range; every
// partition has offsets for all columns.  A missing or empty file is an
// error, like readFromMM (graph_load.hpp:23-48).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <sys/types.h>

#include "bfs_internal.h"

using namespace bfsgb;

namespace {

std::string part_prefix(const char *dir, const char *name, uint32_t parts) {
  std::string base;
  if (dir && dir[0]) {
    base = dir;
  } else {
    const char *pwd = getenv("PWD");  // graph_load.hpp:98-101
    base = std::string(pwd ? pwd : ".") + "/dataset";
  }
  return base + "/" + name + "-csc-" + std::to_string(parts) + "/" + name + "-csc-";
}

bfs_status read_u32_file(const std::string &path, std::vector<uint32_t> *out) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return fail(BFS_ERR_IO, "file not found: " + path);
  if (fseek(f, 0, SEEK_END) != 0) {
    fclose(f);
    return fail(BFS_ERR_IO, "cannot seek: " + path);
  }
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (sz <= 0) {
    fclose(f);
    return fail(BFS_ERR_IO, "file size is 0: " + path);
  }
  out->resize((size_t)sz / 4);
  size_t got = out->empty() ? 0 : fread(out->data(), 4, out->size(), f);
  fclose(f);
  if (got != out->size()) return fail(BFS_ERR_IO, "short read: " + path);
  return BFS_OK;
}

bfs_status write_file(const std::string &path, const void *data, size_t bytes) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return fail(BFS_ERR_IO, "cannot create " + path);
  size_t put = bytes ? fwrite(data, 1, bytes, f) : 0;
  int rc = fclose(f);
  if (put != bytes || rc != 0) return fail(BFS_ERR_IO, "short write: " + path);
  return BFS_OK;
}

struct MetaRec {
  uint32_t rows, cols;
  uint64_t nnz;
  uint32_t start;
};

bfs_status read_meta(const std::string &path, std::vector<MetaRec> *recs) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return fail(BFS_ERR_IO, "file not found: " + path);
  unsigned char b[20];
  // graph_load.hpp:147-167 stops at the first incomplete record
  while (fread(b, 1, 20, f) == 20) {
    MetaRec r;
    std::memcpy(&r.rows, b, 4);
    std::memcpy(&r.cols, b + 4, 4);
    std::memcpy(&r.nnz, b + 8, 8);
    std::memcpy(&r.start, b + 16, 4);
    recs->push_back(r);
  }
  bool bad = ferror(f) != 0;
  fclose(f);
  if (bad) return fail(BFS_ERR_IO, "error reading " + path);
  if (recs->empty()) return fail(BFS_ERR_IO, "no meta records in " + path);
  return BFS_OK;
}

// Destination-row breaks of scripts/generator.py, computed the way numpy and
// scipy compute them there, so that the files come out byte-identical:
//   nnzSplit (:22-40): cum = inclusive prefix of row nnz (in-degree);
//     targets = np.arange(0, total, total / P) -- ceil(total / step) values
//     i * step in float64; break = first row with cum >= target
//     (np.searchsorted, side 'left'); then the row count appended.
//   rowSplit (:42-54): step = int(alignedIncrement(rows / P, 0, 64)), the
//     float quotient rounded up to a multiple of 64 (:249-254); breaks =
//     np.arange(0, rows, step) plus the row count -- fewer than P partitions
//     when step * (P - 1) >= rows.
// Every break is then round8'ed, (x + 4) & ~7 (:11-12), and a partition is
// the row slice [min(lo, rows), min(hi, rows)) (slicing past the end of the
// matrix clips), so the last rows are dropped when round8(rows) < rows.
bfs_status reference_breaks(int32_t split, uint32_t parts, const std::vector<uint64_t> &indeg,
                            std::vector<uint32_t> *brk) {
  const uint64_t rows = indeg.size();
  std::vector<uint64_t> b;
  if (split == BFS_SPLIT_REF_NNZ) {
    std::vector<uint64_t> cum(rows);
    uint64_t run = 0;
    for (uint64_t r = 0; r < rows; r++) cum[r] = run += indeg[r];
    if (run == 0) return fail(BFS_ERR_INVALID_ARG, "the reference's nnz split needs edges");
    const double step = (double)run / (double)parts;
    const uint64_t len = (uint64_t)std::ceil((double)run / step);
    for (uint64_t i = 0; i < len; i++) {
      const double t = (double)i * step;
      uint64_t lo = 0, hi = rows;  // first r with (double)cum[r] >= t
      while (lo < hi) {
        const uint64_t mid = (lo + hi) / 2;
        if ((double)cum[mid] < t) lo = mid + 1; else hi = mid;
      }
      b.push_back(lo);
    }
  } else {
    if (rows == 0) return fail(BFS_ERR_INVALID_ARG, "the reference's row split needs rows");
    double res = (double)rows / (double)parts;
    const double rem = std::fmod(res, 64.0);
    if (rem != 0.0) res += 64.0 - rem;
    const uint64_t step = (uint64_t)res;
    for (uint64_t x = 0; x < rows; x += step) b.push_back(x);
  }
  b.push_back(rows);
  brk->clear();
  for (uint64_t x : b) brk->push_back((uint32_t)std::min<uint64_t>((x + 4) & ~7ull, rows));
  return BFS_OK;
}

}  // namespace

extern "C" {

bfs_status bfs_dataset_read_meta(const char *meta_path, uint32_t *rows, uint32_t *cols,
                                 uint64_t *nnz, uint32_t *start_row, uint32_t max_records,
                                 uint32_t *count) {
  if (!meta_path || !count) return fail(BFS_ERR_INVALID_ARG, "null pointer");
  std::vector<MetaRec> recs;
  bfs_status rc = read_meta(meta_path, &recs);
  if (rc != BFS_OK) return rc;
  *count = (uint32_t)recs.size();
  for (uint32_t i = 0; i < recs.size() && i < max_records; i++) {
    if (rows) rows[i] = recs[i].rows;
    if (cols) cols[i] = recs[i].cols;
    if (nnz) nnz[i] = recs[i].nnz;
    if (start_row) start_row[i] = recs[i].start;
  }
  return BFS_OK;
}

bfs_status bfs_dataset_load(const char *dir, const char *name, uint32_t partitions,
                            bfs_csc_host *out) {
  if (!name || !out || partitions < 1 || partitions > 64)
    return fail(BFS_ERR_INVALID_ARG, "bad dataset arguments");
  std::memset(out, 0, sizeof(*out));
  const std::string pre = part_prefix(dir, name, partitions);
  std::vector<MetaRec> meta;
  bfs_status rc = read_meta(pre + "meta.bin", &meta);
  if (rc != BFS_OK) return rc;
  // host.cpp:86-92: cols from the first record, rows summed over records
  const uint32_t n_cols = meta[0].cols;
  uint64_t n_rows64 = 0;
  for (const MetaRec &m : meta) n_rows64 += m.rows;
  if (n_cols == 0 || n_rows64 > n_cols)
    return fail(BFS_ERR_GRAPH, "meta records give rows > cols or zero cols");
  const uint32_t n_rows = (uint32_t)n_rows64;

  std::vector<std::vector<uint32_t>> ip(partitions), ix(partitions);
  for (uint32_t p = 0; p < partitions; p++) {
    rc = read_u32_file(pre + std::to_string(p) + "-indptr.bin", &ip[p]);
    if (rc != BFS_OK) return rc;
    rc = read_u32_file(pre + std::to_string(p) + "-inds.bin", &ix[p]);
    if (rc != BFS_OK) return rc;
    if (ip[p].size() < (size_t)n_rows + 1)
      return fail(BFS_ERR_GRAPH, "indptr shorter than rows + 1 in partition " +
                                     std::to_string(p));
    // offsets of columns the file does not cover mean "no edges"
    const uint32_t last = ip[p].back();
    ip[p].resize((size_t)n_cols + 1, last);
    if (ip[p][0] != 0) return fail(BFS_ERR_GRAPH, "indptr[0] != 0");
    for (size_t v = 0; v < n_cols; v++)
      if (ip[p][v + 1] < ip[p][v]) return fail(BFS_ERR_GRAPH, "indptr not monotone");
    if (ip[p][n_cols] > ix[p].size())
      return fail(BFS_ERR_GRAPH, "indptr points past the end of inds");
  }
  uint64_t nnz = 0;
  for (uint32_t p = 0; p < partitions; p++) nnz += ip[p][n_cols];
  if (nnz > 0xFFFFFFFFull) return fail(BFS_ERR_UNSUPPORTED, "more than 2^32-1 edges");
  out->indptr = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)n_cols + 1));
  out->inds = (uint32_t *)malloc(sizeof(uint32_t) * (nnz ? nnz : 1));
  if (!out->indptr || !out->inds) {
    bfs_csc_host_free(out);
    return fail(BFS_ERR_OOM, "host allocation failed");
  }
  // merge partitions column by column, in partition order
  uint32_t pos = 0;
  out->indptr[0] = 0;
  for (uint32_t v = 0; v < n_cols; v++) {
    for (uint32_t p = 0; p < partitions; p++) {
      const uint32_t b = ip[p][v], e = ip[p][v + 1];
      for (uint32_t k = b; k < e; k++) {
        const uint32_t d = ix[p][k];
        if (d >= n_cols) {
          bfs_csc_host_free(out);
          return fail(BFS_ERR_GRAPH, "destination id >= cols");
        }
        out->inds[pos++] = d;
      }
    }
    out->indptr[v + 1] = pos;
  }
  out->n_rows = n_rows;
  out->n_cols = n_cols;
  out->nnz = nnz;
  return BFS_OK;
}

bfs_status bfs_dataset_write(const char *dir, const char *name, uint32_t partitions,
                             const bfs_csc_host *g) {
  return bfs_dataset_write_split(dir, name, partitions, g, BFS_SPLIT_BALANCED);
}

bfs_status bfs_dataset_write_split(const char *dir, const char *name, uint32_t partitions,
                                   const bfs_csc_host *g, int32_t split) {
  if (!name || !g || !g->indptr || (!g->inds && g->nnz) || partitions < 1 || partitions > 64)
    return fail(BFS_ERR_INVALID_ARG, "bad dataset arguments");
  if (split != BFS_SPLIT_BALANCED && split != BFS_SPLIT_REF_NNZ && split != BFS_SPLIT_REF_ROW)
    return fail(BFS_ERR_INVALID_ARG, "unknown split mode");
  const uint32_t n = g->n_cols;
  const std::string pre = part_prefix(dir, name, partitions);
  const std::string folder = pre.substr(0, pre.rfind('/'));
  // create the partition folder and its parents (mkdir -p)
  for (size_t i = 1; i <= folder.size(); i++) {
    if (i == folder.size() || folder[i] == '/') {
      const std::string d = folder.substr(0, i);
      struct stat sb;
      if (stat(d.c_str(), &sb) != 0 && mkdir(d.c_str(), 0755) != 0)
        return fail(BFS_ERR_IO, "cannot create directory " + d);
    }
  }
  // destination-row breaks balanced by in-degree (generator.py:22-40)
  std::vector<uint64_t> indeg(n, 0);
  for (uint64_t k = 0; k < g->nnz; k++) {
    if (g->inds[k] >= n) return fail(BFS_ERR_GRAPH, "destination id >= cols");
    indeg[g->inds[k]]++;
  }
  std::vector<uint32_t> brk;
  if (split == BFS_SPLIT_BALANCED) {
    brk.assign(partitions + 1, 0);
    brk[partitions] = g->n_rows;
    uint64_t run = 0;
    uint32_t p = 1;
    for (uint32_t r = 0; r < g->n_rows && p < partitions; r++) {
      while (p < partitions && run >= (g->nnz * p + partitions - 1) / partitions) brk[p++] = r;
      run += indeg[r];
    }
    while (p < partitions) brk[p++] = g->n_rows;
  } else {
    bfs_status rc = reference_breaks(split, partitions, indeg, &brk);
    if (rc != BFS_OK) return rc;
  }
  const uint32_t n_parts = (uint32_t)brk.size() - 1;
  // the balanced split keeps every edge in a single partition (rows may be
  // fewer than cols); the reference's splits keep only destinations inside
  // the (round8-clipped) row range, also for P = 1
  const bool keep_all = split == BFS_SPLIT_BALANCED && partitions == 1;
  std::vector<unsigned char> meta(20 * (size_t)n_parts);
  for (uint32_t p = 0; p < n_parts; p++) {
    const uint32_t lo = brk[p], hi = brk[p + 1];
    std::vector<uint32_t> ip((size_t)n + 1, 0), ix;
    for (uint32_t v = 0; v < n; v++) {
      for (uint32_t k = g->indptr[v]; k < g->indptr[v + 1]; k++) {
        const uint32_t d = g->inds[k];
        if (keep_all || (d >= lo && d < hi)) ix.push_back(d);
      }
      ip[v + 1] = (uint32_t)ix.size();
    }
    bfs_status rc = write_file(pre + std::to_string(p) + "-indptr.bin", ip.data(), ip.size() * 4);
    if (rc != BFS_OK) return rc;
    rc = write_file(pre + std::to_string(p) + "-inds.bin", ix.data(), ix.size() * 4);
    if (rc != BFS_OK) return rc;
    const uint32_t rows = hi - lo;
    const uint64_t nz = ix.size();
    std::memcpy(&meta[20 * p], &rows, 4);
    std::memcpy(&meta[20 * p + 4], &n, 4);
    std::memcpy(&meta[20 * p + 8], &nz, 8);
    std::memcpy(&meta[20 * p + 16], &lo, 4);
  }
  return write_file(pre + "meta.bin", meta.data(), meta.size());
}

}  // extern "C"
