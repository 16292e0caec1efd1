"""Generates the golden fixtures under tests/golden/ (run from the repo root).

The reference ships no tests and no golden vectors, and its only dataset lacks
the inds files.  The fixtures are therefore produced by the reference itself:
every level array and edge count below comes from the reference's own
run_bfs_cpu (src/run_bfs_cpu.hpp:5-85), compiled unmodified into
oracle/_ref/libref_bfs.so by oracle/Makefile.  The graphs are small seeded
cases from this engine's generators plus hand-made known-answer graphs.

It also records facts of the reference's shipped dataset
(dataset/rmat-19-16-nnz-csc-{1..4}): the meta files are copied verbatim (20
bytes per partition) and indptr statistics are stored as JSON, read with numpy
independently of the engine's loader.

Usage:  python tests/golden/make_golden.py [--reference /root/reference]
"""
import argparse
import hashlib
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "bfs-gpu-sycl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import bfs_gb300 as B  # noqa: E402
import bfs_oracle as O  # noqa: E402


def csc_from_edges(n, edges, n_rows=None):
    """Directed edge list -> CSC (duplicates kept in insertion order)."""
    adj = [[] for _ in range(n)]
    for u, v in edges:
        adj[u].append(v)
    indptr = np.zeros(n + 1, np.uint32)
    for i in range(n):
        indptr[i + 1] = indptr[i] + len(adj[i])
    inds = np.array([v for a in adj for v in a], np.uint32)
    return B.Csc(indptr, inds, n_rows if n_rows is not None else n, n)


def kat_graphs():
    g = {}
    # path 0-1-2-3 (both directions) plus isolated vertex 4
    g["path5"] = csc_from_edges(5, [(0, 1), (1, 0), (1, 2), (2, 1), (2, 3), (3, 2)])
    # star: centre 0 with 6 leaves
    g["star7"] = csc_from_edges(7, [(0, i) for i in range(1, 7)] + [(i, 0) for i in range(1, 7)])
    # two components, self-loop at 2 and duplicate edge 0->1
    g["disconnected"] = csc_from_edges(
        8, [(0, 1), (0, 1), (1, 0), (1, 2), (2, 2), (2, 1), (4, 5), (5, 4), (5, 6), (6, 5)])
    # directed cycle 0->1->...->9->0 (no reverse edges)
    g["dcycle10"] = csc_from_edges(10, [(i, (i + 1) % 10) for i in range(10)])
    # rows < cols: vertex 5 has out-edges but is never expanded
    g["rows_lt_cols"] = csc_from_edges(6, [(0, 1), (1, 5), (5, 2), (2, 3), (3, 4)], n_rows=5)
    # no edges at all
    g["empty"] = B.Csc(np.zeros(5, np.uint32), np.zeros(0, np.uint32), 4, 4)
    # binary tree of depth 6
    e = []
    for i in range(63):
        for c in (2 * i + 1, 2 * i + 2):
            if c < 127:
                e += [(i, c), (c, i)]
    g["tree127"] = csc_from_edges(127, e)
    return g


def seeded_graphs():
    return {
        "rmat10_ef16_s1": B.gen_rmat(10, 16, seed=1),
        "rmat11_ef8_s2_directed": B.gen_rmat(11, 8, seed=2, symmetrize=False),
        "grid32_d05_s3": B.gen_grid(32, 32, 0.05, 3),
        "er1024_d16_s4": B.gen_er(1024, 16.0, 4),
    }


def roots_for(name, g):
    if name == "path5":
        return [0, 2, 4]
    if name == "star7":
        return [0, 3]
    if name == "disconnected":
        return [0, 2, 3, 6]
    if name == "dcycle10":
        return [0, 7]
    if name == "rows_lt_cols":
        return [0, 5]
    if name == "empty":
        return [0, 3]
    if name == "tree127":
        return [0, 100]
    deg = g.degree()
    k = int((deg[: g.n_rows] > 0).sum())
    roots = list(B.sample_roots(g, min(4, k), seed=11))
    zero = np.flatnonzero(deg == 0)
    if len(zero):
        roots.append(int(zero[0]))  # a root without out-edges
    return roots


def split_partitions(g, parts):
    """Destination-range split into `parts` partitions (reference layout)."""
    brk = np.linspace(0, g.n_rows, parts + 1).astype(np.int64)
    ips, ixs = [], []
    for p in range(parts):
        lo, hi = brk[p], brk[p + 1]
        ip = np.zeros(g.n_cols + 1, np.uint32)
        ix = []
        for v in range(g.n_cols):
            s = g.inds[g.indptr[v]:g.indptr[v + 1]]
            s = s[(s >= lo) & (s < hi)]
            ix.extend(s.tolist())
            ip[v + 1] = len(ix)
        ips.append(ip)
        ixs.append(np.array(ix, np.uint32))
    return ips, ixs


def make_bfs_fixtures():
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libref_bfs.so missing: run `make -C oracle` where the "
                         "reference tree exists")
    cases = {}
    for name, g in list(kat_graphs().items()) + list(seeded_graphs().items()):
        roots = roots_for(name, g)
        lv = []
        ec = []
        for r in roots:
            levels, edges = O.ref_bfs([g.indptr], [g.inds], r, g.n_rows, g.n_cols)
            lv.append(levels)
            ec.append(edges)
        cases[name] = dict(indptr=g.indptr, inds=g.inds, n_rows=np.uint32(g.n_rows),
                           n_cols=np.uint32(g.n_cols), roots=np.array(roots, np.uint32),
                           levels=np.stack(lv).astype(np.int32),
                           edges=np.array(ec, np.uint64))
    # multi-partition cases for the multi-partition restatement
    g = B.gen_rmat(9, 8, seed=21, symmetrize=False)
    for parts in (2, 3, 4):
        ips, ixs = split_partitions(g, parts)
        roots = roots_for("mp", g)[:3]
        lv, ec = [], []
        for r in roots:
            levels, edges = O.ref_bfs(ips, ixs, r, g.n_rows, g.n_cols)
            lv.append(levels)
            ec.append(edges)
        d = dict(n_rows=np.uint32(g.n_rows), n_cols=np.uint32(g.n_cols),
                 roots=np.array(roots, np.uint32), levels=np.stack(lv).astype(np.int32),
                 edges=np.array(ec, np.uint64), parts=np.uint32(parts))
        for p in range(parts):
            d[f"indptr{p}"] = ips[p]
            d[f"inds{p}"] = ixs[p]
        cases[f"rmat9_ef8_s21_p{parts}"] = d
    out = os.path.join(HERE, "bfs_cases.npz")
    flat = {f"{c}__{k}": v for c, d in cases.items() for k, v in d.items()}
    np.savez_compressed(out, **flat)
    print(f"wrote {out} ({os.path.getsize(out)} bytes, {len(cases)} cases)")


def make_dataset_facts(reference):
    src = os.path.join(reference, "dataset")
    if not os.path.isdir(src):
        print("reference dataset not found; skipping dataset facts")
        return
    meta_dir = os.path.join(HERE, "ref_meta")
    os.makedirs(meta_dir, exist_ok=True)
    facts = {}
    for parts in (1, 2, 3, 4):
        d = os.path.join(src, f"rmat-19-16-nnz-csc-{parts}")
        meta = os.path.join(d, "rmat-19-16-nnz-csc-meta.bin")
        shutil.copyfile(meta, os.path.join(meta_dir, f"rmat-19-16-nnz-csc-{parts}-meta.bin"))
        raw = np.fromfile(meta, dtype=np.uint8)
        recs = []
        for i in range(len(raw) // 20):
            b = raw[20 * i:20 * i + 20].tobytes()
            recs.append(dict(rows=int.from_bytes(b[0:4], "little"),
                             cols=int.from_bytes(b[4:8], "little"),
                             nnz=int.from_bytes(b[8:16], "little"),
                             start_row=int.from_bytes(b[16:20], "little")))
        parts_info = []
        for p in range(parts):
            ip = np.fromfile(os.path.join(d, f"rmat-19-16-nnz-csc-{p}-indptr.bin"), np.uint32)
            deg = np.diff(ip.astype(np.int64))
            parts_info.append(dict(indptr_len=int(len(ip)), indptr_last=int(ip[-1]),
                                   max_degree=int(deg.max()), argmax_degree=int(deg.argmax()),
                                   sha256=hashlib.sha256(ip.tobytes()).hexdigest(),
                                   inds_present=os.path.exists(
                                       os.path.join(d, f"rmat-19-16-nnz-csc-{p}-inds.bin"))))
        facts[str(parts)] = dict(meta=recs, partitions=parts_info)
    with open(os.path.join(HERE, "ref_dataset_facts.json"), "w") as f:
        json.dump(facts, f, indent=1, sort_keys=True)
    print("wrote ref_dataset_facts.json and ref_meta/")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    a = ap.parse_args()
    make_bfs_fixtures()
    make_dataset_facts(a.reference)
