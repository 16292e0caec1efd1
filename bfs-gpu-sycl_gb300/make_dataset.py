"""Writes datasets in the reference's binary CSC layout.

Counterpart of scripts/genGraph.py + scripts/generator.py: produces
<dir>/<name>-csc-<P>/<name>-csc-{meta,<i>-indptr,<i>-inds}.bin for one or more
partition counts P.  --split picks the destination-row breaks:
  balanced (default)  in-degree balanced, exact row counts, every edge kept
  nnz | row           the reference generator's nnzSplit / rowSplit with its
                      round8 breaks (generator.py:11-54): the same files it
                      writes, byte for byte, including its quirks (the last
                      rows dropped when round8 rounds down, empty partitions,
                      fewer than P partitions from the row split); the default
                      name gets the reference's -nnz / -row suffix

Sources:
  rmat SCALE EF    seeded R-MAT (a/b/c/d .57/.19/.19/.05), deduplicated, no
                   self-loops, symmetrised unless --directed   [name rmat-S-EF]
  grid W H         4-neighbour grid, --delete fraction of edges removed
  er N DEG         Erdos-Renyi, average degree DEG
  edgelist FILE    text "u v [w]" per line ('#', '$', '%' comments), as
                   generator.py:loadGraph reads it: duplicate edges merged,
                   self-loops kept, no symmetrisation, --dim vertices
                   (default max id + 1)

Examples:
  python bfs-gpu-sycl_gb300/make_dataset.py rmat 19 16 --partitions 1 2 4
  python bfs-gpu-sycl_gb300/make_dataset.py edgelist my.txt --name my-graph
  python bfs-gpu-sycl_gb300/make_dataset.py edgelist my.txt --split nnz \
      --partitions 1 2 3 4 5 6 7 8        # like: generator.py my nnz
"""
import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import bfs_gb300 as B  # noqa: E402


def csc_from_edgelist(path, dim=None):
    rows = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s[0] in "#$%":
                continue
            p = s.split()
            if len(p) < 2:
                continue
            rows.append((int(p[0]), int(p[1])))
    if not rows:
        raise ValueError(f"{path}: no edges")
    e = np.array(rows, dtype=np.int64)
    n = int(dim) if dim else int(e.max()) + 1
    if e.min() < 0 or e.max() >= n:
        raise ValueError("vertex id outside [0, dim)")
    key = np.unique(e[:, 0] * n + e[:, 1])  # merge duplicates, sort by (u, v)
    u, v = key // n, key % n
    indptr = np.zeros(n + 1, np.uint64)
    np.add.at(indptr, u + 1, 1)
    indptr = np.cumsum(indptr).astype(np.uint32)
    return B.Csc(indptr, v.astype(np.uint32))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("kind", choices=["rmat", "grid", "er", "edgelist"])
    ap.add_argument("args", nargs="+")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--directed", action="store_true", help="R-MAT without symmetrisation")
    ap.add_argument("--delete", type=float, default=0.05, help="grid edge deletion fraction")
    ap.add_argument("--dim", type=int, default=None, help="edge list vertex count")
    ap.add_argument("--partitions", type=int, nargs="+", default=[1])
    ap.add_argument("--dir", default=os.path.join(os.getcwd(), "dataset"))
    ap.add_argument("--name", default=None)
    ap.add_argument("--split", choices=["balanced", "nnz", "row"], default="balanced")
    a = ap.parse_args(argv)
    if a.kind == "rmat":
        scale, ef = int(a.args[0]), int(a.args[1])
        g = B.gen_rmat(scale, ef, seed=a.seed, symmetrize=not a.directed)
        name = a.name or f"rmat-{scale}-{ef}"
    elif a.kind == "grid":
        w, h = int(a.args[0]), int(a.args[1])
        g = B.gen_grid(w, h, a.delete, a.seed)
        name = a.name or f"grid-{w}x{h}"
    elif a.kind == "er":
        n, deg = int(a.args[0]), float(a.args[1])
        g = B.gen_er(n, deg, a.seed)
        name = a.name or f"er-{n}-{deg:g}"
    else:
        g = csc_from_edgelist(a.args[0], a.dim)
        name = a.name or os.path.splitext(os.path.basename(a.args[0]))[0]
    if a.split != "balanced" and not a.name:
        name += "-" + a.split
    for p in a.partitions:
        B.dataset_write(g, name, p, a.dir, split=a.split)
        print(f"{a.dir}/{name}-csc-{p}: {g.n_cols} vertices, {g.nnz} edges, {p} partition(s)")


if __name__ == "__main__":
    main()
