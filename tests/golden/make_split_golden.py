"""Generates tests/golden/ref_splits.npz: dataset files written by the
reference's own dataset generator (scripts/generator.py).

The reference converts a text edge list into its binary CSC layout with
buildGraphManagerSingle(name, dim, pick) (generator.py:86-103): the graph is
transposed, split into destination-row partitions by nnzSplit (in-degree
balanced, generator.py:22-40) or rowSplit (equal row counts rounded up to 64,
generator.py:42-54), every break rounded by round8 (generator.py:11-12), and
written by prepareGraph/serializeGraphData (generator.py:115-195) for
P = 1..8.  This script imports that module from the reference checkout,
points its input and output folders at a temporary directory (the module's
own globals localtxtFolder / graphDataRoot; nothing is written into the
reference), runs it on a few small seeded edge lists and stores every file it
wrote, byte for byte, in one npz:

  <graph>/edges                     uint32 [m, 2] edge list fed to the generator
  <graph>/<pick>/<P>/meta           uint8  the -meta.bin file
  <graph>/<pick>/<P>/<i>/indptr     uint8  the <i>-indptr.bin file
  <graph>/<pick>/<P>/<i>/inds       uint8  the <i>-inds.bin file

Usage:  python tests/golden/make_split_golden.py [--reference /root/reference]
"""
import argparse
import importlib.util
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def edge_lists():
    rng = np.random.default_rng(2024)
    g = {}
    # 61 vertices (round8(61) = 64: rows are clipped to the matrix), uniform
    e = rng.integers(0, 61, size=(400, 2))
    g["u61"] = e
    # 59 vertices (round8(59) = 56: the last 3 destination rows are dropped)
    e = rng.integers(0, 59, size=(300, 2))
    e[0] = (58, 58)  # make sure the vertex count is 59
    g["u59"] = e
    # 203 vertices, skewed in-degree (hubs at low ids), duplicates and self-loops
    src = rng.integers(0, 203, size=1500)
    dst = np.minimum((rng.pareto(1.2, size=1500) * 6).astype(np.int64), 202)
    e = np.stack([src, dst], 1)
    e[:20] = e[20:40]          # duplicate edges
    e[40:45, 1] = e[40:45, 0]  # self-loops
    e[45] = (202, 0)
    g["skew203"] = e
    # 300 vertices, edges only into the last vertices (empty leading partitions)
    src = rng.integers(0, 300, size=200)
    dst = rng.integers(280, 300, size=200)
    g["tail300"] = np.stack([src, dst], 1)
    return g


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    a = ap.parse_args()
    path = os.path.join(a.reference, "scripts", "generator.py")
    spec = importlib.util.spec_from_file_location("ref_generator", path)
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        txt = os.path.join(tmp, "txt") + "/"
        ds = os.path.join(tmp, "dataset") + "/"
        os.makedirs(txt)
        os.makedirs(ds)
        gen.localtxtFolder = txt
        gen.graphDataRoot = ds
        for name, e in edge_lists().items():
            e = np.asarray(e, np.uint32)
            out[f"{name}/edges"] = e
            with open(os.path.join(txt, name + ".txt"), "w") as f:
                f.write("# seeded test graph\n")
                for u, v in e:
                    f.write(f"{u}\t{v}\n")
            for pick in ("nnz", "row"):
                gen.buildGraphManagerSingle(name, None, pick)
                for p in gen.num_cu:
                    folder = os.path.join(ds, f"{name}-{pick}-csc-{p}")
                    pre = os.path.join(folder, f"{name}-{pick}-csc-")
                    key = f"{name}/{pick}/{p}"
                    out[key + "/meta"] = np.fromfile(pre + "meta.bin", np.uint8)
                    n_parts = len(out[key + "/meta"]) // 20
                    for i in range(n_parts):
                        out[f"{key}/{i}/indptr"] = np.fromfile(f"{pre}{i}-indptr.bin", np.uint8)
                        out[f"{key}/{i}/inds"] = np.fromfile(f"{pre}{i}-inds.bin", np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_splits.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_splits.npz"), len(out), "arrays")


if __name__ == "__main__":
    sys.exit(main())
