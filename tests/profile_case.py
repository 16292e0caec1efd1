"""Profiling fixture (not collected by pytest, not part of the engine): small,
self-contained workloads for profiling single kernels with ncu.  The commands
recorded in profiles/*.md run it.

Each case builds its input on the device from a fixed seed, runs the path once
and prints what it ran, so that an ncu capture (`-k <kernel> -s <skip> -c <n>`)
sees a known sequence of launches:

  bfs SCALE ARM [HUB]
                  R-MAT SCALE/EF16 seed 5, one BFS from the first seeded root
                  with the host-driven level loop (every level is a separate
                  launch, which ncu can capture; kernels inside a graph with a
                  conditional node cannot be).  ARM is llb|glb|slb followed by
                  the block size, e.g. glb256.  HUB: the hub layout's prefix
                  size (0 = off; default: automatic).  Prints (level,
                  frontier entries, edges) per level.
  grid SIDE ARM   SIDE x SIDE 4-neighbour grid with 5 % of edges deleted (seed
                  3), one BFS from the first seeded root, host-driven level
                  loop, as above: thousands of small levels (level generation
                  takes its warp path after each).
  batch SCALE     R-MAT SCALE/EF16 seed 6, one 64-root multi-source pass
                  (host-driven level loop, as above).
  multi [B I C]   the 256-graph mixed batch of the benchmark, one launch of
                  the persistent multi-graph kernel: B threads per block, I
                  items per lane, clusters of C blocks for the largest graphs
                  (default 512 4 1).

Examples:
  python tests/profile_case.py bfs 24 glb256
  ncu --set full --clock-control none -k regex:explore_global -s 2 -c 2 \\
      -o prof python tests/profile_case.py bfs 24 glb256
"""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "bfs-gpu-sycl_gb300"))
import torch  # noqa: E402

import bfs_gb300 as B  # noqa: E402


def case_bfs(scale, arm, hub=-1):
    dg = B.Graph.gen_rmat_device(scale, 16, seed=5)
    dg.hub_configure(hub)
    r = int(B.sample_roots(dg.download(), 1, 5)[0])
    lv = torch.empty(dg.n_cols, dtype=torch.int32, device="cuda")
    st = dg.run_device(r, lv.data_ptr(),
                       opts=B.options(arm[:3], int(arm[3:]), loop="host", record=1))
    t = st.levels_table()
    print("levels", [(i, t["frontier"][i], t["edges"][i]) for i in range(st.recorded)])
    print("ms", st.device_ms, "edges", st.edges_count)


def case_grid(side, arm):
    dg = B.Graph.upload(B.gen_grid(side, side, 0.05, 3), validate=False)
    r = int(B.sample_roots(dg.download(), 1, 3)[0])
    lv = torch.empty(dg.n_cols, dtype=torch.int32, device="cuda")
    st = dg.run_device(r, lv.data_ptr(), opts=B.options(arm[:3], int(arm[3:]), loop="host"))
    print("levels", st.num_levels, "ms", st.device_ms, "edges", st.edges_count)


def case_batch(scale):
    dg = B.Graph.gen_rmat_device(scale, 16, seed=6)
    roots = B.sample_roots(dg.download(), 64, 6)
    out = torch.empty((64, dg.n_cols), dtype=torch.int32, device="cuda")
    ec, st = dg.run_batch(roots, out.data_ptr(), loop="host")
    print("ms", st.device_ms, "levels", st.max_levels, "launches", st.launches,
          "edges", int(ec.sum()))


def case_multi(block=512, ipt=4, cluster=1):
    graphs, roots = B.multi_batch_graphs(B.multi_batch_specs())
    mb = B.MultiBatch(graphs)
    out = torch.empty(mb.total_cols, dtype=torch.int32, device="cuda")
    ec, ms = mb.run(roots, out.data_ptr(), block, ipt, cluster)
    print("ms", ms, "edges", int(ec.sum()), "vertices", mb.total_cols)


def main(argv):
    if not argv:
        print(__doc__)
        return 2
    torch.cuda.set_device(0)
    if argv[0] == "bfs" and len(argv) in (3, 4):
        case_bfs(int(argv[1]), argv[2], *(int(x) for x in argv[3:]))
    elif argv[0] == "grid" and len(argv) == 3:
        case_grid(int(argv[1]), argv[2])
    elif argv[0] == "batch" and len(argv) == 2:
        case_batch(int(argv[1]))
    elif argv[0] == "multi" and len(argv) in (1, 4):
        case_multi(*(int(x) for x in argv[1:]))
    else:
        print(__doc__)
        return 2
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
