"""bench.py's N > 1 path (replicas only): the cross-rank reduction of times
(max) and edges (sum), on two gloo ranks on the CPU."""
import multiprocessing as mp
import os
import socket

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    r, w, local = bench.dist_setup("gloo")
    mx, sm = bench.reduce_max_sum([1.5 + r, 7.0 - r], [10.0 * (r + 1)], w)
    bench.barrier(w)
    q.put((r, w, mx, sm))
    dist.destroy_process_group()


def test_two_rank_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, mx, sm in out:
        assert w == 2
        assert mx == [2.5, 7.0]
        assert sm == [30.0]
