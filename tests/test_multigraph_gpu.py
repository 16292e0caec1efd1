"""Many small graphs in one persistent, CUDA-graph-captured launch: every
graph's levels and edgesCount equal its own oracle run, for every block size x
items-per-thread configuration the autotuner chooses from."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def oracle_all(O, graphs, roots):
    out = []
    for g, r in zip(graphs, roots):
        out.append(O.oracle_bfs(g.indptr, g.inds, int(r), g.n_rows, g.n_cols))
    return out


def check(mb, graphs, refs, out, ec):
    host = out.cpu().numpy()
    for i, (g, (lv, e)) in enumerate(zip(graphs, refs)):
        off = mb.offset(i)
        assert np.array_equal(host[off:off + g.n_cols], lv), i
        assert ec[i] == e, i


def test_config5b_256_uneven_rmat_graphs_every_config(B, O, tmp_path):
    torch = torch_cuda()
    specs = B.multi_batch_specs()
    assert len(specs) == 256 and {s[0] for s in specs} == set(range(10, 17))
    graphs, roots = B.multi_batch_graphs(specs)
    refs = oracle_all(O, graphs, roots)
    mb = B.MultiBatch(graphs)
    out = torch.empty(mb.total_cols, dtype=torch.int32, device="cuda")
    for blk, ipt in B.MULTI_CONFIGS:
        out.fill_(7)
        ec, ms = mb.run(roots, out.data_ptr(), blk, ipt)
        assert ms > 0
        check(mb, graphs, refs, out, ec)
    # the largest graphs shared by clusters of 2 / 4 / 8 blocks
    for blk, ipt, cl in B.MULTI_CONFIGS_ALL[len(B.MULTI_CONFIGS):]:
        out.fill_(7)
        ec, ms = mb.run(roots, out.data_ptr(), blk, ipt, cl)
        check(mb, graphs, refs, out, ec)
    cache = str(tmp_path / "autotune.tsv")
    best, times = mb.autotune(roots, out.data_ptr(), reps=2, cache_path=cache, clusters=False)
    assert best in B.MULTI_CONFIGS and all(t > 0 for t in times)
    best2, times2 = mb.autotune(roots, out.data_ptr(), cache_path=cache, clusters=False)
    assert best2 == best and all(t == -1 for t in times2)  # served from the cache
    ec, _ = mb.run(roots, out.data_ptr(), *best)
    check(mb, graphs, refs, out, ec)
    best3, times3 = mb.autotune(roots, out.data_ptr(), reps=2, cache_path=cache)
    assert best3 in B.MULTI_CONFIGS_ALL and len(times3) == len(B.MULTI_CONFIGS_ALL)
    ec, _ = mb.run(roots, out.data_ptr(), *best3)
    check(mb, graphs, refs, out, ec)
    mb.free()


def test_clusters_on_deep_and_degenerate_graphs(B, O):
    """Clustered runs on a batch whose large members are deep (grids), have
    rows < cols, or start from a root without out-edges."""
    torch = torch_cuda()
    g1 = B.gen_grid(200, 150, 0.05, 4)                     # hundreds of levels
    g2 = B.gen_rmat(13, 16, seed=5)
    g3 = B.Csc(g2.indptr, g2.inds, g2.n_cols - 100, g2.n_cols)
    small = [B.gen_rmat(8, 8, seed=s) for s in range(6)]
    graphs = [g1, g2, g3] + small
    zero_deg = int(np.flatnonzero(g2.degree() == 0)[0])
    roots = np.array([0, zero_deg, int(B.sample_roots(g3, 1, 3)[0])] +
                     [int(B.sample_roots(g, 1, 4)[0]) for g in small], np.uint32)
    refs = oracle_all(O, graphs, roots)
    mb = B.MultiBatch(graphs)
    out = torch.empty(mb.total_cols, dtype=torch.int32, device="cuda")
    for blk, ipt, cl in ((256, 2, 2), (512, 4, 4), (256, 4, 8), (512, 2, 8)):
        for _ in range(2):  # the second call reuses the captured launch
            out.fill_(7)
            ec, _ = mb.run(roots, out.data_ptr(), blk, ipt, cl)
            check(mb, graphs, refs, out, ec)
    mb.free()


def test_edge_cases(B, O):
    torch = torch_cuda()
    g1 = B.gen_rmat(10, 8, seed=1)
    g2 = B.Csc(g1.indptr, g1.inds, g1.n_cols - 50, g1.n_cols)  # rows < cols
    g3 = B.Csc(np.zeros(6, np.uint32), np.zeros(0, np.uint32))  # no edges
    g4 = B.gen_grid(64, 64, 0.05, 2)                               # 120+ levels
    graphs = [g1, g2, g3, g4]
    zero_deg = int(np.flatnonzero(g1.degree() == 0)[0])
    roots = np.array([zero_deg, int(B.sample_roots(g2, 1, 2)[0]), 3, 0], np.uint32)
    refs = oracle_all(O, graphs, roots)
    mb = B.MultiBatch(graphs)
    out = torch.empty(mb.total_cols, dtype=torch.int32, device="cuda")
    for blk, ipt in ((128, 1), (512, 4)):
        ec, _ = mb.run(roots, out.data_ptr(), blk, ipt)
        check(mb, graphs, refs, out, ec)
    # new roots on the same batch
    roots2 = np.array([5, 7, 0, 4095], np.uint32)
    refs2 = oracle_all(O, graphs, roots2)
    ec, _ = mb.run(roots2, out.data_ptr(), 256, 2)
    check(mb, graphs, refs2, out, ec)
    with pytest.raises(B.BfsError):
        mb.run(np.array([0, 0, 9, 0], np.uint32), out.data_ptr())  # root >= n_cols
    mb.free()
    big = B.Csc(np.zeros((1 << 18) + 2, np.uint32), np.zeros(0, np.uint32))
    with pytest.raises(B.BfsError):
        B.MultiBatch([big])
