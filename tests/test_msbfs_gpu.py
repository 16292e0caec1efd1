"""Batched multi-source BFS (64 roots per uint64 lane): every root's level row
and edgesCount must equal its own single-root run (oracle / golden)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_golden_cases_as_batches(B, cases):
    torch = torch_cuda()
    for name, c in cases.items():
        if "parts" in c:
            continue
        g = B.Graph.upload(B.Csc(c["indptr"], c["inds"], int(c["n_rows"]), int(c["n_cols"])))
        roots = c["roots"]
        out = torch.empty((len(roots), g.n_cols), dtype=torch.int32, device="cuda")
        ec, st = g.run_batch(roots, out.data_ptr())
        assert np.array_equal(out.cpu().numpy(), c["levels"]), name
        assert np.array_equal(ec, c["edges"]), name
        g.free()


def test_partial_batches_duplicates_and_odd_roots(B, O):
    torch = torch_cuda()
    g = B.gen_rmat(16, 16, seed=12)
    deg = g.degree()
    roots = list(B.sample_roots(g, 100, 12))
    zero = int(np.flatnonzero(deg == 0)[0])
    roots[5] = roots[3]          # duplicate inside one pass
    roots[70] = zero             # root without out-edges
    roots[99] = roots[0]         # duplicate across passes
    dg = B.Graph.upload(g)
    out = torch.empty((len(roots), g.n_cols), dtype=torch.int32, device="cuda")
    ec, st = dg.run_batch(roots, out.data_ptr())
    assert st.batches == 2
    ref, rec = O.oracle_bfs_many(g.indptr, g.inds, roots)
    assert np.array_equal(out.cpu().numpy(), ref)
    assert np.array_equal(ec, rec)
    # a second call reuses the workspace
    ec2, _ = dg.run_batch(roots[:7], out.data_ptr())
    assert np.array_equal(out[:7].cpu().numpy(), ref[:7]) and np.array_equal(ec2, rec[:7])
    # the host-driven level loop gives the same rows and counts
    out.fill_(7)
    ec3, st3 = dg.run_batch(roots, out.data_ptr(), loop="host")
    assert st3.batches == 2 and st3.launches == st.launches
    assert np.array_equal(out.cpu().numpy(), ref) and np.array_equal(ec3, rec)
    dg.free()


def test_rows_lt_cols(B, O):
    torch = torch_cuda()
    g = B.gen_rmat(12, 8, seed=3)
    h = B.Csc(g.indptr, g.inds, g.n_cols - 300, g.n_cols)
    dg = B.Graph.upload(h)
    roots = list(B.sample_roots(h, 10, 3)) + [g.n_cols - 1]  # last root is never expanded
    out = torch.empty((len(roots), g.n_cols), dtype=torch.int32, device="cuda")
    ec, _ = dg.run_batch(roots, out.data_ptr())
    ref, rec = O.oracle_bfs_many(h.indptr, h.inds, roots, n_rows=h.n_rows)
    assert np.array_equal(out.cpu().numpy(), ref) and np.array_equal(ec, rec)
    dg.free()


def test_config5a_rmat22_1024_roots(B, O):
    """RMAT-22/EF16 seed 6, 1024 seeded roots in 16 passes of 64; every row
    bit-exact to a single-root CPU run."""
    torch = torch_cuda()
    dg = B.Graph.gen_rmat_device(22, 16, seed=6)
    g = dg.download()
    roots = B.sample_roots(g, 1024, 6)
    out = torch.empty((64, g.n_cols), dtype=torch.int32, device="cuda")
    for b in range(16):
        rs = roots[64 * b:64 * (b + 1)]
        ec, st = dg.run_batch(rs, out.data_ptr())
        ref, rec = O.oracle_bfs_many(g.indptr, g.inds, rs, queue_form=True)
        assert np.array_equal(out.cpu().numpy(), ref), b
        assert np.array_equal(ec, rec), b
    dg.free()


def test_history_boundary_depths(B, O):
    """Paths whose searches end just before, at and after the 16-level mask
    history (the level rows are then written from the history, at the
    boundary, or partly direct), with the graph and the host loop."""
    torch = torch_cuda()
    for n in range(14, 21):
        src = np.arange(n - 1)
        u = np.concatenate([src, src + 1])
        v = np.concatenate([src + 1, src])
        order = np.lexsort((v, u))
        indptr = np.zeros(n + 1, np.uint32)
        np.add.at(indptr, u + 1, 1)
        g = B.Csc(np.cumsum(indptr).astype(np.uint32), v[order].astype(np.uint32))
        dg = B.Graph.upload(g)
        roots = [0, n - 1, n // 2, 1, 0]
        ref, rec = O.oracle_bfs_many(g.indptr, g.inds, roots)
        for loop in ("graph", "host"):
            out = torch.full((len(roots), n), 9, dtype=torch.int32, device="cuda")
            ec, st = dg.run_batch(roots, out.data_ptr(), loop=loop)
            assert np.array_equal(out.cpu().numpy(), ref), (n, loop)
            assert np.array_equal(ec, rec), (n, loop)
            assert st.max_levels == int(ref.max()) + 1
        dg.free()


def test_batch_into_host_arrays(B, O):
    """bfs_run_batch_host: rows copied to host per pass, equal to the device
    entry point's rows and to the oracle."""
    torch = torch_cuda()
    g = B.gen_rmat(14, 8, seed=31)
    dg = B.Graph.upload(g)
    roots = B.sample_roots(g, 80, 31)
    lv, ec, st = dg.run_batch_host(roots)
    assert st.batches == 2 and st.device_ms > 0
    ref, rec = O.oracle_bfs_many(g.indptr, g.inds, roots)
    assert np.array_equal(lv, ref) and np.array_equal(ec, rec)
    none, ec2, _ = dg.run_batch_host(roots, want_levels=False)
    assert none is None and np.array_equal(ec2, rec)
    out = torch.empty((len(roots), g.n_cols), dtype=torch.int32, device="cuda")
    ec3, _ = dg.run_batch(roots, out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), lv) and np.array_equal(ec3, ec)
    dg.free()


@pytest.mark.parametrize("K,min_edges", [(1024, 1), (1 << 14, 0)])
def test_hub_layout_batches(B, O, K, min_edges):
    """Batches on the relabelled graph of the hub layout: roots mapped in,
    rows written in original ids, and (min_edges = 1) the shared-memory
    bitmap of hubs every root has reached skipping mask probes on every
    level; a later change of layout rebuilds the batch workspace."""
    torch = torch_cuda()
    g = B.gen_rmat(16, 16, seed=14)
    dg = B.Graph.upload(g)
    roots = B.sample_roots(g, 96, 14)
    ref, rec = O.oracle_bfs_many(g.indptr, g.inds, roots)
    out = torch.empty((len(roots), g.n_cols), dtype=torch.int32, device="cuda")
    for hub in (K, 0, K):
        dg.hub_configure(hub, min_edges=min_edges)
        assert dg.hub_info()[1] == (hub > 0)
        for loop in ("graph", "host"):
            out.fill_(7)
            ec, st = dg.run_batch(roots, out.data_ptr(), loop=loop)
            assert np.array_equal(out.cpu().numpy(), ref), (hub, loop)
            assert np.array_equal(ec, rec), (hub, loop)
    dg.free()


def test_hub_layout_batches_past_the_history(B, O):
    """A star (a hub with 3000 leaves) with a 120-vertex chain hanging off it:
    relabelled (the hub takes half the edge endpoints) and deeper than the
    16-level history, so the deeper levels are written straight into the rows
    through the id map."""
    torch = torch_cuda()
    leaves, chain = 3000, 120
    n = 1 + leaves + chain
    src, dst = [], []
    for v in range(1, leaves + 1):
        src += [0, v]
        dst += [v, 0]
    prev = leaves
    for v in range(leaves + 1, n):
        src += [prev, v]
        dst += [v, prev]
        prev = v
    src, dst = np.array(src), np.array(dst)
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    indptr = np.zeros(n + 1, np.uint32)
    np.add.at(indptr, src + 1, 1)
    indptr = np.cumsum(indptr).astype(np.uint32)
    g = B.Csc(indptr, dst.astype(np.uint32), n, n)
    dg = B.Graph.upload(g)
    dg.hub_configure(128, min_edges=1)
    assert dg.hub_info()[:2] == (128, True)
    roots = np.array([0, 5, leaves, leaves + 7, n - 1] + list(range(10, 80)), np.uint32)
    ref, rec = O.oracle_bfs_many(g.indptr, g.inds, roots)
    assert ref.max() > 16
    out = torch.empty((len(roots), n), dtype=torch.int32, device="cuda")
    for loop in ("graph", "host"):
        out.fill_(7)
        ec, _ = dg.run_batch(roots, out.data_ptr(), loop=loop)
        assert np.array_equal(out.cpu().numpy(), ref), loop
        assert np.array_equal(ec, rec), loop
    dg.free()
