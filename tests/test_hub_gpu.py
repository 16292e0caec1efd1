"""GPU parity of the hub layout (degree-ordered relabelling plus the
shared-memory hub filter of the GLB explore kernel) and of the 16-byte chunk
walk of GLB, against the oracle.

The layout is internal to a graph handle: levels, parents and edge counts must
be exactly those of the plain path, whatever the prefix size, with the filter
loaded on every level (min_edges = 1) or only on large ones, relabelled or not,
in both level-loop drivers and with every explore arm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ARMS = [(lb, blk) for lb in ("llb", "glb", "slb") for blk in (128, 256, 512)]


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def check_tree(indptr, inds, levels, parents, root):
    """BFS-tree check: every reached non-root vertex's parent is an
    in-neighbour one level up; unreached vertices have parent -1."""
    assert parents[root] == root
    assert np.all(parents[levels < 0] == -1)
    v = np.flatnonzero(levels > 0)
    p = parents[v].astype(np.int64)
    assert np.all(p >= 0)
    assert np.all(levels[p] == levels[v] - 1)
    # v must appear in p's adjacency list (lists need not be sorted)
    lo = indptr[p].astype(np.int64)
    hi = indptr[p + 1].astype(np.int64)
    for a, b, x in zip(lo, hi, v):
        assert np.any(inds[a:b] == x), (int(x), int(a), int(b))


def single_cases(cases):
    return {k: v for k, v in cases.items() if "parts" not in v}


@pytest.mark.parametrize("hub", [0, 128, -1])
@pytest.mark.parametrize("loop", ["graph", "host"])
def test_golden_cases_hub(B, cases, hub, loop):
    """Golden vectors of the reference's run_bfs_cpu with the layout off, a
    128-vertex prefix (relabelled wherever the graph is larger) and the
    automatic one, the filter loaded on every level."""
    torch_cuda()
    for name, c in single_cases(cases).items():
        g = B.Graph.upload(B.Csc(c["indptr"], c["inds"], int(c["n_rows"]), int(c["n_cols"])))
        g.hub_configure(hub, min_edges=1)
        k, relabelled, mx = g.hub_info()
        assert mx > 0
        n_cols = int(c["n_cols"])
        if hub == 0:
            assert k == 0
        elif n_cols <= (128 if hub == 128 else mx) or int(c["n_rows"]) != n_cols:
            assert k > 0 and not relabelled, name  # identity prefix
        else:
            # relabelled when the prefix covers a quarter of the edge
            # endpoints, else no layout at all
            indeg = np.bincount(c["inds"].astype(np.int64), minlength=n_cols)
            covered = np.sort(indeg)[::-1][:min(hub if hub > 0 else mx, n_cols)].sum()
            if 4 * covered >= len(c["inds"]):
                assert k > 0 and relabelled, name
            else:
                assert k == 0, name
        for lb, blk in ARMS:
            for i, r in enumerate(c["roots"]):
                lv, pa, st = g.run(int(r), B.options(lb, blk, loop=loop), parents=True)
                assert np.array_equal(lv, c["levels"][i]), (name, hub, lb, blk, int(r))
                assert st.edges_count == int(c["edges"][i]), (name, hub, lb, blk, int(r))
                if int(c["n_cols"]) <= 4096:
                    check_tree(c["indptr"], c["inds"], lv, pa, int(r))
        g.free()


@pytest.mark.parametrize("K,min_edges", [(1024, 1), (4096, 0), (1 << 14, 1)])
def test_rmat_relabelled_every_arm(B, O, K, min_edges):
    """R-MAT-16 relabelled around prefixes smaller than the graph: every arm
    and the learned schedule, levels, edge counts and parent trees."""
    torch_cuda()
    g = B.gen_rmat(16, 16, seed=21)
    dg = B.Graph.upload(g)
    dg.hub_configure(K, min_edges=min_edges)
    k, relabelled, _ = dg.hub_info()
    assert k == K and relabelled
    roots = B.sample_roots(g, 3, 21)
    refs = {int(r): O.oracle_bfs(g.indptr, g.inds, int(r)) for r in roots}
    plans = ARMS + [("learned", 256)]
    for loop in ("graph", "host"):
        for lb, blk in plans:
            for r in roots:
                lv, pa, st = dg.run(int(r), B.options(lb, blk, loop=loop), parents=True)
                ref, ec = refs[int(r)]
                assert np.array_equal(lv, ref), (lb, blk, loop, int(r))
                assert st.edges_count == ec
                check_tree(g.indptr, g.inds, lv, pa, int(r))
    dg.free()


def test_rmat20_filter_on_large_levels(B, O):
    """R-MAT-20 with the default level threshold, so the large levels load the
    filter and the small ones do not: the automatic prefix and a 64 K one
    (both relabelled), ipt 4 and 8; device output through bfs_run_device
    checked against the oracle."""
    torch = torch_cuda()
    g = B.gen_rmat(20, 16, seed=5)
    dg = B.Graph.upload(g)
    roots = B.sample_roots(g, 2, 5)
    lv = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    for hub in (-1, 1 << 16):
        dg.hub_configure(hub)
        assert dg.hub_info()[1]
        for r in roots:
            ref, ec = O.oracle_bfs(g.indptr, g.inds, int(r))
            for lb, ipt in (("glb", 4), ("glb", 8), ("learned", 4)):
                st = dg.run_device(int(r), lv.data_ptr(), opts=B.options(lb, 256, ipt=ipt))
                assert np.array_equal(lv.cpu().numpy(), ref), (hub, lb, ipt, int(r))
                assert st.edges_count == ec
    dg.free()


@pytest.mark.parametrize("shift", [1, 2, 3])
def test_chunk_walk_misaligned_edges(B, O, shift):
    """The chunk walk counts 16-byte chunks from the boundary below inds: a
    wrapped device graph whose edge array starts 4, 8 or 12 bytes past a
    16-byte boundary (first and last chunks partly outside the array)."""
    torch = torch_cuda()
    g = B.gen_rmat(13, 8, seed=9)
    ip = torch.from_numpy(g.indptr.view(np.int32)).cuda()
    buf = torch.zeros(g.nnz + 8, dtype=torch.int32, device="cuda")
    buf[shift:shift + g.nnz] = torch.from_numpy(g.inds.view(np.int32)).cuda()
    ix_ptr = buf.data_ptr() + 4 * shift
    assert ix_ptr % 16 == 4 * shift
    dg = B.Graph.wrap_device(ip.data_ptr(), ix_ptr, g.n_rows, g.n_cols, g.nnz)
    for hub in (0, -1):
        dg.hub_configure(hub, min_edges=1)
        for r in B.sample_roots(g, 3, shift):
            for lb, loop in (("glb", "graph"), ("glb", "host"), ("learned", "graph")):
                lv, pa, st = dg.run(int(r), B.options(lb, 256, loop=loop), parents=True)
                ref, ec = O.oracle_bfs(g.indptr, g.inds, int(r))
                assert np.array_equal(lv, ref) and st.edges_count == ec, (shift, hub, lb, loop)
                check_tree(g.indptr, g.inds, lv, pa, int(r))
    dg.free()


def test_flat_degree_graph_gets_no_layout(B, O):
    """A uniform random graph has no hubs to speak of: the automatic request
    builds no layout (no relabelled copy), and results are unchanged."""
    torch_cuda()
    g = B.gen_er(1 << 16, 8.0, 4)
    dg = B.Graph.upload(g)
    dg.hub_configure(1024)
    assert dg.hub_info()[:2] == (0, False)
    r = int(B.sample_roots(g, 1, 4)[0])
    lv, _, st = dg.run(r, B.options("glb", 256))
    ref, ec = O.oracle_bfs(g.indptr, g.inds, r)
    assert np.array_equal(lv, ref) and st.edges_count == ec
    dg.free()


def test_rows_lt_cols_identity_prefix(B, O):
    """n_rows < n_cols keeps original ids (no relabelling across the row
    boundary); the prefix filter still runs."""
    torch_cuda()
    g = B.gen_rmat(13, 8, seed=4)
    n_rows = g.n_cols - 300
    dg = B.Graph.upload(B.Csc(g.indptr, g.inds, n_rows, g.n_cols))
    dg.hub_configure(256, min_edges=1)
    k, relabelled, _ = dg.hub_info()
    assert k == 256 and not relabelled
    for r in B.sample_roots(B.Csc(g.indptr, g.inds, n_rows, g.n_cols), 3, 4):
        lv, _, st = dg.run(int(r), B.options("glb", 512, loop="host"))
        ref, ec = O.oracle_bfs(g.indptr, g.inds, int(r), n_rows, g.n_cols)
        assert np.array_equal(lv, ref) and st.edges_count == ec
    dg.free()


def test_hub_layout_out_of_memory_runs_plain(B, O, monkeypatch):
    """A layout whose copy cannot be allocated leaves the handle without one;
    runs go on, on the original graph, with the same results."""
    torch_cuda()
    g = B.gen_rmat(14, 16, seed=2)
    dg = B.Graph.upload(g)
    monkeypatch.setenv("BFS_GB300_FAIL_ALLOC_BYTES", str(g.nnz * 4))
    dg.hub_configure(1024, min_edges=1)
    assert dg.hub_info()[0] == 0
    r = int(B.sample_roots(g, 1, 2)[0])
    lv, _, st = dg.run(r, B.options("glb", 256))
    ref, ec = O.oracle_bfs(g.indptr, g.inds, r)
    assert np.array_equal(lv, ref) and st.edges_count == ec
    monkeypatch.delenv("BFS_GB300_FAIL_ALLOC_BYTES")
    dg.hub_configure(1024, min_edges=1)
    assert dg.hub_info()[:2] == (1024, True)
    lv, _, st = dg.run(r, B.options("glb", 256))
    assert np.array_equal(lv, ref) and st.edges_count == ec
    dg.free()


def test_hub_configure_rejects_bad_request(B):
    torch_cuda()
    g = B.gen_rmat(10, 4, seed=1)
    dg = B.Graph.upload(g)
    with pytest.raises(B.BfsError):
        dg.hub_configure(-2)
    dg.free()


def star_and_path(B, n_leaves=3000, n_path=700, seed=13):
    """A star (centre of in-degree n_leaves) with a path of n_path vertices
    hanging off one leaf, ids shuffled: a 128-vertex prefix relabels the
    centre and scatters moved ids, and the path's levels run past 254."""
    n = 1 + n_leaves + n_path
    rng = np.random.default_rng(seed)
    ids = rng.permutation(n)  # logical vertex -> id
    c = ids[0]
    edges = []
    for k in range(1, n_leaves + 1):
        edges += [(c, ids[k]), (ids[k], c)]
    prev = ids[n_leaves]
    for k in range(n_leaves + 1, n):
        edges += [(prev, ids[k]), (ids[k], prev)]
        prev = ids[k]
    e = np.array(edges, np.int64)
    order = np.lexsort((e[:, 1], e[:, 0]))
    e = e[order]
    indptr = np.zeros(n + 1, np.uint32)
    indptr[1:] = np.cumsum(np.bincount(e[:, 0], minlength=n))
    return B.Csc(indptr, e[:, 1].astype(np.uint32)), int(c), int(ids[n - 1])


def test_deep_levels_relabelled(B, O):
    """Levels past the one-byte working range (>= 254) on a relabelled graph:
    deep levels are written in original ids during the BFS and kept by the
    output pass; shallow ones come from the working levels through pinv.
    Output buffers 16-byte aligned and not (the output pass's scalar path)."""
    torch = torch_cuda()
    g, centre, tail = star_and_path(B)
    dg = B.Graph.upload(g)
    dg.hub_configure(128, min_edges=1)
    assert dg.hub_info()[:2] == (128, True)
    buf = torch.empty(g.n_cols + 4, dtype=torch.int32, device="cuda")
    for r in (centre, tail):
        ref, ec = O.oracle_bfs(g.indptr, g.inds, r)
        assert ref.max() > 600
        for lb, loop in (("glb", "graph"), ("glb", "host"), ("learned", "graph"),
                         ("llb", "host"), ("slb", "graph")):
            lv, pa, st = dg.run(r, B.options(lb, 256, loop=loop), parents=True)
            assert np.array_equal(lv, ref), (r, lb, loop)
            assert st.edges_count == ec
            check_tree(g.indptr, g.inds, lv, pa, r)
        for shift in (0, 1, 3):
            ptr = buf.data_ptr() + 4 * shift
            st = dg.run_device(r, ptr, opts=B.options("glb", 256))
            out = buf[shift:shift + g.n_cols].cpu().numpy()
            assert np.array_equal(out, ref), (r, shift)
    dg.free()
