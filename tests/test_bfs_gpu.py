"""GPU parity of the CUDA BFS against the oracle and the reference's golden
vectors, through the C ABI.  Every explore form (LLB/GLB/SLB) at every block
size (128/256/512), both level-loop drivers (device CUDA-graph loop and host
loop), bit-exact levels and edgesCount; parent arrays checked as BFS trees."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ARMS = [(lb, blk) for lb in ("llb", "glb", "slb") for blk in (128, 256, 512)]


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def check_parents(indptr, inds, levels, parents, root):
    reached = np.flatnonzero(levels >= 0)
    assert parents[root] == root
    assert np.all(parents[levels < 0] == -1)
    for v in reached:
        if v == root:
            continue
        p = int(parents[v])
        assert levels[p] == levels[v] - 1, (v, p)
        assert v in inds[indptr[p]:indptr[p + 1]], (v, p)


def single_cases(cases):
    return {k: v for k, v in cases.items() if "parts" not in v}


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_golden_cases_every_arm(B, cases, loop):
    torch_cuda()
    for name, c in single_cases(cases).items():
        g = B.Graph.upload(B.Csc(c["indptr"], c["inds"], int(c["n_rows"]), int(c["n_cols"])))
        for lb, blk in ARMS:
            o = B.options(lb, blk, loop=loop)
            for i, r in enumerate(c["roots"]):
                lv, pa, st = g.run(int(r), o, parents=True)
                assert np.array_equal(lv, c["levels"][i]), (name, lb, blk, int(r))
                assert st.edges_count == int(c["edges"][i]), (name, lb, blk, int(r))
                assert st.reached == int((lv >= 0).sum())
                assert st.num_levels == int(lv.max()) + 1
                if int(c["n_cols"]) <= 2048:
                    check_parents(c["indptr"], c["inds"], lv, pa, int(r))
        g.free()


def test_multi_partition_dataset_through_loader(B, cases, tmp_path):
    """P > 1 reference layout: merged by the loader, BFS equals the reference's
    multi-partition run_bfs_cpu (golden)."""
    torch_cuda()
    for name, c in cases.items():
        if "parts" not in c:
            continue
        P = int(c["parts"])
        folder = tmp_path / f"mp-csc-{P}"
        folder.mkdir()
        meta = b""
        start = 0
        for p in range(P):
            c[f"indptr{p}"].astype(np.uint32).tofile(folder / f"mp-csc-{p}-indptr.bin")
            ix = c[f"inds{p}"].astype(np.uint32)
            (ix if len(ix) else np.zeros(1, np.uint32)).tofile(folder / f"mp-csc-{p}-inds.bin")
            rows = int(c["n_rows"]) // P if p < P - 1 else int(c["n_rows"]) - start
            meta += (np.array([rows, int(c["n_cols"])], np.uint32).tobytes()
                     + np.array([len(ix)], np.uint64).tobytes()
                     + np.array([start], np.uint32).tobytes())
            start += rows
        (folder / "mp-csc-meta.bin").write_bytes(meta)
        h = B.dataset_load("mp", P, str(tmp_path))
        g = B.Graph.upload(h)
        for i, r in enumerate(c["roots"]):
            lv, _, st = g.run(int(r), B.options("glb", 256))
            assert np.array_equal(lv, c["levels"][i]), name
            assert st.edges_count == int(c["edges"][i])
        g.free()
        import shutil
        shutil.rmtree(folder)


def test_run_device_and_validator(B):
    torch = torch_cuda()
    g = B.gen_rmat(14, 16, seed=9)
    dg = B.Graph.upload(g)
    lv = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    pa = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    for r in B.sample_roots(g, 3, 2):
        for lb, blk in ARMS:
            st = dg.run_device(int(r), lv.data_ptr(), pa.data_ptr(), B.options(lb, blk))
            torch.cuda.synchronize()
            assert dg.validate_device(int(r), lv.data_ptr(), pa.data_ptr()) == 0
            host = lv.cpu().numpy()
            from bfs_oracle import oracle_bfs
            ref, ec = oracle_bfs(g.indptr, g.inds, int(r))
            assert np.array_equal(host, ref) and st.edges_count == ec
        # the validator catches a wrong level and a wrong parent
        bad = lv.clone()
        k = int(torch.nonzero(bad > 1)[0])
        bad[k] += 1
        assert dg.validate_device(int(r), bad.data_ptr()) > 0
        badp = pa.clone()
        badp[k] = int(r) if int(lv[k]) != 1 else -1
        assert dg.validate_device(int(r), lv.data_ptr(), badp.data_ptr()) > 0
    dg.free()


def test_edge_cases(B):
    torch_cuda()
    # no edges at all
    g = B.Graph.upload(B.Csc(np.zeros(9, np.uint32), np.zeros(0, np.uint32)))
    lv, pa, st = g.run(3, parents=True)
    assert lv.tolist() == [-1, -1, -1, 0, -1, -1, -1, -1]
    assert st.edges_count == 0 and st.num_levels == 1 and pa[3] == 3
    with pytest.raises(B.BfsError) as e:
        g.run(8)
    assert e.value.status == "BFS_ERR_ROOT"
    g.free()
    # single vertex with a self-loop
    g = B.Graph.upload(B.Csc(np.array([0, 1], np.uint32), np.array([0], np.uint32)))
    lv, _, st = g.run(0)
    assert lv.tolist() == [0] and st.edges_count == 1
    g.free()
    # malformed CSC is rejected at upload
    with pytest.raises(B.BfsError) as e:
        B.Graph.upload(B.Csc(np.array([0, 2, 1], np.uint32), np.array([0, 1], np.uint32)))
    assert e.value.status == "BFS_ERR_GRAPH"
    with pytest.raises(B.BfsError) as e:
        B.Graph.upload(B.Csc(np.array([0, 1, 1], np.uint32), np.array([5], np.uint32)))
    assert e.value.status == "BFS_ERR_GRAPH"
    # bad options
    g = B.Graph.upload(B.gen_grid(4, 4, 0.0, 1))
    o = B.options()
    o.block = 100
    with pytest.raises(B.BfsError) as e:
        g.run(0, o)
    assert e.value.status == "BFS_ERR_INVALID_ARG"
    g.free()


def test_high_degree_hub_and_long_path(B, O):
    """A hub of degree 200k next to a 3000-vertex path: tiles with huge and
    tiny degrees, and thousands of levels through the device loop."""
    torch_cuda()
    n_hub = 200_000
    n_path = 3000
    n = 1 + n_hub + n_path
    adj = [[] for _ in range(n)]
    adj[0] = list(range(1, n_hub + 1))
    for v in range(1, n_hub + 1):
        adj[v].append(0)
    adj[n_hub].append(n_hub + 1)
    for i in range(n_hub + 1, n - 1):
        adj[i].append(i + 1)
        adj[i + 1].append(i)
    indptr = np.zeros(n + 1, np.uint32)
    indptr[1:] = np.cumsum([len(a) for a in adj])
    inds = np.array([v for a in adj for v in sorted(set(a))], np.uint32)
    g = B.Csc(indptr, inds)
    dg = B.Graph.upload(g)
    ref, ec = O.oracle_bfs_queue(indptr, inds, 0)
    assert ref.max() > 3000
    for lb, blk in ARMS:
        for loop in ("graph", "host"):
            lv, _, st = dg.run(0, B.options(lb, blk, loop=loop))
            assert np.array_equal(lv, ref), (lb, blk, loop)
            assert st.edges_count == ec
    dg.free()


def test_device_generator_equals_host_generator(B):
    torch_cuda()
    for scale, ef, sym in ((12, 16, True), (15, 8, False), (16, 16, True)):
        h = B.gen_rmat(scale, ef, seed=scale, symmetrize=sym)
        d = B.Graph.gen_rmat_device(scale, ef, seed=scale, symmetrize=sym)
        dh = d.download()
        assert np.array_equal(h.indptr, dh.indptr) and np.array_equal(h.inds, dh.inds)
        d.free()


def test_repeated_runs_bit_identical(B):
    """All runs of one root agree (areAllRowsEqualToLast, functions.hpp:131)."""
    torch_cuda()
    g = B.gen_rmat(16, 16, seed=3)
    dg = B.Graph.upload(g)
    r = int(B.sample_roots(g, 1, 3)[0])
    first, _, _ = dg.run(r)
    for lb, blk in ARMS:
        for _ in range(3):
            lv, _, _ = dg.run(r, B.options(lb, blk))
            assert np.array_equal(lv, first)
    dg.free()


def _check_config(B, O, g, roots, arms, queue_form=False, threads=None):
    dg = B.Graph.upload(g, validate=True)
    for chunk in range(0, len(roots), 16):
        rs = roots[chunk:chunk + 16]
        ref, ec = O.oracle_bfs_many(g.indptr, g.inds, rs, n_threads=threads,
                                    queue_form=queue_form)
        for lb, blk in arms:
            o = B.options(lb, blk)
            for i, r in enumerate(rs):
                lv, _, st = dg.run(int(r), o)
                assert np.array_equal(lv, ref[i]), (lb, blk, int(r))
                assert st.edges_count == int(ec[i])
    dg.free()


def test_config1_rmat19_llb_20_roots(B, O):
    torch_cuda()
    g = B.gen_rmat(19, 16, seed=1)
    _check_config(B, O, g, B.sample_roots(g, 20, 1), [("llb", 256)])


def test_config2_rmat23_every_arm_64_roots(B, O):
    torch_cuda()
    dg = B.Graph.gen_rmat_device(23, 16, seed=2)
    g = dg.download()
    dg.free()
    assert 200_000_000 < g.nnz < 280_000_000
    _check_config(B, O, g, B.sample_roots(g, 64, 2), ARMS)


def test_config3a_grid4096_32_roots(B, O):
    torch_cuda()
    g = B.gen_grid(4096, 4096, 0.05, 3)
    _check_config(B, O, g, B.sample_roots(g, 32, 3), [("llb", 256), ("glb", 256),
                                                     ("slb", 128)], queue_form=True)


def test_config3b_er22_32_roots(B, O):
    torch_cuda()
    g = B.gen_er(1 << 22, 16.0, 4)
    _check_config(B, O, g, B.sample_roots(g, 32, 4), ARMS)


def test_rmat25_full_size(B, O):
    """Held-out RMAT-25/EF16 (seed 5): oracle bit-exact on one root, and for
    more roots the size-independent checks (device validator, all arms equal)."""
    torch = torch_cuda()
    dg = B.Graph.gen_rmat_device(25, 16, seed=5)
    roots = None
    lv = torch.empty(dg.n_cols, dtype=torch.int32, device="cuda")
    pa = torch.empty(dg.n_cols, dtype=torch.int32, device="cuda")
    g = dg.download()
    roots = B.sample_roots(g, 3, 5)
    ref, ec = O.oracle_bfs_queue(g.indptr, g.inds, int(roots[0]))
    for lb, blk in ARMS:
        st = dg.run_device(int(roots[0]), lv.data_ptr(), None, B.options(lb, blk))
        torch.cuda.synchronize()
        assert np.array_equal(lv.cpu().numpy(), ref), (lb, blk)
        assert st.edges_count == ec
    for r in roots[1:]:
        first = None
        for lb, blk in (("llb", 256), ("glb", 512), ("slb", 256)):
            st = dg.run_device(int(r), lv.data_ptr(), pa.data_ptr(), B.options(lb, blk))
            assert dg.validate_device(int(r), lv.data_ptr(), pa.data_ptr()) == 0
            cur = lv.cpu().numpy()
            if first is None:
                first = cur
            assert np.array_equal(cur, first)
    dg.free()


def test_pinned_host_outputs(B, O):
    """bfs_run into pinned host buffers and into pageable ones: same levels
    and parents, twice; and into a pinned buffer at an odd offset."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g = B.gen_rmat(15, 16, seed=41)
    dg = B.Graph.upload(g)
    n = g.n_cols
    for r in B.sample_roots(g, 2, 41):
        ref, ec = O.oracle_bfs(g.indptr, g.inds, int(r))
        for rep in range(2):
            lv_p = torch.full((n,), 7, dtype=torch.int32, pin_memory=True)
            pa_p = torch.full((n,), 7, dtype=torch.int32, pin_memory=True)
            st = dg.run_into(int(r), lv_p.data_ptr(), pa_p.data_ptr())
            assert np.array_equal(lv_p.numpy(), ref) and st.edges_count == ec
            lv, pa, _ = dg.run(int(r), parents=True)
            assert np.array_equal(lv, ref)
            pp = pa_p.numpy()
            kids = np.flatnonzero(ref > 0)
            assert np.all(ref[pp[kids]] == ref[kids] - 1) and pp[int(r)] == int(r)
        # an odd-sized tail: a pinned buffer offset by one element
        big = torch.full((n + 1,), 7, dtype=torch.int32, pin_memory=True)
        dg.run_into(int(r), big.data_ptr() + 4)
        assert np.array_equal(big.numpy()[1:], ref) and big[0].item() == 7
    dg.free()


def test_run_roots_pinned_and_pageable(B, O):
    """bfs_run_roots: several roots in one call, each run's levels (and
    parents) in its own host buffer -- pinned (copies overlap the next run)
    and pageable (serial) -- equal to the oracle; a bad root anywhere in the
    list is refused before any run."""
    torch = torch_cuda()
    g = B.gen_rmat(14, 16, seed=43)
    dg = B.Graph.upload(g)
    n = g.n_cols
    roots = [int(r) for r in B.sample_roots(g, 4, 43)]
    roots = roots + [roots[0]]  # a root repeated, as the reference's num_runs loop does
    refs = [O.oracle_bfs(g.indptr, g.inds, r) for r in roots]
    w = np.random.default_rng(43).normal(0, 1.0, B.SCHED_PARAMS).astype(np.float32)
    dg.sched_attach(w)  # random weights: arbitrary arms per level
    for learned in (False, True):
        opts = B.options("learned") if learned else B.options("glb", 256)
        lv = [torch.full((n,), 7, dtype=torch.int32, pin_memory=True) for _ in roots]
        pa = [torch.full((n,), 7, dtype=torch.int32, pin_memory=True) for _ in roots]
        sts = dg.run_roots(roots, [t.data_ptr() for t in lv], [t.data_ptr() for t in pa], opts)
        for r, (ref, ec), st, l, p in zip(roots, refs, sts, lv, pa):
            assert np.array_equal(l.numpy(), ref) and st.edges_count == ec
            pp = p.numpy()
            kids = np.flatnonzero(ref > 0)
            assert np.all(ref[pp[kids]] == ref[kids] - 1) and pp[r] == r
    hv = [np.full(n, 7, np.int32) for _ in roots]
    sts = dg.run_roots(roots, [a.ctypes.data for a in hv])
    for (ref, ec), st, a in zip(refs, sts, hv):
        assert np.array_equal(a, ref) and st.edges_count == ec
    # one root; then none
    one = np.full(n, 7, np.int32)
    dg.run_roots(roots[1:2], [one.ctypes.data])
    assert np.array_equal(one, refs[1][0])
    assert dg.run_roots([], []) == []
    bad = [np.full(n, 7, np.int32) for _ in range(3)]
    with pytest.raises(B.BfsError):
        dg.run_roots([roots[0], n, roots[1]], [a.ctypes.data for a in bad])
    assert all(np.all(a == 7) for a in bad)
    dg.free()


def test_sparse_level_generation_slice_overflow(B, O):
    """After a level with few edges, level generation runs per warp: warp g
    takes the 32-word groups g, g + G, g + 2G, ... (G warps: 3 blocks of 8 per
    SM) into a 1024-entry slice and flushes it when the next group would not
    fit.  A root whose 2048 out-edges fill groups 0 and G (every vertex new,
    2048 edges < words / 8) makes warp 0 flush between its groups; levels and
    edge counts stay exact, in both loops and every arm."""
    torch = torch_cuda()
    G = torch.cuda.get_device_properties(0).multi_processor_count * 3 * 8
    n = max((G + 1) * 1024 * 4, 1 << 22)
    targets = np.concatenate([np.arange(0, 1024), np.arange(G * 1024, G * 1024 + 1024)])
    root = n - 1
    # root -> targets; every target -> root + a second hop to a fresh vertex
    second = (targets + 2 * G * 1024 + 5) % (n - 1)
    src = np.concatenate([np.full(len(targets), root), targets, targets])
    dst = np.concatenate([targets, np.full(len(targets), root), second])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    keep = np.ones(len(src), bool)
    keep[1:] = (src[1:] != src[:-1]) | (dst[1:] != dst[:-1])
    src, dst = src[keep], dst[keep]
    indptr = np.zeros(n + 1, np.uint32)
    indptr[1:] = np.cumsum(np.bincount(src, minlength=n))
    g = B.Csc(indptr, dst.astype(np.uint32))
    dg = B.Graph.upload(g)
    ref, ec = O.oracle_bfs(g.indptr, g.inds, root)
    assert (ref == 1).sum() == 2048
    for lb, blk in (("llb", 256), ("glb", 256), ("slb", 128), ("learned", 256)):
        for loop in ("graph", "host"):
            lv, _, st = dg.run(root, B.options(lb, blk, loop=loop))
            assert np.array_equal(lv, ref), (lb, loop)
            assert st.edges_count == ec
    dg.free()
