"""Out-of-memory paths, reached without filling the device: the engine's
allocation hook (BFS_GB300_FAIL_ALLOC_BYTES=N fails every device request of
N bytes or more).  Each failing call reports BFS_ERR_OOM and leaves nothing
half-built; a handle stays usable after one of its calls ran out of memory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HOOK = "BFS_GB300_FAIL_ALLOC_BYTES"


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def expect_oom(B, fn):
    with pytest.raises(B.BfsError) as e:
        fn()
    assert e.value.status == "BFS_ERR_OOM", e.value


def test_allocation_failures_are_reported(B, O, monkeypatch):
    torch = torch_cuda()
    g = B.gen_rmat(14, 16, seed=47)
    n = g.n_cols
    # every device allocation fails
    monkeypatch.setenv(HOOK, "1")
    expect_oom(B, lambda: B.Graph.upload(g))
    expect_oom(B, lambda: B.Graph.gen_rmat_device(12, 8, seed=1))
    expect_oom(B, lambda: B.MultiBatch([g]))
    monkeypatch.delenv(HOOK)

    dg = B.Graph.upload(g)
    roots = [int(r) for r in B.sample_roots(g, 3, 47)]
    ref, rec = O.oracle_bfs_many(g.indptr, g.inds, roots)
    out = torch.full((len(roots), n), 7, dtype=torch.int32, device="cuda")
    # the batched workspace (18 masks of 8 bytes per vertex) cannot be had;
    # single-root runs, which need 4 bytes per vertex at a time, go on
    monkeypatch.setenv(HOOK, str(64 * n))
    expect_oom(B, lambda: dg.run_batch(roots, out.data_ptr()))
    lv, _, st = dg.run(roots[0])
    assert np.array_equal(lv, ref[0]) and st.edges_count == rec[0]
    hv = [np.full(n, 7, np.int32) for _ in roots]
    sts = dg.run_roots(roots, [a.ctypes.data for a in hv])
    for a, r, e, s in zip(hv, ref, rec, sts):
        assert np.array_equal(a, r) and s.edges_count == e
    # the limit lifted, the same handle runs the batch
    monkeypatch.delenv(HOOK)
    ec, _ = dg.run_batch(roots, out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), ref) and np.array_equal(ec, rec)
    dg.free()
