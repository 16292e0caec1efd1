"""bfs_run_device_noalloc: the BFS entry point for callers that cannot
allocate device memory (code inside an allocator or pool callback, processes
under a fixed device-memory budget, plugins that may not allocate after
start-up).  It keeps its workspace in a fixed device array inside the
library, so its results must equal those of the regular entry point
bfs_run_device, call after call, even though every call reuses the array
left over from the previous one.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test; it also passes on its own in a
fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def noalloc_fn(B):
    f = B.lib().bfs_run_device_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                  C.c_void_p, C.POINTER(C.c_uint64), C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_matches_regular_entry_point_two_calls(B, O):
    torch = torch_cuda()
    f = noalloc_fn(B)
    g = B.gen_rmat(17, 16, seed=31)
    assert g.n_cols <= (1 << 20)
    dg = B.Graph.upload(g)
    d_indptr, d_inds = dg.device_csc()
    roots = B.sample_roots(g, 2, 31)
    ref_lv = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    out = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    # two calls in a row: the second reuses the first call's scratch contents
    for r in (roots[0], roots[1], roots[0]):
        st = dg.run_device(int(r), ref_lv.data_ptr(), opts=B.options("glb", 256))
        out.fill_(12345)
        edges = C.c_uint64(0)
        rc = f(d_indptr, d_inds, g.n_rows, g.n_cols, g.nnz, int(r), out.data_ptr(),
               C.byref(edges), None)
        assert rc == 0, B.lib().bfs_last_error()
        torch.cuda.synchronize()
        # integer results: bit-exact (the tolerance is zero)
        assert torch.equal(out, ref_lv)
        assert edges.value == st.edges_count
    # and against the oracle once
    lv, ec = O.oracle_bfs(g.indptr, g.inds, int(roots[0]))
    assert np.array_equal(out.cpu().numpy(), lv) and edges.value == ec
    dg.free()


def test_noalloc_on_a_stream_and_rows_lt_cols(B, O):
    torch = torch_cuda()
    f = noalloc_fn(B)
    # rows < cols: vertex ids >= n_rows are reached but never expanded
    g = B.gen_rmat(12, 8, seed=5)
    n_rows = g.n_cols - 100
    ip = torch.tensor(g.indptr.astype(np.int64), dtype=torch.int64).to(torch.int32).cuda()
    ix = torch.tensor(g.inds.astype(np.int64), dtype=torch.int64).to(torch.int32).cuda()
    out = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    for r in B.sample_roots(B.Csc(g.indptr, g.inds, n_rows, g.n_cols), 2, 2):
        edges = C.c_uint64(0)
        rc = f(ip.data_ptr(), ix.data_ptr(), n_rows, g.n_cols, g.nnz, int(r), out.data_ptr(),
               C.byref(edges), C.c_void_p(s.cuda_stream))
        assert rc == 0, B.lib().bfs_last_error()
        s.synchronize()
        lv, ec = O.oracle_bfs(g.indptr, g.inds, int(r), n_rows, g.n_cols)
        assert np.array_equal(out.cpu().numpy(), lv) and edges.value == ec


def test_noalloc_rejects_oversized_and_bad_input(B):
    torch_cuda()
    f = noalloc_fn(B)
    out = C.c_void_p(1)  # never dereferenced: the call fails before any launch
    rc = f(C.c_void_p(1), C.c_void_p(1), (1 << 20) + 1, (1 << 20) + 1, 10, 0, out, None, None)
    assert rc == 1
    msg = B.lib().bfs_last_error().decode()
    assert "at most 1048576 vertices" in msg
    assert f(None, None, 4, 4, 0, 0, out, None, None) == 1
    assert f(C.c_void_p(1), C.c_void_p(1), 4, 4, 0, 9, out, None, None) == 2  # root


def test_noalloc_takes_no_device_memory_after_warmup(B, O, monkeypatch):
    """The property the entry point exists for: once a warm-up call has
    loaded the library's device code and array on this device, further calls
    leave the device's free memory unchanged, and they still succeed when
    every allocation through the engine's allocation hook is made to fail."""
    torch = torch_cuda()
    f = noalloc_fn(B)
    g = B.gen_rmat(15, 16, seed=8)
    ip = torch.from_numpy(g.indptr.view(np.int32)).cuda()
    ix = torch.from_numpy(g.inds.view(np.int32)).cuda()
    out = torch.empty(g.n_cols, dtype=torch.int32, device="cuda")
    roots = B.sample_roots(g, 3, 8)
    edges = C.c_uint64(0)
    assert f(ip.data_ptr(), ix.data_ptr(), g.n_rows, g.n_cols, g.nnz, int(roots[0]),
             out.data_ptr(), C.byref(edges), None) == 0  # warm-up
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    monkeypatch.setenv("BFS_GB300_FAIL_ALLOC_BYTES", "1")
    for r in roots[1:]:
        rc = f(ip.data_ptr(), ix.data_ptr(), g.n_rows, g.n_cols, g.nnz, int(r), out.data_ptr(),
               C.byref(edges), None)
        assert rc == 0, B.lib().bfs_last_error()
        lv, ec = O.oracle_bfs(g.indptr, g.inds, int(r))
        assert np.array_equal(out.cpu().numpy(), lv) and edges.value == ec
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
