"""The C-ABI library loads and exports every function include/*.h declares."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT, has_gpu


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(bfs_\w+)\s*\(", text,
                             flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("bfs_graph_upload", "bfs_run", "bfs_run_roots", "bfs_run_device", "bfs_graph_free",
              "bfs_dataset_load", "bfs_gen_rmat_host", "bfs_validate_device"):
        assert n in names


def test_library_exports_every_declared_symbol(B):
    lib = C.CDLL(B.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_status_strings_and_defaults(B):
    L = B.lib()
    assert L.bfs_abi_version() == 1
    assert L.bfs_status_string(0) == b"ok"
    assert L.bfs_status_string(7) == b"level limit exceeded"
    o = B.options()
    assert (o.lb, o.block, o.loop, o.l2_pin) == (0, 256, 0, 1)


def test_upload_without_gpu_fails_cleanly(B):
    if has_gpu():
        pytest.skip("a GPU is present")
    g = B.gen_grid(4, 4, 0.0, 1)
    with pytest.raises(B.BfsError) as e:
        B.Graph.upload(g)
    assert e.value.status == "BFS_ERR_NO_DEVICE"


def test_argument_errors_without_gpu(B):
    L = B.lib()
    h = B.VP()
    # null pointers and bad sizes are rejected before any device work
    assert L.bfs_graph_upload(None, None, 1, 1, 0, 0, C.byref(h)) == 1
    import numpy as np
    ip = np.zeros(3, np.uint32)
    assert L.bfs_graph_upload(ip.ctypes.data_as(B.U32P), ip.ctypes.data_as(B.U32P), 3, 2, 0, 0,
                              C.byref(h)) == 1  # n_rows > n_cols
    assert L.bfs_run(None, 0, None, None, None, None) == 1
    assert L.bfs_run_roots(None, None, 0, None, None, None, None) == 1
    roots = np.zeros(2, np.uint32)
    assert L.bfs_run_roots(None, roots.ctypes.data_as(B.U32P), 2, None, None, None, None) == 1
