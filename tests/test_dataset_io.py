"""The reference's binary CSC dataset layout (src/graph_load.hpp:7-132)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_reference_meta_files_parse(B):
    """The meta files shipped with the reference decode to the recorded facts."""
    facts = json.load(open(os.path.join(GOLDEN, "ref_dataset_facts.json")))
    for parts, f in facts.items():
        path = os.path.join(GOLDEN, "ref_meta", f"rmat-19-16-nnz-csc-{parts}-meta.bin")
        recs = B.dataset_read_meta(path)
        assert len(recs) == int(parts)
        for r, m in zip(recs, f["meta"]):
            assert r == (m["rows"], m["cols"], m["nnz"], m["start_row"])
    one = facts["1"]["meta"][0]
    # host.cpp:86-92 on the P=1 dataset: rows < cols because of round8
    assert (one["rows"], one["cols"], one["nnz"]) == (524176, 524177, 8388607)
    p0 = facts["1"]["partitions"][0]
    assert p0["indptr_len"] == one["cols"] + 1 and p0["indptr_last"] == one["nnz"]
    assert (p0["max_degree"], p0["argmax_degree"]) == (42514, 0)


def test_reference_dataset_loader_when_present(B):
    """Optional: point BFS_REFERENCE_DATASET at the reference's dataset folder.
    Its inds files are missing, so the loader must fail with an I/O error
    naming the missing file (readFromMM throws the same way)."""
    d = os.environ.get("BFS_REFERENCE_DATASET")
    if not d or not os.path.isdir(d):
        pytest.skip("BFS_REFERENCE_DATASET not set")
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("rmat-19-16-nnz", 1, d)
    assert e.value.status == "BFS_ERR_IO" and "inds.bin" in str(e.value)


@pytest.mark.parametrize("parts", [1, 2, 3, 4])
def test_write_load_round_trip(B, O, tmp_path, parts):
    g = B.gen_rmat(10, 8, seed=7, symmetrize=False)
    B.dataset_write(g, "rt", parts, str(tmp_path))
    folder = tmp_path / f"rt-csc-{parts}"
    files = sorted(os.listdir(folder))
    assert "rt-csc-meta.bin" in files
    for p in range(parts):
        assert f"rt-csc-{p}-indptr.bin" in files and f"rt-csc-{p}-inds.bin" in files
    meta = B.dataset_read_meta(str(folder / "rt-csc-meta.bin"))
    assert sum(m[0] for m in meta) == g.n_rows and all(m[1] == g.n_cols for m in meta)
    assert sum(m[2] for m in meta) == g.nnz
    assert [m[3] for m in meta] == list(np.cumsum([0] + [m[0] for m in meta[:-1]]))
    h = B.dataset_load("rt", parts, str(tmp_path))
    assert (h.n_rows, h.n_cols, h.nnz) == (g.n_rows, g.n_cols, g.nnz)
    # merged CSC keeps each vertex's neighbour set; BFS results are identical
    ips = [np.fromfile(folder / f"rt-csc-{p}-indptr.bin", np.uint32) for p in range(parts)]
    ixs = [np.fromfile(folder / f"rt-csc-{p}-inds.bin", np.uint32) for p in range(parts)]
    for r in B.sample_roots(g, 3, 1):
        a = O.oracle_bfs(g.indptr, g.inds, int(r))
        b = O.oracle_bfs(h.indptr, h.inds, int(r))
        c = O.oracle_bfs_multi(ips, ixs, int(r), g.n_rows, g.n_cols)
        assert np.array_equal(a[0], b[0]) and a[1] == b[1]
        assert np.array_equal(a[0], c[0]) and a[1] == c[1]
        if O.ref_available() and parts <= 4:
            d = O.ref_bfs(ips, ixs, int(r), g.n_rows, g.n_cols)
            assert np.array_equal(a[0], d[0]) and a[1] == d[1]


def test_pwd_default_directory(B, tmp_path, monkeypatch):
    g = B.gen_grid(5, 5, 0.0, 1)
    monkeypatch.setenv("PWD", str(tmp_path))
    B.dataset_write(g, "gridpwd", 1)
    assert (tmp_path / "dataset" / "gridpwd-csc-1" / "gridpwd-csc-0-inds.bin").exists()
    h = B.dataset_load("gridpwd", 1)
    assert np.array_equal(h.indptr, g.indptr) and np.array_equal(h.inds, g.inds)


def test_loader_errors(B, tmp_path):
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("nothing", 1, str(tmp_path))
    assert e.value.status == "BFS_ERR_IO"
    g = B.gen_grid(4, 4, 0.0, 1)
    B.dataset_write(g, "bad", 1, str(tmp_path))
    folder = tmp_path / "bad-csc-1"
    # empty inds file (graph_load.hpp:35-40 rejects size 0)
    open(folder / "bad-csc-0-inds.bin", "wb").close()
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("bad", 1, str(tmp_path))
    assert e.value.status == "BFS_ERR_IO"
    # truncated inds: offsets point past the end
    B.dataset_write(g, "bad", 1, str(tmp_path))
    ix = np.fromfile(folder / "bad-csc-0-inds.bin", np.uint32)
    ix[:-3].tofile(folder / "bad-csc-0-inds.bin")
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("bad", 1, str(tmp_path))
    assert e.value.status == "BFS_ERR_GRAPH"
    # destination out of range
    B.dataset_write(g, "bad", 1, str(tmp_path))
    ix = np.fromfile(folder / "bad-csc-0-inds.bin", np.uint32)
    ix[0] = 999
    ix.tofile(folder / "bad-csc-0-inds.bin")
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("bad", 1, str(tmp_path))
    assert e.value.status == "BFS_ERR_GRAPH"
    # non-monotone indptr
    B.dataset_write(g, "bad", 1, str(tmp_path))
    ip = np.fromfile(folder / "bad-csc-0-indptr.bin", np.uint32)
    ip[3], ip[4] = ip[4] + 1, ip[3]
    ip.tofile(folder / "bad-csc-0-indptr.bin")
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("bad", 1, str(tmp_path))
    assert e.value.status == "BFS_ERR_GRAPH"
    # incomplete meta record: ignored like the reference (no records -> error)
    with open(folder / "bad-csc-meta.bin", "wb") as f:
        f.write(b"\x01" * 12)
    with pytest.raises(B.BfsError) as e:
        B.dataset_load("bad", 1, str(tmp_path))
    assert e.value.status == "BFS_ERR_IO"
