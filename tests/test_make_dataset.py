"""make_dataset.py: the scripts/genGraph.py + generator.py counterpart."""
import os
import subprocess
import sys

import numpy as np

from conftest import PKG

TOOL = os.path.join(PKG, "make_dataset.py")


def test_edgelist_conversion(B, O, tmp_path):
    txt = tmp_path / "g.txt"
    # duplicates merge, self-loops stay, comments skipped, weights ignored
    txt.write_text("# comment\n0\t1\t1\n0\t1\t1\n1\t2\t1\n2\t2\t1\n3\t0\t1\n% other\n")
    r = subprocess.run([sys.executable, TOOL, "edgelist", str(txt), "--dir", str(tmp_path / "ds"),
                        "--partitions", "1", "2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = B.dataset_load("g", 1, str(tmp_path / "ds"))
    assert g.n_cols == 4 and g.nnz == 4
    assert g.indptr.tolist() == [0, 1, 2, 3, 4]
    assert g.inds.tolist() == [1, 2, 2, 0]
    h = B.dataset_load("g", 2, str(tmp_path / "ds"))
    assert np.array_equal(O.oracle_bfs(g.indptr, g.inds, 3)[0],
                          O.oracle_bfs(h.indptr, h.inds, 3)[0])


def test_generated_datasets(B, tmp_path):
    for args, name in ((["rmat", "10", "8"], "rmat-10-8"), (["grid", "16", "8"], "grid-16x8"),
                       (["er", "500", "6"], "er-500-6")):
        r = subprocess.run([sys.executable, TOOL] + args + ["--dir", str(tmp_path)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        g = B.dataset_load(name, 1, str(tmp_path))
        assert g.nnz > 0 and int(g.indptr[-1]) == g.nnz
    ref = B.gen_rmat(10, 8, seed=1)
    g = B.dataset_load("rmat-10-8", 1, str(tmp_path))
    assert np.array_equal(g.indptr, ref.indptr) and np.array_equal(g.inds, ref.inds)


def _golden_files(z, key):
    meta = z[key + "/meta"].tobytes()
    parts = [(z[f"{key}/{i}/indptr"].tobytes(), z[f"{key}/{i}/inds"].tobytes())
             for i in range(len(meta) // 20)]
    return meta, parts


def test_reference_splits_byte_identical(B, tmp_path):
    """nnz / row splits against files written by the reference's own
    scripts/generator.py (tests/golden/make_split_golden.py), P = 1..8."""
    import make_dataset as M
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_splits.npz"))
    graphs = sorted({k.split("/")[0] for k in z.files})
    assert graphs == ["skew203", "tail300", "u59", "u61"]
    for gname in graphs:
        e = z[f"{gname}/edges"]
        txt = tmp_path / f"{gname}.txt"
        txt.write_text("".join(f"{u}\t{v}\n" for u, v in e))
        g = M.csc_from_edgelist(str(txt))
        for pick in ("nnz", "row"):
            for p in range(1, 9):
                d = tmp_path / pick
                B.dataset_write(g, gname, p, str(d), split=pick)
                pre = d / f"{gname}-csc-{p}" / f"{gname}-csc-"
                meta, parts = _golden_files(z, f"{gname}/{pick}/{p}")
                assert (pre.parent / (pre.name + "meta.bin")).read_bytes() == meta, (gname, pick, p)
                for i, (ip, ix) in enumerate(parts):
                    assert (pre.parent / f"{pre.name}{i}-indptr.bin").read_bytes() == ip
                    assert (pre.parent / f"{pre.name}{i}-inds.bin").read_bytes() == ix
                assert not (pre.parent / f"{pre.name}{len(parts)}-indptr.bin").exists()


def test_reference_split_cli_names(tmp_path):
    txt = tmp_path / "tiny.txt"
    txt.write_text("".join(f"{i}\t{(i * 7 + 3) % 40}\n" for i in range(40)))
    r = subprocess.run([sys.executable, TOOL, "edgelist", str(txt), "--dir", str(tmp_path),
                        "--split", "nnz", "--partitions", "1", "2"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "tiny-nnz-csc-2" / "tiny-nnz-csc-meta.bin").exists()
    # 40 rows: round8(40) = 40, every edge kept at P = 1
    meta = (tmp_path / "tiny-nnz-csc-1" / "tiny-nnz-csc-meta.bin").read_bytes()
    assert np.frombuffer(meta[:8], np.uint32).tolist() == [40, 40]
    assert np.frombuffer(meta[8:16], np.uint64)[0] == 40
