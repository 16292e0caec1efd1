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
