"""The reference-compatible command line driver (src/host.cpp surface) and its
JSON report (src/host.cpp:192-271, run_bfs_gpu.hpp:784-790)."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import PKG, ROOT, has_gpu

CLI = os.path.join(PKG, "bin", "bfs_gb300")


def run_cli(args, cwd):
    return subprocess.run([CLI] + args, cwd=cwd, capture_output=True, text=True,
                          env=dict(os.environ, PWD=str(cwd)), timeout=300)


def test_json_header_round_trip(tmp_path):
    exe = tmp_path / "jrt"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "json_roundtrip.cpp"), "-o", str(exe)],
                   check=True)
    src = {"b": [1, 2, {"x": None, "y": True}], "a": 0.1, "s": "tést", "n": -7}
    r = subprocess.run([str(exe)], input=json.dumps(src), capture_output=True, text=True,
                       check=True)
    out = json.loads(r.stdout)
    assert out["b"] == src["b"] and out["a"] == 0.1 and out["s"] == src["s"] and out["n"] == -7
    assert out["added"]["nested"] == [1.5, 2.0, -3.25e-7]
    assert out["added"]["count"] == 18446744073709551615
    assert out["added"]["text"] == 'a"b\\c\n'
    assert r.stdout.splitlines()[1].startswith("    ")  # 4-space indent, like dump(4)
    assert list(out.keys()) == sorted(out.keys())


def test_cli_arguments_and_loader_errors(B, tmp_path):
    r = run_cli(["--dataset", "missing", "--bogus=1", "--root"], tmp_path)
    assert r.returncode == 1
    assert "Warning: No value provided for argument --root" in r.stderr
    assert "file not found" in r.stderr
    g = B.gen_rmat(9, 8, seed=1)
    B.dataset_write(g, "small", 1, str(tmp_path / "dataset"))
    r = run_cli(["--dataset=small", "--num_runs", "2", "--root=3"], tmp_path)
    out = r.stdout
    assert "- dataset" in out and "Load [OK]" in out
    assert re.search(rf"- # vertices\s+{g.n_cols}\b", out)
    if not has_gpu():
        assert r.returncode == 1 and "no CUDA device" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("lb,key", [("llb", "local"), ("glb", "global"), ("slb", "local_strided"),
                                    ("learned", "learned")])
def test_cli_report_matches_oracle(B, O, tmp_path, lb, key):
    g = B.gen_rmat(13, 16, seed=21)
    B.dataset_write(g, "rm", 1, str(tmp_path / "dataset"))
    root = int(B.sample_roots(g, 1, 21)[0])
    r = run_cli([f"--dataset=rm", f"--root={root}", "--num_runs=5", f"--lb={lb}"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert "[SUCCESS]" in r.stdout
    rep = json.load(open(tmp_path / "data.json"))
    obj = rep[f"rm_5_{key}"]["1"]
    lv, ec = O.oracle_bfs(g.indptr, g.inds, root)
    assert obj["edgesCount"] == ec and obj["valid"] is True and obj["startVertex"] == root
    assert obj["numLevels"] == int(lv.max()) + 1
    assert obj["LevelsGPU"] == [int((lv == i).sum()) for i in range(int(lv.max()) + 1)]
    assert len(obj["rawExecutionTimeAll"]) == 5
    for k in ("avgExecutionTime", "avgExecutionTimeFiltered", "minExecutionTimeFiltered",
              "avgExecutionTime90f", "minExecutionTime90f", "totalExecutionTime", "avgMTEPS",
              "avgMTEPS90f", "avgMTEPSFilter", "maxMTEPSFilter", "edgesCoverage"):
        assert obj[k] > 0, k
    assert isinstance(obj["avgGTEPS90f"], str)
    assert abs(obj["edgesCoverage"] - 100.0 * ec / g.nnz) < 1e-9


@pytest.mark.gpu
def test_cli_partitions_and_merge(B, O, tmp_path):
    g = B.gen_rmat(12, 8, seed=4, symmetrize=False)
    for P in (1, 3):
        B.dataset_write(g, "mp", P, str(tmp_path / "dataset"))
    root = int(B.sample_roots(g, 1, 4)[0])
    for P in (1, 3):
        r = run_cli(["--dataset=mp", f"--root={root}", f"--partitions={P}", "--lb=glb"], tmp_path)
        assert r.returncode == 0, r.stderr
    rep = json.load(open(tmp_path / "data.json"))
    lv, ec = O.oracle_bfs(g.indptr, g.inds, root)
    for P in ("1", "3"):
        obj = rep["mp_1_global"][P]
        assert obj["edgesCount"] == ec and obj["valid"] is True


@pytest.mark.gpu
def test_cli_batch_option(B, O, tmp_path):
    """--batch K runs the root and K - 1 seeded roots as 64-root passes; the
    root's row and edge count agree with the single-root runs."""
    g = B.gen_rmat(13, 16, seed=22)
    B.dataset_write(g, "rb", 1, str(tmp_path / "dataset"))
    root = int(B.sample_roots(g, 1, 22)[0])
    r = run_cli(["--dataset=rb", f"--root={root}", "--num_runs=2", "--lb=glb", "--batch=70"],
                tmp_path)
    assert r.returncode == 0, r.stderr
    obj = json.load(open(tmp_path / "data.json"))["rb_2_global"]["1"]
    lv, ec = O.oracle_bfs(g.indptr, g.inds, root)
    assert obj["batchRoots"] == 70 and obj["batchValid"] is True
    assert obj["batchMs"] > 0 and obj["batchRootsPerSec"] > 0
    assert obj["batchMaxLevels"] >= int(lv.max()) + 1
    assert obj["edgesCount"] == ec
    r = run_cli(["--dataset=rb", f"--root={root}", "--batch=-1"], tmp_path)
    assert r.returncode == 1
