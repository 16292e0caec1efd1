"""Pins the oracle (CPU restatement of src/run_bfs_cpu.hpp:5-85) to the
reference: golden fixtures made by the reference's own run_bfs_cpu, and the
compiled reference itself where the reference tree exists."""
import numpy as np
import pytest


def single_cases(cases):
    return {k: v for k, v in cases.items() if "parts" not in v}


def test_golden_cases_present(cases):
    assert len(single_cases(cases)) >= 10
    assert any("parts" in v for v in cases.values())


def test_oracle_matches_golden(cases, O):
    for name, c in single_cases(cases).items():
        for i, r in enumerate(c["roots"]):
            lv, ec = O.oracle_bfs(c["indptr"], c["inds"], int(r), int(c["n_rows"]),
                                  int(c["n_cols"]))
            assert np.array_equal(lv, c["levels"][i]), (name, int(r))
            assert ec == int(c["edges"][i]), (name, int(r))


def test_queue_oracle_matches_golden(cases, O):
    for name, c in single_cases(cases).items():
        for i, r in enumerate(c["roots"]):
            lv, ec = O.oracle_bfs_queue(c["indptr"], c["inds"], int(r), int(c["n_rows"]),
                                        int(c["n_cols"]))
            assert np.array_equal(lv, c["levels"][i]), (name, int(r))
            assert ec == int(c["edges"][i]), (name, int(r))


def test_oracle_many_matches_single(cases, O):
    c = cases["rmat10_ef16_s1"]
    for qf in (False, True):
        lv, ec = O.oracle_bfs_many(c["indptr"], c["inds"], c["roots"], n_threads=3,
                                   queue_form=qf)
        assert np.array_equal(lv, c["levels"])
        assert np.array_equal(ec, c["edges"])


def test_multi_partition_oracle_matches_golden(cases, O):
    for name, c in cases.items():
        if "parts" not in c:
            continue
        P = int(c["parts"])
        ips = [c[f"indptr{p}"] for p in range(P)]
        ixs = [c[f"inds{p}"] for p in range(P)]
        for i, r in enumerate(c["roots"]):
            lv, ec = O.oracle_bfs_multi(ips, ixs, int(r), int(c["n_rows"]), int(c["n_cols"]))
            assert np.array_equal(lv, c["levels"][i]), (name, int(r))
            assert ec == int(c["edges"][i])


def test_known_answers(cases):
    """Hand-checked levels of the known-answer graphs."""
    p = cases["path5"]
    assert p["levels"][0].tolist() == [0, 1, 2, 3, -1]
    assert int(p["edges"][0]) == 6
    assert p["levels"][2].tolist() == [-1, -1, -1, -1, 0]  # isolated root
    s = cases["star7"]
    assert s["levels"][1].tolist() == [1, 2, 2, 0, 2, 2, 2]
    d = cases["dcycle10"]
    assert d["levels"][0].tolist() == list(range(10))
    # rows < cols: vertex 5 is reached but never expanded; a root >= rows
    # expands nothing (run_bfs_cpu.hpp:31)
    rl = cases["rows_lt_cols"]
    assert rl["levels"][0].tolist() == [0, 1, -1, -1, -1, 2]
    assert rl["levels"][1].tolist() == [-1, -1, -1, -1, -1, 0]
    assert int(rl["edges"][1]) == 0
    e = cases["empty"]
    assert e["levels"][0].tolist() == [0, -1, -1, -1]
    assert int(e["edges"][0]) == 0


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_compiled_reference(O, B, seed):
    if not O.ref_available():
        pytest.skip("reference tree not present: oracle pinned by the golden fixtures only")
    g = B.gen_rmat(12, 8, seed=seed, symmetrize=bool(seed % 2))
    for r in B.sample_roots(g, 4, seed):
        a = O.oracle_bfs(g.indptr, g.inds, int(r))
        b = O.ref_bfs([g.indptr], [g.inds], int(r), g.n_rows, g.n_cols)
        assert np.array_equal(a[0], b[0]) and a[1] == b[1]


def test_oracle_rejects_bad_graph(O):
    with pytest.raises(ValueError):
        O.oracle_bfs(np.array([0, 2, 1], np.uint32), np.array([0, 1], np.uint32), 0)
    with pytest.raises(ValueError):
        O.oracle_bfs(np.array([0, 1, 1], np.uint32), np.array([7], np.uint32), 0)
    with pytest.raises(ValueError):
        O.oracle_bfs(np.array([0, 1, 1], np.uint32), np.array([1], np.uint32), 5)
