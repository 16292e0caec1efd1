"""Seeded synthetic graphs (host builders): determinism, CSC invariants."""
import numpy as np
import pytest


def csc_ok(g):
    assert g.indptr[0] == 0 and int(g.indptr[-1]) == g.nnz
    assert np.all(np.diff(g.indptr.astype(np.int64)) >= 0)
    assert g.nnz == 0 or int(g.inds.max()) < g.n_cols
    for v in range(min(g.n_cols, 4096)):
        s = g.inds[g.indptr[v]:g.indptr[v + 1]]
        assert np.all(np.diff(s.astype(np.int64)) > 0), "sorted, no duplicates"
        assert not np.any(s == v), "no self-loops"


def is_symmetric(g):
    src = np.repeat(np.arange(g.n_cols, dtype=np.int64), np.diff(g.indptr.astype(np.int64)))
    a = set(zip(src.tolist(), g.inds.astype(np.int64).tolist()))
    return all((v, u) in a for (u, v) in a)


def test_rmat_deterministic_and_valid(B):
    a = B.gen_rmat(11, 16, seed=1)
    b = B.gen_rmat(11, 16, seed=1)
    c = B.gen_rmat(11, 16, seed=2)
    assert np.array_equal(a.indptr, b.indptr) and np.array_equal(a.inds, b.inds)
    assert not np.array_equal(a.inds, c.inds)
    csc_ok(a)
    assert is_symmetric(a)
    # R-MAT skew: vertex 0 is the hub (a = 0.57)
    assert int(np.argmax(a.degree())) == 0
    assert a.nnz < 2 * 16 * 2048


def test_rmat_directed_not_symmetrized(B):
    g = B.gen_rmat(10, 8, seed=3, symmetrize=False)
    csc_ok(g)
    assert not is_symmetric(g)
    assert g.nnz <= 8 * 1024


def test_rmat19_size_matches_survey_probe(B):
    g = B.gen_rmat(19, 16, seed=1)
    # deduplicated + symmetrised RMAT-19/EF16 has ~15.5M directed entries
    assert 15_000_000 < g.nnz < 16_000_000
    assert g.n_cols == 1 << 19


def test_grid(B):
    g = B.gen_grid(40, 30, 0.05, 3)
    csc_ok(g)
    assert is_symmetric(g)
    full = 2 * (39 * 30 + 40 * 29)
    assert 0.85 * full < g.nnz < full
    g0 = B.gen_grid(8, 8, 0.0, 3)
    assert g0.nnz == 2 * (7 * 8 + 8 * 7)
    assert g0.inds[g0.indptr[9]:g0.indptr[10]].tolist() == [1, 8, 10, 17]


def test_er(B):
    g = B.gen_er(4096, 16.0, 4)
    csc_ok(g)
    assert is_symmetric(g)
    assert abs(g.nnz / 4096 - 16.0) < 0.5


def test_roots(B):
    g = B.gen_rmat(10, 16, seed=1)
    r = B.sample_roots(g, 20, 5)
    assert len(set(r.tolist())) == 20
    assert np.all(g.degree()[r] > 0)
    assert np.array_equal(r, B.sample_roots(g, 20, 5))
    with pytest.raises(B.BfsError) as e:
        B.sample_roots(B.gen_grid(2, 1, 1.0, 0), 1, 0)
    assert e.value.status == "BFS_ERR_GRAPH"


def test_bad_generator_args(B):
    with pytest.raises(B.BfsError):
        B.gen_rmat(0, 16)
    with pytest.raises(B.BfsError):
        B.gen_rmat(10, 16, a=0.9, b=0.2, c=0.1)
    with pytest.raises(B.BfsError):
        B.gen_grid(0, 5)
