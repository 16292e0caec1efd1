"""Pins the oracle's R-MAT generator and root sampler (oracle/graph_gen_oracle.c)
to the engine's host builders, byte for byte.  bench.py's reference arm builds
its graph and roots with the oracle's copies, so that it never loads the engine
library; these tests are what makes that graph the engine's graph."""
import numpy as np
import pytest

import bfs_gb300 as B
import bfs_oracle as O


@pytest.mark.parametrize("scale", [10, 11, 12, 13, 14])
@pytest.mark.parametrize("symmetrize", [True, False])
def test_rmat_matches_engine(scale, symmetrize):
    seed = 100 + scale
    a = O.oracle_gen_rmat(scale, 16, seed=seed, symmetrize=symmetrize)
    b = B.gen_rmat(scale, 16, seed=seed, symmetrize=symmetrize)
    assert a.nnz == b.nnz
    assert np.array_equal(a.indptr, b.indptr)
    assert np.array_equal(a.inds, b.inds)


def test_rmat_other_params_and_threads():
    # skewed quadrants, edge factor 8, one thread vs many: same bytes
    a1 = O.oracle_gen_rmat(12, 8, a=0.45, b=0.25, c=0.15, seed=9, threads=1)
    a4 = O.oracle_gen_rmat(12, 8, a=0.45, b=0.25, c=0.15, seed=9, threads=4)
    b = B.gen_rmat(12, 8, a=0.45, b=0.25, c=0.15, seed=9)
    for a in (a1, a4):
        assert np.array_equal(a.indptr, b.indptr)
        assert np.array_equal(a.inds, b.inds)


@pytest.mark.parametrize("seed", [0, 1, 5, 1005])
def test_roots_match_engine(seed):
    g = B.gen_rmat(13, 16, seed=3)
    for count in (1, 20, 400):
        assert np.array_equal(O.oracle_sample_roots(g.indptr, count, seed),
                              B.sample_roots(g, count, seed))


def test_roots_errors():
    indptr = np.array([0, 1, 1, 2], np.uint32)  # two vertices with out-edges
    assert sorted(O.oracle_sample_roots(indptr, 2, 1).tolist()) == [0, 2]
    with pytest.raises(ValueError):
        O.oracle_sample_roots(indptr, 3, 1)


def test_bad_parameters():
    with pytest.raises(ValueError):
        O.oracle_gen_rmat(0, 16)
    with pytest.raises(ValueError):
        O.oracle_gen_rmat(10, 16, a=0.6, b=0.3, c=0.3)
