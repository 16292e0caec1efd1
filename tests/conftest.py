import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bfs-gpu-sycl_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    import build as pkg_build  # bfs-gpu-sycl_gb300/build.py
    pkg_build.build(verbose=False)
    import bfs_oracle
    bfs_oracle.build()  # make rebuilds only what changed


_ensure_built()


@pytest.fixture(scope="session")
def B():
    import bfs_gb300
    return bfs_gb300


@pytest.fixture(scope="session")
def O():
    import bfs_oracle
    return bfs_oracle


GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_cases():
    """Golden BFS cases produced by the reference's own run_bfs_cpu."""
    z = np.load(os.path.join(GOLDEN, "bfs_cases.npz"))
    cases = {}
    for key in z.files:
        c, k = key.split("__", 1)
        cases.setdefault(c, {})[k] = z[key]
    return cases


@pytest.fixture(scope="session")
def cases():
    return load_cases()


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
