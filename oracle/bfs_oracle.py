"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the parity checker.

  oracle_bfs*  -- liboracle.so, the C restatement of the reference CPU BFS
                  (src/run_bfs_cpu.hpp:5-85), see bfs_oracle.c
  ref_bfs      -- _ref/libref_bfs.so, the reference's own run_bfs_cpu compiled
                  in place by the Makefile (only where the reference exists)
  oracle_gen_rmat, oracle_sample_roots
               -- graph_gen_oracle.c, an independent restatement of the
                  engine's seeded R-MAT generator and root sampler, so that
                  the CPU baseline builds its inputs without the engine

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the engine never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_bfs.so")

U32P = C.POINTER(C.c_uint32)
I32P = C.POINTER(C.c_int32)
U64P = C.POINTER(C.c_uint64)

_lib = None
_ref = None


def build(quiet=True):
    """Builds liboracle.so and, where the reference tree exists, _ref/."""
    r = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if not quiet:
        print(r.stdout)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.oracle_bfs.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, U32P, U32P, C.c_uint32,
                                 I32P, U64P]
        L.oracle_bfs_many.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, U32P, U32P, U32P,
                                      C.c_uint32, C.c_int, C.c_int, I32P, U64P]
        L.oracle_bfs_queue.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, U32P, U32P,
                                       C.c_uint32, I32P, U64P]
        L.oracle_bfs_multi.argtypes = [C.c_uint32, C.c_uint32, C.c_int, C.POINTER(U32P),
                                       C.POINTER(U32P), U64P, C.c_uint32, I32P, U64P]
        L.oracle_gen_rmat.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                      C.c_double, C.c_uint64, C.c_int, C.c_int,
                                      C.POINTER(U32P), C.POINTER(U32P), U64P]
        L.oracle_sample_roots.argtypes = [U32P, C.c_uint32, C.c_uint32, C.c_uint64, U32P]
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_free.restype = None
        _lib = L
    return _lib


def ref_available():
    return os.path.exists(REF_LIB)


def _load_ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB)
        for p in (1, 2, 3, 4):
            f = getattr(R, f"ref_bfs_p{p}")
            f.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(U32P), C.POINTER(U32P), U64P,
                          C.c_uint32, I32P, U64P]
        _ref = R
    return _ref


def _arr(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def oracle_bfs(indptr, inds, root, n_rows=None, n_cols=None):
    """Returns (levels int32[n_cols], edges_count)."""
    ip = _arr(indptr, np.uint32)
    ix = _arr(inds, np.uint32) if len(inds) else np.zeros(1, np.uint32)
    n_cols = int(n_cols if n_cols is not None else len(ip) - 1)
    n_rows = int(n_rows if n_rows is not None else n_cols)
    lv = np.empty(n_cols, np.int32)
    ec = C.c_uint64(0)
    rc = _load().oracle_bfs(n_rows, n_cols, len(inds), ip.ctypes.data_as(U32P),
                            ix.ctypes.data_as(U32P), int(root), lv.ctypes.data_as(I32P),
                            C.byref(ec))
    if rc != 0:
        raise ValueError(f"oracle_bfs failed with status {rc}")
    return lv, ec.value


def oracle_bfs_queue(indptr, inds, root, n_rows=None, n_cols=None):
    """O(n + nnz) queue form; same levels and edge count as oracle_bfs."""
    ip = _arr(indptr, np.uint32)
    ix = _arr(inds, np.uint32) if len(inds) else np.zeros(1, np.uint32)
    n_cols = int(n_cols if n_cols is not None else len(ip) - 1)
    n_rows = int(n_rows if n_rows is not None else n_cols)
    lv = np.empty(n_cols, np.int32)
    ec = C.c_uint64(0)
    rc = _load().oracle_bfs_queue(n_rows, n_cols, len(inds), ip.ctypes.data_as(U32P),
                                  ix.ctypes.data_as(U32P), int(root), lv.ctypes.data_as(I32P),
                                  C.byref(ec))
    if rc != 0:
        raise ValueError(f"oracle_bfs_queue failed with status {rc}")
    return lv, ec.value


def oracle_bfs_many(indptr, inds, roots, n_threads=None, n_rows=None, n_cols=None,
                    keep_levels=True, queue_form=False):
    """Independent BFS per root on n_threads host threads.
    Returns (levels int32[len(roots), n_cols] or None, edges uint64[len(roots)])."""
    ip = _arr(indptr, np.uint32)
    ix = _arr(inds, np.uint32) if len(inds) else np.zeros(1, np.uint32)
    rt = _arr(roots, np.uint32)
    n_cols = int(n_cols if n_cols is not None else len(ip) - 1)
    n_rows = int(n_rows if n_rows is not None else n_cols)
    n_threads = n_threads or os.cpu_count() or 1
    lv = np.empty((len(rt), n_cols), np.int32) if keep_levels else None
    ec = np.zeros(len(rt), np.uint64)
    rc = _load().oracle_bfs_many(n_rows, n_cols, len(inds), ip.ctypes.data_as(U32P),
                                 ix.ctypes.data_as(U32P), rt.ctypes.data_as(U32P), len(rt),
                                 int(n_threads), int(queue_form),
                                 lv.ctypes.data_as(I32P) if lv is not None
                                 else None, ec.ctypes.data_as(U64P))
    if rc != 0:
        raise ValueError(f"oracle_bfs_many failed with status {rc}")
    return lv, ec


def _parts(indptrs, indss):
    ips = [_arr(a, np.uint32) for a in indptrs]
    ixs = [_arr(a, np.uint32) if len(a) else np.zeros(1, np.uint32) for a in indss]
    P = len(ips)
    ipa = (U32P * P)(*[a.ctypes.data_as(U32P) for a in ips])
    ixa = (U32P * P)(*[a.ctypes.data_as(U32P) for a in ixs])
    nnz = np.array([len(a) for a in indss], np.uint64)
    return ips, ixs, ipa, ixa, nnz


def oracle_bfs_multi(indptrs, indss, root, n_rows, n_cols):
    """Multi-partition restatement (run_bfs_cpu.hpp:47-62)."""
    ips, ixs, ipa, ixa, nnz = _parts(indptrs, indss)
    lv = np.empty(n_cols, np.int32)
    ec = C.c_uint64(0)
    rc = _load().oracle_bfs_multi(n_rows, n_cols, len(ips), ipa, ixa,
                                  nnz.ctypes.data_as(U64P), int(root),
                                  lv.ctypes.data_as(I32P), C.byref(ec))
    if rc != 0:
        raise ValueError(f"oracle_bfs_multi failed with status {rc}")
    return lv, ec.value


def ref_bfs(indptrs, indss, root, n_rows, n_cols):
    """The reference's own run_bfs_cpu with len(indptrs) partitions (1..4)."""
    ips, ixs, ipa, ixa, nnz = _parts(indptrs, indss)
    f = getattr(_load_ref(), f"ref_bfs_p{len(ips)}")
    lv = np.empty(n_cols, np.int32)
    ec = C.c_uint64(0)
    rc = f(n_rows, n_cols, ipa, ixa, nnz.ctypes.data_as(U64P), int(root),
           lv.ctypes.data_as(I32P), C.byref(ec))
    if rc != 0:
        raise ValueError(f"ref_bfs failed with status {rc}")
    return lv, ec.value


class Csc:
    """A CSC graph held in arrays that the oracle library allocated; each
    buffer is released when the last numpy view of it is garbage collected."""

    def __init__(self, indptr_p, inds_p, n, nnz):
        self.n_rows = self.n_cols = n
        self.nnz = nnz
        self.indptr = _owned(indptr_p, n + 1)
        self.inds = _owned(inds_p, max(nnz, 1))[:nnz]


def _owned(ptr, count):
    import weakref
    base = np.ctypeslib.as_array(ptr, shape=(count,))
    weakref.finalize(base, _load().oracle_free, C.cast(ptr, C.c_void_p).value)
    return base


def oracle_gen_rmat(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1, symmetrize=True,
                    threads=0):
    """Seeded R-MAT CSC (deduplicated, self-loops dropped), built on the host
    by graph_gen_oracle.c; the same bytes as the engine's generator."""
    ip, ix, nnz = U32P(), U32P(), C.c_uint64(0)
    rc = _load().oracle_gen_rmat(int(scale), int(edge_factor), float(a), float(b), float(c),
                                 int(seed), int(bool(symmetrize)), int(threads), C.byref(ip),
                                 C.byref(ix), C.byref(nnz))
    if rc != 0:
        raise ValueError(f"oracle_gen_rmat failed with status {rc}")
    return Csc(ip, ix, 1 << int(scale), int(nnz.value))


def oracle_sample_roots(indptr, count, seed, n_rows=None):
    """count distinct seeded roots with out-degree > 0."""
    ip = _arr(indptr, np.uint32)
    n_rows = int(n_rows if n_rows is not None else len(ip) - 1)
    out = np.empty(max(int(count), 1), np.uint32)
    rc = _load().oracle_sample_roots(ip.ctypes.data_as(U32P), n_rows, int(count), int(seed),
                                     out.ctypes.data_as(U32P))
    if rc != 0:
        raise ValueError(f"oracle_sample_roots failed with status {rc}")
    return out[:int(count)]
