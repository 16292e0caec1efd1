"""Python binding of the C ABI in include/bfs_gb300.h (ctypes, no torch types).

The library is the product; this module only marshals numpy arrays and raw
device pointers into the C calls.  It raises if lib/libbfs_gb300.so is
missing: there is no CPU fallback anywhere in the engine.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libbfs_gb300.so")

LB_LLB, LB_GLB, LB_SLB, LB_LEARNED = 0, 1, 2, 3
LB_NAMES = {"llb": LB_LLB, "glb": LB_GLB, "slb": LB_SLB, "learned": LB_LEARNED}
LOOP_GRAPH, LOOP_HOST = 0, 1
MAX_RECORDED_LEVELS = 4096

STATUS = {
    0: "BFS_OK", 1: "BFS_ERR_INVALID_ARG", 2: "BFS_ERR_ROOT", 3: "BFS_ERR_GRAPH",
    4: "BFS_ERR_CUDA", 5: "BFS_ERR_OOM", 6: "BFS_ERR_IO", 7: "BFS_ERR_LEVEL_LIMIT",
    8: "BFS_ERR_NO_DEVICE", 9: "BFS_ERR_UNSUPPORTED", 10: "BFS_ERR_DEVICE",
}


class BfsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code
        self.status = STATUS.get(code, str(code))


class Options(C.Structure):
    _fields_ = [("lb", C.c_int32), ("block", C.c_int32), ("sm_factor", C.c_int32),
                ("loop", C.c_int32), ("l2_pin", C.c_int32), ("record", C.c_int32),
                ("ipt", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("edges_count", C.c_uint64), ("num_levels", C.c_uint32),
                ("reached", C.c_uint32), ("device_ms", C.c_double),
                ("launches", C.c_uint32), ("recorded", C.c_uint32),
                ("level_frontier", C.c_uint32 * MAX_RECORDED_LEVELS),
                ("level_edges", C.c_uint32 * MAX_RECORDED_LEVELS),
                ("level_arm", C.c_int32 * MAX_RECORDED_LEVELS),
                ("level_explore_ms", C.c_float * MAX_RECORDED_LEVELS),
                ("level_gen_ms", C.c_float * MAX_RECORDED_LEVELS)]

    def levels_table(self):
        n = self.recorded
        return {"frontier": list(self.level_frontier[:n]),
                "edges": list(self.level_edges[:n]),
                "arm": list(self.level_arm[:n]),
                "explore_ms": list(self.level_explore_ms[:n]),
                "gen_ms": list(self.level_gen_ms[:n])}


SCHED_INPUTS, SCHED_ARMS, SCHED_PARAMS = 5, 9, 1545
ARM_NAMES = [f"{lb}{blk}" for lb in ("llb", "glb", "slb") for blk in (128, 256, 512)]


class LevelSample(C.Structure):
    _fields_ = [("features", C.c_float * SCHED_INPUTS), ("arm_ms", C.c_float * SCHED_ARMS),
                ("level", C.c_uint32), ("frontier", C.c_uint32), ("edges", C.c_uint32)]


class TrainOpts(C.Structure):
    _fields_ = [("epochs", C.c_uint32), ("lr", C.c_float), ("seed", C.c_uint64)]


class BatchStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("batches", C.c_uint32),
                ("max_levels", C.c_uint32), ("launches", C.c_uint32)]


class CscHost(C.Structure):
    _fields_ = [("n_rows", C.c_uint32), ("n_cols", C.c_uint32), ("nnz", C.c_uint64),
                ("indptr", C.POINTER(C.c_uint32)), ("inds", C.POINTER(C.c_uint32))]


_lib = None
U32P = C.POINTER(C.c_uint32)
I32P = C.POINTER(C.c_int32)
VP = C.c_void_p


def _sig(lib, name, args, res=C.c_int):
    f = getattr(lib, name)
    f.argtypes = args
    f.restype = res
    return f


def lib():
    """Loads the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} not found: run bfs-gpu-sycl_gb300/build.py first")
    L = C.CDLL(LIB_PATH)
    _sig(L, "bfs_abi_version", [])
    _sig(L, "bfs_status_string", [C.c_int], C.c_char_p)
    _sig(L, "bfs_last_error", [], C.c_char_p)
    _sig(L, "bfs_options_default", [C.POINTER(Options)], None)
    _sig(L, "bfs_graph_upload", [U32P, U32P, C.c_uint32, C.c_uint32, C.c_uint64, C.c_int,
                                 C.POINTER(VP)])
    _sig(L, "bfs_graph_wrap_device", [VP, VP, C.c_uint32, C.c_uint32, C.c_uint64, C.c_int,
                                      C.POINTER(VP)])
    _sig(L, "bfs_graph_free", [VP])
    _sig(L, "bfs_graph_info", [VP, U32P, U32P, C.POINTER(C.c_uint64)])
    _sig(L, "bfs_graph_device_csc", [VP, C.POINTER(VP), C.POINTER(VP)])
    _sig(L, "bfs_hub_configure", [VP, C.c_int64, C.c_uint32])
    _sig(L, "bfs_hub_info", [VP, U32P, I32P, U32P])
    _sig(L, "bfs_run", [VP, C.c_uint32, C.POINTER(Options), I32P, I32P, C.POINTER(Stats)])
    _sig(L, "bfs_run_device", [VP, C.c_uint32, C.POINTER(Options), VP, VP, C.POINTER(Stats)])
    _sig(L, "bfs_run_roots", [VP, U32P, C.c_uint32, C.POINTER(Options), C.POINTER(VP),
                              C.POINTER(VP), C.POINTER(Stats)])
    _sig(L, "bfs_validate_device", [VP, C.c_uint32, VP, VP, C.POINTER(C.c_uint64)])
    _sig(L, "bfs_csc_host_free", [C.POINTER(CscHost)], None)
    _sig(L, "bfs_gen_rmat_host", [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                  C.c_uint64, C.c_int, C.POINTER(CscHost)])
    _sig(L, "bfs_gen_rmat_device", [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                    C.c_uint64, C.c_int, C.POINTER(VP)])
    _sig(L, "bfs_gen_grid_host", [C.c_uint32, C.c_uint32, C.c_double, C.c_uint64,
                                  C.POINTER(CscHost)])
    _sig(L, "bfs_gen_er_host", [C.c_uint32, C.c_double, C.c_uint64, C.POINTER(CscHost)])
    _sig(L, "bfs_graph_download", [VP, C.POINTER(CscHost)])
    _sig(L, "bfs_sample_roots", [U32P, C.c_uint32, C.c_uint32, C.c_uint64, U32P])
    _sig(L, "bfs_dataset_load", [C.c_char_p, C.c_char_p, C.c_uint32, C.POINTER(CscHost)])
    _sig(L, "bfs_dataset_write", [C.c_char_p, C.c_char_p, C.c_uint32, C.POINTER(CscHost)])
    _sig(L, "bfs_dataset_write_split", [C.c_char_p, C.c_char_p, C.c_uint32, C.POINTER(CscHost),
                                        C.c_int32])
    _sig(L, "bfs_dataset_read_meta", [C.c_char_p, U32P, U32P, C.POINTER(C.c_uint64), U32P,
                                      C.c_uint32, U32P])
    _sig(L, "bfs_sched_record", [VP, C.c_uint32, C.c_int32, C.c_int32, C.POINTER(LevelSample),
                                 C.c_uint32, U32P])
    _sig(L, "bfs_sched_train", [C.POINTER(LevelSample), C.c_uint32, C.POINTER(TrainOpts),
                                C.POINTER(C.c_float), C.POINTER(C.c_float)])
    _sig(L, "bfs_sched_predict", [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint32, I32P,
                                  C.POINTER(C.c_float)])
    _sig(L, "bfs_sched_attach", [VP, C.POINTER(C.c_float), C.c_float])
    _sig(L, "bfs_run_batch", [VP, U32P, C.c_uint32, VP, C.POINTER(C.c_uint64),
                              C.POINTER(BatchStats)])
    _sig(L, "bfs_run_batch_host", [VP, U32P, C.c_uint32, I32P, C.POINTER(C.c_uint64),
                                   C.POINTER(BatchStats)])
    _sig(L, "bfs_run_batch_loop", [VP, U32P, C.c_uint32, VP, C.POINTER(C.c_uint64),
                                   C.c_int32, C.POINTER(BatchStats)])
    _sig(L, "bfs_multi_create", [C.c_uint32, C.POINTER(U32P), C.POINTER(U32P), U32P, U32P,
                                 C.POINTER(C.c_uint64), C.POINTER(VP)])
    _sig(L, "bfs_multi_free", [VP])
    _sig(L, "bfs_multi_level_offset", [VP, C.c_uint32, C.POINTER(C.c_uint64)])
    _sig(L, "bfs_multi_run", [VP, U32P, C.c_int32, C.c_int32, VP, C.POINTER(C.c_uint64),
                              C.POINTER(C.c_double)])
    _sig(L, "bfs_multi_run_ex", [VP, U32P, C.c_int32, C.c_int32, C.c_int32, VP,
                                 C.POINTER(C.c_uint64), C.POINTER(C.c_double)])
    _sig(L, "bfs_multi_autotune_ex", [VP, U32P, VP, C.c_int32, C.c_char_p, I32P, I32P, I32P,
                                      C.POINTER(C.c_float)])
    _sig(L, "bfs_multi_num_configs", [I32P, I32P, I32P, C.c_int32], C.c_int32)
    _sig(L, "bfs_multi_autotune", [VP, U32P, VP, C.c_int32, C.c_char_p, I32P, I32P,
                                   C.POINTER(C.c_float)])
    _lib = L
    return L


def check(code):
    if code != 0:
        raise BfsError(code, lib().bfs_last_error().decode(errors="replace"))


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(U32P)


class Csc:
    """Host CSC graph in the reference layout (numpy arrays)."""

    def __init__(self, indptr, inds, n_rows=None, n_cols=None):
        self.indptr = np.ascontiguousarray(indptr, dtype=np.uint32)
        self.inds = np.ascontiguousarray(inds, dtype=np.uint32)
        self.n_cols = int(n_cols if n_cols is not None else len(self.indptr) - 1)
        self.n_rows = int(n_rows if n_rows is not None else self.n_cols)

    @property
    def nnz(self):
        return int(self.inds.shape[0])

    def degree(self):
        return np.diff(self.indptr.astype(np.int64))

    @staticmethod
    def _from_c(ch):
        n = ch.n_cols
        ip = np.ctypeslib.as_array(ch.indptr, shape=(n + 1,)).copy()
        ix = (np.ctypeslib.as_array(ch.inds, shape=(ch.nnz,)).copy() if ch.nnz
              else np.zeros(0, np.uint32))
        out = Csc(ip, ix, ch.n_rows, ch.n_cols)
        lib().bfs_csc_host_free(C.byref(ch))
        return out

    def _to_c(self):
        ch = CscHost()
        ch.n_rows, ch.n_cols, ch.nnz = self.n_rows, self.n_cols, self.nnz
        ch.indptr = self.indptr.ctypes.data_as(U32P)
        ch.inds = self.inds.ctypes.data_as(U32P)
        return ch


def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, symmetrize=True):
    ch = CscHost()
    check(lib().bfs_gen_rmat_host(scale, edge_factor, a, b, c, seed, int(symmetrize),
                                  C.byref(ch)))
    return Csc._from_c(ch)


def gen_grid(width, height, delete_prob=0.05, seed=3):
    ch = CscHost()
    check(lib().bfs_gen_grid_host(width, height, delete_prob, seed, C.byref(ch)))
    return Csc._from_c(ch)


def gen_er(n, avg_degree=16.0, seed=4):
    ch = CscHost()
    check(lib().bfs_gen_er_host(n, avg_degree, seed, C.byref(ch)))
    return Csc._from_c(ch)


def sample_roots(g, count, seed):
    ip, ipp = _u32(g.indptr)
    out = np.zeros(count, np.uint32)
    check(lib().bfs_sample_roots(ipp, g.n_rows, count, seed, out.ctypes.data_as(U32P)))
    return out


def dataset_load(name, partitions=1, directory=None):
    ch = CscHost()
    check(lib().bfs_dataset_load(directory.encode() if directory else None, name.encode(),
                                 partitions, C.byref(ch)))
    return Csc._from_c(ch)


SPLITS = {"balanced": 0, "nnz": 1, "row": 2}


def dataset_write(g, name, partitions=1, directory=None, split="balanced"):
    """Writes g as <directory>/<name>-csc-<partitions>/.  split: "balanced"
    (in-degree balanced, exact rows) or the reference generator's "nnz" /
    "row" splits with its round8 breaks (byte-identical files)."""
    ch = g._to_c()
    check(lib().bfs_dataset_write_split(directory.encode() if directory else None,
                                        name.encode(), partitions, C.byref(ch), SPLITS[split]))


def dataset_read_meta(path, max_records=64):
    rows = np.zeros(max_records, np.uint32)
    cols = np.zeros(max_records, np.uint32)
    nnz = np.zeros(max_records, np.uint64)
    start = np.zeros(max_records, np.uint32)
    cnt = C.c_uint32(0)
    check(lib().bfs_dataset_read_meta(path.encode(), rows.ctypes.data_as(U32P),
                                      cols.ctypes.data_as(U32P),
                                      nnz.ctypes.data_as(C.POINTER(C.c_uint64)),
                                      start.ctypes.data_as(U32P), max_records, C.byref(cnt)))
    k = min(cnt.value, max_records)
    return [(int(rows[i]), int(cols[i]), int(nnz[i]), int(start[i])) for i in range(k)]


def samples_to_arrays(samples):
    """LevelSample array -> (features float32[n,5], arm_ms float32[n,9], meta uint32[n,3])."""
    n = len(samples)
    f = np.array([list(x.features) for x in samples], np.float32).reshape(n, SCHED_INPUTS)
    t = np.array([list(x.arm_ms) for x in samples], np.float32).reshape(n, SCHED_ARMS)
    m = np.array([[x.level, x.frontier, x.edges] for x in samples], np.uint32).reshape(n, 3)
    return f, t, m


def arrays_to_samples(features, arm_ms, meta=None):
    n = len(features)
    arr = (LevelSample * n)()
    for i in range(n):
        for j in range(SCHED_INPUTS):
            arr[i].features[j] = float(features[i][j])
        for j in range(SCHED_ARMS):
            arr[i].arm_ms[j] = float(arm_ms[i][j])
        if meta is not None:
            arr[i].level, arr[i].frontier, arr[i].edges = (int(x) for x in meta[i])
    return arr


def sched_train(features, arm_ms, epochs=1500, lr=3e-3, seed=1):
    """Trains the scheduler MLP on the device; returns (weights float32[1545], loss)."""
    samples = arrays_to_samples(features, arm_ms)
    w = np.zeros(SCHED_PARAMS, np.float32)
    loss = C.c_float(0)
    o = TrainOpts(epochs, lr, seed)
    check(lib().bfs_sched_train(samples, len(samples), C.byref(o),
                                w.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
    return w, loss.value


def sched_predict(weights, features):
    w = np.ascontiguousarray(weights, np.float32)
    x = np.ascontiguousarray(features, np.float32).reshape(-1, SCHED_INPUTS)
    arms = np.zeros(len(x), np.int32)
    conf = np.zeros(len(x), np.float32)
    check(lib().bfs_sched_predict(w.ctypes.data_as(C.POINTER(C.c_float)),
                                  x.ctypes.data_as(C.POINTER(C.c_float)), len(x),
                                  arms.ctypes.data_as(I32P),
                                  conf.ctypes.data_as(C.POINTER(C.c_float))))
    return arms, conf


def options(lb="llb", block=256, sm_factor=0, loop="graph", l2_pin=True, record=0, ipt=4):
    o = Options()
    lib().bfs_options_default(C.byref(o))
    o.lb = LB_NAMES[lb] if isinstance(lb, str) else int(lb)
    o.block = int(block)
    o.sm_factor = int(sm_factor)
    o.loop = LOOP_GRAPH if loop == "graph" else LOOP_HOST
    o.l2_pin = int(bool(l2_pin))
    o.record = int(record)
    o.ipt = int(ipt)
    return o


MULTI_CONFIGS = [(b, p) for b in (128, 256, 512) for p in (1, 2, 4)]
# (block, ipt, cluster): the single-block configurations, then the clustered
# ones, in the library's order (bfs_multi_num_configs)
MULTI_CONFIGS_ALL = [(b, p, 1) for b, p in MULTI_CONFIGS] + \
    [(b, p, c) for c in (2, 4, 8) for b in (256, 512) for p in (2, 4)]


def multi_batch_specs(n=256, first_seed=100, scales=(10, 16), edge_factor=16):
    """(scale, edge_factor, seed) of the uneven R-MAT batch: seeds first_seed ..
    first_seed + n - 1, scales drawn uniformly from the closed range with a
    fixed-seed numpy generator (identical on every machine)."""
    rng = np.random.default_rng(20251203)
    sc = rng.integers(scales[0], scales[1] + 1, size=n)
    return [(int(sc[i]), edge_factor, first_seed + i) for i in range(n)]


def multi_batch_graphs(specs):
    """Host-generated graphs and one seeded root (degree > 0) per graph."""
    graphs, roots = [], []
    for scale, ef, seed in specs:
        g = gen_rmat(scale, ef, seed=seed)
        graphs.append(g)
        roots.append(int(sample_roots(g, 1, seed)[0]))
    return graphs, np.array(roots, np.uint32)


class MultiBatch:
    """Many small graphs packed on the device for single-launch BFS."""

    def __init__(self, graphs):
        self._keep = [(np.ascontiguousarray(g.indptr, np.uint32),
                       np.ascontiguousarray(g.inds if g.nnz else np.zeros(1, np.uint32),
                                            np.uint32)) for g in graphs]
        n = len(graphs)
        ips = (U32P * n)(*[k[0].ctypes.data_as(U32P) for k in self._keep])
        ixs = (U32P * n)(*[k[1].ctypes.data_as(U32P) for k in self._keep])
        rows = np.array([g.n_rows for g in graphs], np.uint32)
        cols = np.array([g.n_cols for g in graphs], np.uint32)
        nnz = np.array([g.nnz for g in graphs], np.uint64)
        self.h = VP()
        check(lib().bfs_multi_create(n, ips, ixs, rows.ctypes.data_as(U32P),
                                     cols.ctypes.data_as(U32P),
                                     nnz.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(self.h)))
        self.n_graphs = n
        self.n_cols = cols
        self.total_cols = int(cols.astype(np.int64).sum())
        self._keep = None

    def offset(self, g):
        off = C.c_uint64(0)
        check(lib().bfs_multi_level_offset(self.h, g, C.byref(off)))
        return off.value

    def run(self, roots, levels_ptr, block=256, ipt=2, cluster=1):
        """One launch over the batch; cluster > 1 runs the largest graphs on
        clusters of that many thread blocks."""
        rt = np.ascontiguousarray(roots, np.uint32)
        ec = np.zeros(self.n_graphs, np.uint64)
        ms = C.c_double(0)
        check(lib().bfs_multi_run_ex(self.h, rt.ctypes.data_as(U32P), block, ipt, cluster,
                                     VP(levels_ptr), ec.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     C.byref(ms)))
        return ec, ms.value

    def autotune(self, roots, levels_ptr, reps=3, cache_path=None, clusters=True):
        """Fastest configuration on this batch: (block, ipt, cluster) and the
        timings of MULTI_CONFIGS_ALL (clusters=True), else (block, ipt) and
        the timings of MULTI_CONFIGS."""
        rt = np.ascontiguousarray(roots, np.uint32)
        b, p, c = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        cp = cache_path.encode() if cache_path else None
        if clusters:
            t = (C.c_float * len(MULTI_CONFIGS_ALL))()
            check(lib().bfs_multi_autotune_ex(self.h, rt.ctypes.data_as(U32P), VP(levels_ptr),
                                              reps, cp, C.byref(b), C.byref(p), C.byref(c), t))
            return (b.value, p.value, c.value), list(t)
        t = (C.c_float * len(MULTI_CONFIGS))()
        check(lib().bfs_multi_autotune(self.h, rt.ctypes.data_as(U32P), VP(levels_ptr), reps,
                                       cp, C.byref(b), C.byref(p), t))
        return (b.value, p.value), list(t)

    def free(self):
        if self.h:
            lib().bfs_multi_free(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Graph:
    """A graph resident on the current CUDA device (owns a C handle)."""

    def __init__(self, handle):
        self.h = VP(handle) if not isinstance(handle, VP) else handle
        r, c_, z = C.c_uint32(), C.c_uint32(), C.c_uint64()
        check(lib().bfs_graph_info(self.h, C.byref(r), C.byref(c_), C.byref(z)))
        self.n_rows, self.n_cols, self.nnz = r.value, c_.value, z.value

    @staticmethod
    def upload(g, validate=True):
        ip, ipp = _u32(g.indptr)
        ix, ixp = _u32(g.inds if g.nnz else np.zeros(1, np.uint32))
        h = VP()
        check(lib().bfs_graph_upload(ipp, ixp, g.n_rows, g.n_cols, g.nnz, int(validate),
                                     C.byref(h)))
        return Graph(h)

    @staticmethod
    def wrap_device(d_indptr, d_inds, n_rows, n_cols, nnz, validate=True):
        h = VP()
        check(lib().bfs_graph_wrap_device(VP(d_indptr), VP(d_inds), n_rows, n_cols, nnz,
                                          int(validate), C.byref(h)))
        return Graph(h)

    @staticmethod
    def gen_rmat_device(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1,
                        symmetrize=True):
        h = VP()
        check(lib().bfs_gen_rmat_device(scale, edge_factor, a, b, c, seed, int(symmetrize),
                                        C.byref(h)))
        return Graph(h)

    def download(self):
        ch = CscHost()
        check(lib().bfs_graph_download(self.h, C.byref(ch)))
        return Csc._from_c(ch)

    def hub_configure(self, vertices=-1, min_edges=0):
        """Hub layout of the single-root path: vertices -1 automatic, 0 off,
        K > 0; min_edges: level size from which explore loads the prefix
        (0 automatic)."""
        check(lib().bfs_hub_configure(self.h, int(vertices), int(min_edges)))

    def hub_info(self):
        """(K, relabelled, largest K the device allows) of the current layout."""
        k, rl, mx = C.c_uint32(), C.c_int32(), C.c_uint32()
        check(lib().bfs_hub_info(self.h, C.byref(k), C.byref(rl), C.byref(mx)))
        return k.value, bool(rl.value), mx.value

    def device_csc(self):
        ip, ix = VP(), VP()
        check(lib().bfs_graph_device_csc(self.h, C.byref(ip), C.byref(ix)))
        return ip.value, ix.value

    def run(self, root, opts=None, parents=False, stats=True):
        """One BFS into host arrays; returns (levels, parents or None, Stats)."""
        lv = np.empty(self.n_cols, np.int32)
        pa = np.empty(self.n_cols, np.int32) if parents else None
        st = Stats() if stats else None
        check(lib().bfs_run(self.h, int(root), C.byref(opts) if opts is not None else None,
                            lv.ctypes.data_as(I32P),
                            pa.ctypes.data_as(I32P) if parents else None,
                            C.byref(st) if st is not None else None))
        return lv, pa, st

    def run_into(self, root, levels_host_ptr, parents_host_ptr=None, opts=None, stats=True):
        """One BFS into caller-provided host buffers (e.g. pinned memory)."""
        st = Stats() if stats else None
        check(lib().bfs_run(self.h, int(root), C.byref(opts) if opts is not None else None,
                            C.cast(levels_host_ptr, I32P),
                            C.cast(parents_host_ptr, I32P) if parents_host_ptr else None,
                            C.byref(st) if st is not None else None))
        return st

    def run_roots(self, roots, levels_host_ptrs, parents_host_ptrs=None, opts=None):
        """One BFS per root in one call (bfs_run_roots): run i writes host
        buffer levels_host_ptrs[i] (and parents_host_ptrs[i]); returns the
        runs' Stats.  With pinned buffers run i's copy overlaps run i + 1."""
        r = np.ascontiguousarray(roots, np.uint32)
        k = len(r)
        if len(levels_host_ptrs) != k or (parents_host_ptrs is not None
                                          and len(parents_host_ptrs) != k):
            raise ValueError("one output buffer per root")
        lp = (VP * max(k, 1))(*[VP(p) for p in levels_host_ptrs])
        pp = (VP * max(k, 1))(*[VP(p) for p in parents_host_ptrs]) if parents_host_ptrs else None
        st = (Stats * max(k, 1))()
        check(lib().bfs_run_roots(self.h, r.ctypes.data_as(U32P), k,
                                  C.byref(opts) if opts is not None else None, lp, pp, st))
        return list(st)[:k]

    def run_device(self, root, levels_ptr, parents_ptr=None, opts=None, stats=True):
        st = Stats() if stats else None
        check(lib().bfs_run_device(self.h, int(root),
                                   C.byref(opts) if opts is not None else None,
                                   VP(levels_ptr), VP(parents_ptr) if parents_ptr else None,
                                   C.byref(st) if st is not None else None))
        return st

    def run_batch(self, roots, levels_ptr, want_edges=True, loop="graph"):
        """Multi-source BFS of len(roots) roots into a device int32 buffer of
        len(roots) x n_cols; returns (edges uint64[len(roots)] or None, BatchStats).
        loop="host" launches every kernel separately (for profilers)."""
        rt = np.ascontiguousarray(roots, np.uint32)
        ec = np.zeros(len(rt), np.uint64) if want_edges else None
        st = BatchStats()
        check(lib().bfs_run_batch_loop(self.h, rt.ctypes.data_as(U32P), len(rt),
                                       VP(levels_ptr),
                                       ec.ctypes.data_as(C.POINTER(C.c_uint64)) if want_edges
                                       else None,
                                       LOOP_GRAPH if loop == "graph" else LOOP_HOST, C.byref(st)))
        return ec, st

    def run_batch_host(self, roots, want_levels=True):
        """Multi-source BFS into host arrays: (levels int32[len(roots), n_cols]
        or None, edges uint64[len(roots)], BatchStats)."""
        rt = np.ascontiguousarray(roots, np.uint32)
        lv = np.empty((len(rt), self.n_cols), np.int32) if want_levels else None
        ec = np.zeros(len(rt), np.uint64)
        st = BatchStats()
        check(lib().bfs_run_batch_host(self.h, rt.ctypes.data_as(U32P), len(rt),
                                       lv.ctypes.data_as(I32P) if want_levels else None,
                                       ec.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(st)))
        return lv, ec, st

    def sched_record(self, root, ipt=4, reps=3, max_levels=1 << 16):
        """Per-level features and explore times of all 9 arms for one BFS."""
        buf = (LevelSample * max_levels)()
        n = C.c_uint32(0)
        check(lib().bfs_sched_record(self.h, int(root), ipt, reps, buf, max_levels, C.byref(n)))
        return buf[:n.value]

    def sched_attach(self, weights, min_confidence=0.0):
        if weights is None:
            check(lib().bfs_sched_attach(self.h, None, 0.0))
            return
        w = np.ascontiguousarray(weights, np.float32)
        assert w.size == SCHED_PARAMS
        check(lib().bfs_sched_attach(self.h, w.ctypes.data_as(C.POINTER(C.c_float)),
                                     float(min_confidence)))

    def validate_device(self, root, levels_ptr, parents_ptr=None):
        bad = C.c_uint64(0)
        check(lib().bfs_validate_device(self.h, int(root), VP(levels_ptr),
                                        VP(parents_ptr) if parents_ptr else None,
                                        C.byref(bad)))
        return bad.value

    def free(self):
        if self.h:
            lib().bfs_graph_free(self.h)
            self.h = VP()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
