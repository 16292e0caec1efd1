#!/usr/bin/env python
"""Benchmark: GTEPS of single-root top-down BFS on R-MAT scale 25, edge factor
16 (seed 5, a/b/c/d = .57/.19/.19/.05, deduplicated, symmetrised, uint32 CSC),
on one GB300, with the learned per-level schedule; fixed LLB beside it; and
roots/s of 64-root batched BFS.

One step = one BFS from one seeded root (degree > 0), the unit the reference
times per run (src/run_bfs_gpu.hpp:679-728).  GTEPS = edgesCount / BFS time
(src/host.cpp:196), edgesCount = sum of out-degrees of expanded vertices.

  value     device time (CUDA events on the engine's stream) of the whole BFS
            with the graph resident in HBM: level init, every level, no copies;
            explore arm picked per level by the learned scheduler
  e2e       the same metric through the public C call bfs_run_roots, one call
            for the timed steps: each step's root in, its n-entry int32 level
            array copied back to its own pinned host buffer inside the timed
            region (step i's copy overlaps step i + 1's BFS), wall clock;
            e2e_bfs_run beside it: one blocking bfs_run call per step
  roofline  the explore kernels (dominant): algorithmic bytes 4*E + 8*F per
            launch (edges + frontier {beg, prefix} entries) / their CUDA-event
            time, from a host-loop pass with per-kernel events
  fixed_llb the same workload with the fixed LLB/256 explore (the reference's
            default build, src/CMakeLists.txt:10-11)
  batched   64 roots per bfs_run_batch pass vs 64 sequential single-root runs
  cpu_baseline  the oracle (C restatement of run_bfs_cpu) on one root of the
            same graph, one host thread

--impl reference times the reference's CPU BFS (the oracle port of
run_bfs_cpu; the compiled reference cannot travel to this machine) on every
host thread: each step runs one single-threaded BFS per thread, distinct roots.

N > 1 (torchrun): replicas only -- every rank runs the same workload on its own
GPU with its own roots; value = edges of all ranks / max time over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bfs-gpu-sycl_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "GTEPS at RMAT-25/EF16 on 1xGB300: learned-schedule vs fixed-LLB; roots/s batched"
WEIGHTS = os.path.join(PKG, "sched_weights.f32")
UNIT = "GTEPS"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=int, default=25)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--lb", default="learned", help="explore plan for `value`")
    ap.add_argument("--loop", default="graph", choices=["graph", "host"],
                    help="level-loop driver (host: every kernel a plain launch, for ncu)")
    ap.add_argument("--skip-batched", action="store_true", help="omit the batched leg")
    ap.add_argument("--skip-multigraph", action="store_true",
                    help="omit the 256-graph single-launch leg")
    ap.add_argument("--block", type=int, default=256)
    ap.add_argument("--skip-cpu", action="store_true", help="omit the cpu_baseline leg")
    ap.add_argument("--skip-arms", action="store_true", help="omit the per-arm table")
    ap.add_argument("--skip-suites", action="store_true",
                    help="omit the per-variant tables on RMAT-23, the 4096^2 grid and ER-2^22")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling in the background (read-only)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
              "utilization.gpu")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.path = os.path.join("/tmp", f"bfs_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                rows.append(dict(sm=float(p[1]), smax=float(p[2]), power=float(p[3]),
                                 hw=p[5], hwt=p[6], swt=p[7], pcap=p[8],
                                 util=float(p[9]) if p[9] not in ("", "[N/A]") else 0.0))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        busy = [r for r in rows if r["util"] > 0] or rows
        reasons = set()
        for r in busy:
            for k, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                            ("swt", "sw_thermal_slowdown"), ("pcap", "sw_power_cap")):
                if r[k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in busy),
                "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": sorted(reasons), "samples": len(busy),
                "power_w_max": max(r["power"] for r in rows)}


def dist_setup(backend):
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    return rank, world, local


def reduce_max_sum(vals_max, vals_sum, world):
    """Max over ranks of vals_max and sum over ranks of vals_sum."""
    if world == 1:
        return list(vals_max), list(vals_sum)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    a = torch.tensor(vals_max, dtype=torch.float64, device=dev)
    b = torch.tensor(vals_sum, dtype=torch.float64, device=dev)
    dist.all_reduce(a, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return a.cpu().tolist(), b.cpu().tolist()


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def bfs_bytes(edges, reached, n):
    """Algorithmic bytes of one BFS: 4 per traversed edge, 16 per reached
    vertex (indptr pair, frontier write, frontier read), 4 per vertex (level)."""
    return 4.0 * edges + 16.0 * reached + 4.0 * n


PLANS = [(lb, blk) for lb in ("llb", "glb", "slb") for blk in (128, 256, 512)]


def suite_table(B, torch, graph, roots, weights, hbm_peak):
    """Per-variant GTEPS, HBM GB/s (the bytes-moved formula of bfs_bytes over
    each run's edges and reached vertices) and roofline fraction of the
    single-root engine on one graph: every explore form x block size and the
    learned schedule, the same roots for every plan, device time."""
    n = graph.n_cols
    lv = torch.empty(n, dtype=torch.int32, device="cuda")
    plans = list(PLANS)
    if weights is not None:
        graph.sched_attach(weights)
        plans.append(("learned", 256))
    rows = {}
    for lb, blk in plans:
        o = B.options(lb, blk)
        graph.run_device(int(roots[0]), lv.data_ptr(), opts=o)  # builds the loop graph
        ms, edges, byts = 0.0, 0.0, 0.0
        for r in roots:
            st = graph.run_device(int(r), lv.data_ptr(), opts=o)
            ms += st.device_ms
            edges += st.edges_count
            byts += bfs_bytes(st.edges_count, st.reached, n)
        gbs = byts / (ms * 1e-3) / 1e9
        rows["learned" if lb == "learned" else f"{lb}{blk}"] = {
            "gteps": round(edges / (ms * 1e-3) / 1e9, 3), "ms_per_bfs": round(ms / len(roots), 4),
            "hbm_gbs": round(gbs, 1), "roofline_frac": round(gbs / hbm_peak, 4)}
    best = max((k for k in rows if k != "learned"), key=lambda k: rows[k]["gteps"])
    out = {"variants": rows, "best_fixed": best}
    if "learned" in rows:
        out["learned_vs_best_fixed"] = round(rows["learned"]["gteps"] / rows[best]["gteps"], 3)
        out["learned_vs_llb256"] = round(rows["learned"]["gteps"] / rows["llb256"]["gteps"], 3)
    del lv
    return out


def run_suites(B, torch, weights, hbm_peak):
    """BASELINE's configurations 2 and 3, measured per variant."""
    res = {}
    g = B.Graph.gen_rmat_device(23, 16, seed=2)
    t = suite_table(B, torch, g, B.sample_roots(g.download(), 64, 2), weights, hbm_peak)
    t["workload"] = ("RMAT-23/EF16 seed 2 (deduplicated, symmetrised), 64 seeded roots, "
                     "graph level loop")
    res["rmat23"] = t
    g.free()
    for key, make, roots_seed, label in (
            ("grid4096", lambda: B.gen_grid(4096, 4096, 0.05, 3), 3,
             "4096x4096 4-neighbour grid, 5% of edges deleted (seed 3), 32 seeded roots"),
            ("er22", lambda: B.gen_er(1 << 22, 16.0, 4), 4,
             "Erdos-Renyi, 2^22 vertices, average degree 16 (seed 4), 32 seeded roots")):
        h = make()
        g = B.Graph.upload(h, validate=False)
        t = suite_table(B, torch, g, B.sample_roots(h, 32, roots_seed), weights, hbm_peak)
        t["workload"] = label + ", graph level loop"
        res[key] = t
        g.free()
        del h
    return res


def run_gb300(a):
    import numpy as np
    import torch
    import bfs_gb300 as B

    rank, world, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    hbm_peak, peak_kind = peaks()

    t = time.perf_counter()
    dg = B.Graph.gen_rmat_device(a.scale, a.edge_factor, seed=a.seed)
    gen_s = time.perf_counter() - t
    n = dg.n_cols
    host = dg.download()
    roots = B.sample_roots(host, a.warmup + a.steps + 8, a.seed + 1000 * rank)
    lv = torch.empty(n, dtype=torch.int32, device="cuda")
    t = time.perf_counter()
    dg.hub_configure(-1)  # the default layout, built here rather than in the first run
    hub_s = round(time.perf_counter() - t, 3)
    hub = dg.hub_info()
    weights = None
    if os.path.exists(WEIGHTS):
        weights = np.fromfile(WEIGHTS, dtype="<f4")
        dg.sched_attach(weights)
    opts = B.options(a.lb, a.block, loop=a.loop)

    sampler = ClockSampler(local)
    sampler.start()
    for r in roots[:a.warmup]:
        dg.run_device(int(r), lv.data_ptr(), opts=opts)
    torch.cuda.synchronize()
    barrier(world)
    wall0 = time.perf_counter()
    dev_ms, edges, reached, launches = [], [], [], 0
    for r in roots[a.warmup:a.warmup + a.steps]:
        st = dg.run_device(int(r), lv.data_ptr(), opts=opts)
        dev_ms.append(st.device_ms)
        edges.append(st.edges_count)
        reached.append(st.reached)
        launches += st.launches
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    # correctness spot check of the last timed run (device Graph500 checks)
    bad = dg.validate_device(int(roots[a.warmup + a.steps - 1]), lv.data_ptr())
    barrier(world)
    # keep the GPU busy a little longer so the clock record has load samples
    extra = 0.0
    while extra < 0.6:
        t = time.perf_counter()
        dg.run_device(int(roots[a.warmup]), lv.data_ptr(), opts=opts)
        extra += time.perf_counter() - t
    clocks = sampler.stop()

    total_ms = sum(dev_ms)
    tot_edges = float(sum(edges))
    (max_ms,), (sum_edges,) = reduce_max_sum([total_ms], [tot_edges], world)
    value = sum_edges / (max_ms * 1e-3) / 1e9

    # e2e through bfs_run_roots: the steps' roots in, each step's level array
    # out to its own pinned host buffer, all inside the timed region
    e2e_steps = max(3, min(a.steps, 64))  # the timed steps' roots (at most 64 pinned arrays)
    e_roots = [int(r) for r in roots[a.warmup:a.warmup + e2e_steps]]
    pinned = [torch.empty(n, dtype=torch.int32, pin_memory=True) for _ in e_roots]
    ptrs = [t.data_ptr() for t in pinned]
    dg.run_roots([int(r) for r in roots[:2]], ptrs[:2], opts=opts)
    barrier(world)
    t = time.perf_counter()
    sts = dg.run_roots(e_roots, ptrs, opts=opts)
    e_wall = time.perf_counter() - t
    e_edges = float(sum(st.edges_count for st in sts))
    (e_wall_max,), (e_edges_sum,) = reduce_max_sum([e_wall], [e_edges], world)
    e2e = e_edges_sum / e_wall_max / 1e9
    # one blocking bfs_run per step (no overlap of copy and next BFS)
    e_edges, e_wall = 0.0, 0.0
    barrier(world)
    for r, p in zip(e_roots, ptrs):
        t = time.perf_counter()
        st = dg.run_into(r, p, opts=opts)
        e_wall += time.perf_counter() - t
        e_edges += st.edges_count
    (e_wall_max,), (e_edges_sum,) = reduce_max_sum([e_wall], [e_edges], world)
    e2e_single = e_edges_sum / e_wall_max / 1e9
    del pinned

    # fixed LLB/256 on the same roots (the reference's default build)
    llb_ms, llb_edges = 0.0, 0.0
    o_llb = B.options("llb", 256, loop=a.loop)
    dg.run_device(int(roots[0]), lv.data_ptr(), opts=o_llb)
    for r in roots[a.warmup:a.warmup + a.steps]:
        st = dg.run_device(int(r), lv.data_ptr(), opts=o_llb)
        llb_ms += st.device_ms
        llb_edges += st.edges_count
    llb_gteps = llb_edges / (llb_ms * 1e-3) / 1e9

    # explore-kernel roofline: per-level CUDA-event times in the host loop.
    # Dominant launch = the level with the most edges (same level of every
    # profiled root is averaged); all levels are also aggregated.
    prof_bytes, prof_ms, gen_ms, lvl_rows = 0.0, 0.0, 0.0, []
    dom_bytes, dom_ms, dom_edges, dom_n = 0.0, 0.0, 0.0, 0
    for r in roots[a.warmup:a.warmup + 3]:
        st = dg.run_device(int(r), lv.data_ptr(),
                           opts=B.options(a.lb, a.block, loop="host", record=2))
        tab = st.levels_table()
        big = max(range(st.recorded), key=lambda i: tab["edges"][i])
        for i in range(st.recorded):
            F, EF = tab["frontier"][i], tab["edges"][i]
            if F == 0:
                continue
            prof_bytes += 4.0 * EF + 8.0 * F
            prof_ms += tab["explore_ms"][i]
            gen_ms += tab["gen_ms"][i]
            if i == big:
                dom_bytes += 4.0 * EF + 8.0 * F
                dom_ms += tab["explore_ms"][i]
                dom_edges += EF
                dom_n += 1
            if r == roots[a.warmup]:
                lvl_rows.append([i, F, EF, B.ARM_NAMES[tab["arm"][i]],
                                 round(tab["explore_ms"][i], 4), round(tab["gen_ms"][i], 4)])
    achieved_all = prof_bytes / (prof_ms * 1e-3) / 1e9 if prof_ms > 0 else None
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9 if dom_ms > 0 else None
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "explore_traffic.json")
    if os.path.exists(tfile) and dom_n:
        try:
            per_edge = json.load(open(tfile))["traffic_bytes_per_edge"]
            traffic = round(per_edge * dom_edges / dom_n)
        except Exception:
            traffic = None

    # per-arm table (GTEPS of every explore form x block size, graph loop),
    # with the learned schedule on the same roots for a like-for-like row
    arms = {}
    if not a.skip_arms:
        plans = [(lb, blk) for lb in ("llb", "glb", "slb") for blk in (128, 256, 512)]
        if weights is not None:
            plans.append(("learned", 256))
        for lb, blk in plans:
            o = B.options(lb, blk)
            dg.run_device(int(roots[0]), lv.data_ptr(), opts=o)
            ms, ed = 0.0, 0.0
            for r in roots[a.warmup:a.warmup + 4]:
                st = dg.run_device(int(r), lv.data_ptr(), opts=o)
                ms += st.device_ms
                ed += st.edges_count
            arms["learned" if lb == "learned" else f"{lb}{blk}"] = \
                round(ed / (ms * 1e-3) / 1e9, 3)

    # batched: multi-source passes of 64 roots vs 64 sequential runs.
    # (1) the batched configuration: RMAT-22/EF16 seed 6, 1024 seeded roots in
    #     16 passes; (2) one 64-root pass on this RMAT-25 graph.
    batched = batched25 = None
    if not a.skip_batched:
        def seq_ms(graph, rs, o):
            graph.run_device(int(rs[0]), seq_lv.data_ptr(), opts=o)
            return sum(graph.run_device(int(r), seq_lv.data_ptr(), opts=o).device_ms
                       for r in rs)

        g22 = B.Graph.gen_rmat_device(22, 16, seed=6)
        if weights is not None:
            g22.sched_attach(weights)
        r22 = B.sample_roots(g22.download(), 1024, 6)
        out = torch.empty((64, g22.n_cols), dtype=torch.int32, device="cuda")
        g22.run_batch(r22[:64], out.data_ptr(), want_edges=False)
        b_ms = 0.0
        for b in range(16):
            _, bst = g22.run_batch(r22[64 * b:64 * (b + 1)], out.data_ptr(), want_edges=False)
            b_ms += bst.device_ms
        seq_lv = torch.empty(g22.n_cols, dtype=torch.int32, device="cuda")
        s_llb = seq_ms(g22, r22[:64], B.options("llb", 256))
        s_lrn = seq_ms(g22, r22[:64], B.options(a.lb, a.block))
        batched = {"roots_per_s": round(1024 / (b_ms * 1e-3), 1),
                   "ms_per_64_roots": round(b_ms / 16, 3),
                   "sequential_llb256_roots_per_s": round(64 / (s_llb * 1e-3), 1),
                   "sequential_learned_roots_per_s": round(64 / (s_lrn * 1e-3), 1),
                   "speedup_vs_sequential_llb256": round(s_llb / (b_ms / 16), 2),
                   "speedup_vs_sequential_learned": round(s_lrn / (b_ms / 16), 2),
                   "workload": "RMAT-22/EF16 seed 6, 1024 seeded roots in 16 bfs_run_batch "
                               "passes of 64 vs 64 sequential bfs_run_device runs (device "
                               "CUDA-event time)"}
        del out, seq_lv
        g22.free()
        broots = B.sample_roots(host, 64, a.seed + 7)
        out = torch.empty((64, n), dtype=torch.int32, device="cuda")
        dg.run_batch(broots, out.data_ptr(), want_edges=False)
        bms = [dg.run_batch(broots, out.data_ptr(), want_edges=False)[1].device_ms
               for _ in range(3)]
        b25 = min(bms)
        del out
        seq_lv = torch.empty(n, dtype=torch.int32, device="cuda")
        s_llb = seq_ms(dg, broots, B.options("llb", 256))
        s_lrn = seq_ms(dg, broots, opts)
        del seq_lv
        batched25 = {"roots_per_s": round(64 / (b25 * 1e-3), 1), "batch64_ms": round(b25, 3),
                     "sequential_llb256_roots_per_s": round(64 / (s_llb * 1e-3), 1),
                     "sequential_learned_roots_per_s": round(64 / (s_lrn * 1e-3), 1),
                     "speedup_vs_sequential_llb256": round(s_llb / b25, 2),
                     "speedup_vs_sequential_learned": round(s_lrn / b25, 2)}

    # many small graphs: 256 uneven R-MAT graphs (scales 10-16, EF16, seeds
    # 100-355), one root each, one autotuned CUDA-graph launch vs one
    # single-graph BFS after another
    multigraph = None
    if not a.skip_multigraph:
        import tempfile
        graphs, mroots = B.multi_batch_graphs(B.multi_batch_specs())
        mb = B.MultiBatch(graphs)
        mout = torch.empty(mb.total_cols, dtype=torch.int32, device="cuda")
        cache = os.path.join(tempfile.gettempdir(), "bfs_gb300_multigraph_autotune.tsv")
        best, tune_ms = mb.autotune(mroots, mout.data_ptr(), reps=3, cache_path=cache)
        mb.run(mroots, mout.data_ptr(), *best)
        mms = sorted(mb.run(mroots, mout.data_ptr(), *best)[1] for _ in range(5))
        m_ms = mms[len(mms) // 2]
        seq_plain, seq_graph = 0.0, 0.0
        handles = [B.Graph.upload(g, validate=False) for g in graphs]
        for h, r in zip(handles, mroots):
            slv = torch.empty(h.n_cols, dtype=torch.int32, device="cuda")
            h.run_device(int(r), slv.data_ptr(), opts=B.options("llb", 256, loop="host"))
            seq_plain += h.run_device(int(r), slv.data_ptr(),
                                      opts=B.options("llb", 256, loop="host")).device_ms
            h.run_device(int(r), slv.data_ptr(), opts=B.options("llb", 256))
            seq_graph += h.run_device(int(r), slv.data_ptr(),
                                      opts=B.options("llb", 256)).device_ms
            h.free()
        mb.free()
        del mout
        multigraph = {
            "graphs_per_s": round(len(graphs) / (m_ms * 1e-3), 1),
            "launch_ms": round(m_ms, 4),
            "autotuned": {"block": best[0], "items_per_thread": best[1], "cluster": best[2],
                          "times_ms": {f"{b}x{p}" + (f"c{c}" if c > 1 else ""): round(t, 4)
                                       for (b, p, c), t in zip(B.MULTI_CONFIGS_ALL, tune_ms)}},
            "sequential_plain_launches_graphs_per_s": round(len(graphs) / (seq_plain * 1e-3), 1),
            "sequential_graph_loop_graphs_per_s": round(len(graphs) / (seq_graph * 1e-3), 1),
            "speedup_vs_sequential_plain_launches": round(seq_plain / m_ms, 2),
            "speedup_vs_sequential_graph_loop": round(seq_graph / m_ms, 2),
            "workload": "256 R-MAT graphs, scales drawn from 10-16, EF16, seeds 100-355, one "
                        "root each; one persistent CUDA-graph launch vs 256 single-graph BFS "
                        "(LLB/256, device time summed)"}

    # learned scheduler regret on this held-out graph: every level of two
    # roots timed with all 9 arms from the same state (bfs_sched_record), the
    # model's choice from the level's features, against the per-level best
    regret = None
    if weights is not None and not a.skip_arms:
        t_sel, t_best, per_level = 0.0, 0.0, []
        for r in roots[a.warmup:a.warmup + 2]:
            smp = dg.sched_record(int(r), reps=2)
            feats = np.array([list(x.features) for x in smp], np.float32)
            ms = np.array([list(x.arm_ms) for x in smp], np.float64)
            chosen, _ = B.sched_predict(weights, feats)
            for i in range(len(smp)):
                best = ms[i].min()
                t_sel += ms[i][chosen[i]]
                t_best += best
                per_level.append(round(float(ms[i][chosen[i]] / best - 1.0), 4) if best > 0 else 0.0)
        regret = {"explore_regret_frac": round(t_sel / t_best - 1.0, 4),
                  "per_level_regret": per_level,
                  "roots": 2, "levels": len(per_level),
                  "method": "bfs_sched_record: every level timed with all 9 explore arms from the "
                            "same state (best of 2); regret = time of the model's arm / best arm - 1"}
    arms_best = None
    if arms:
        fixed = {k: v for k, v in arms.items() if k != "learned"}
        arms_best = max(fixed, key=fixed.get)

    suites = None
    if not a.skip_suites:
        suites = run_suites(B, torch, weights, hbm_peak)

    # CPU baseline: the oracle on one root, one thread (rank 0 only)
    cpu = None
    if rank == 0 and not a.skip_cpu:
        import bfs_oracle as O
        r = int(roots[a.warmup])
        t = time.perf_counter()
        ref, ec = O.oracle_bfs(host.indptr, host.inds, r)
        cpu_s = time.perf_counter() - t
        st = dg.run_device(r, lv.data_ptr(), opts=opts)
        match = bool(np.array_equal(lv.cpu().numpy(), ref)) and st.edges_count == ec
        cpu = {"value": round(ec / cpu_s / 1e9, 4), "unit": UNIT, "cores": 1,
               "kind": "port", "sample": f"one BFS from root {r} of the same RMAT-{a.scale} "
               f"graph, level-synchronous run_bfs_cpu restatement, {cpu_s:.2f} s",
               "parity_with_gpu": match}

    plan = "learned per-level schedule" if a.lb == "learned" else f"{a.lb}{a.block}"
    mean_edges = tot_edges / len(edges)
    mean_reached = sum(reached) / len(reached)
    bfs_gbs = bfs_bytes(mean_edges, mean_reached, n) / ((total_ms / len(dev_ms)) * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": round(total_ms / len(dev_ms), 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic (seeded R-MAT generated on the device)",
        "config": {"workload": workload(a), "explore_plan": plan, "level_loop": a.loop,
                   "scheduler_weights": os.path.basename(WEIGHTS) if weights is not None
                   else None,
                   "vertices": n, "edges": dg.nnz, "roots_timed": a.steps,
                   "l2": "inputs larger than L2 (4 B x edges >> 129 MB)",
                   "graph_gen_s": round(gen_s, 2), "timed_wall_s": round(wall, 4)},
        "e2e": {"value": round(e2e, 4), "unit": UNIT, "h2d_bytes_per_step": 4,
                "d2h_bytes_per_step": 4 * n, "api": "bfs_run_roots", "steps": len(e_roots),
                "output": "one pinned host level array per step"},
        "e2e_bfs_run": {"value": round(e2e_single, 4), "unit": UNIT,
                        "api": "bfs_run, one blocking call per step"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None,
                     "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(achieved / hbm_peak, 4) if achieved else None,
                     "traffic": traffic,
                     "kernel": "explore, largest level (4 B/edge + 8 B/entry per launch)",
                     "algorithmic_bytes_per_launch": round(dom_bytes / dom_n) if dom_n else None,
                     "achieved_all_levels": round(achieved_all, 1) if achieved_all else None,
                     "traffic_source": "profiles/explore_traffic.json: ncu DRAM bytes per edge "
                                       "of the RMAT-24 largest launch x this launch's edges",
                     "peak_kind": peak_kind,
                     "bfs_bytes_per_s_GBs": round(bfs_gbs, 1),
                     "bfs_frac": round(bfs_gbs / hbm_peak, 4),
                     "explore_share": round(prof_ms / (prof_ms + gen_ms), 3) if prof_ms else None},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches,
        "validator_violations": int(bad),
        "fixed_llb256": {"value": round(llb_gteps, 4), "unit": UNIT},
        "learned_vs_fixed_llb256": round(value / llb_gteps, 3) if a.lb == "learned" else None,
        "learned_vs_best_fixed": ({"best_fixed": arms_best,
                                   "ratio": round(arms["learned"] / arms[arms_best], 4)}
                                  if arms and "learned" in arms else None),
        "scheduler_regret_rmat25": regret,
        "hub_layout": {"vertices": hub[0], "relabelled": hub[1], "build_s": hub_s},
        "batched": batched,
        "batched_rmat25": batched25,
        "multigraph": multigraph,
        "arms_gteps": arms,
        "suites": suites,
        "levels_first_root": lvl_rows,
    }
    if rank == 0:
        print(json.dumps(out))
    dg.free()


def workload(a):
    """The workload name both arms print in config.workload."""
    return f"RMAT-{a.scale}/EF{a.edge_factor} seed {a.seed}, single-root BFS"


def run_reference(a):
    """The reference's CPU BFS (oracle port of run_bfs_cpu) on every host
    thread, same workload; rank 0 only.  The graph and roots come from the
    oracle's own restatement of the generator and root sampler (pinned to the
    engine's bytes by tests/test_oracle_gen.py), so this arm never loads the
    engine library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import bfs_oracle as O
    nthreads = os.cpu_count() or 1
    t = time.perf_counter()
    g = O.oracle_gen_rmat(a.scale, a.edge_factor, seed=a.seed, threads=nthreads)
    gen_s = time.perf_counter() - t
    roots = O.oracle_sample_roots(g.indptr, nthreads * (a.warmup + a.steps), a.seed)
    times, edges = [], []
    for s in range(a.warmup + a.steps):
        rs = roots[s * nthreads:(s + 1) * nthreads]
        t = time.perf_counter()
        _, ec = O.oracle_bfs_many(g.indptr, g.inds, rs, n_threads=nthreads, keep_levels=False)
        dt = time.perf_counter() - t
        if s >= a.warmup:
            times.append(dt)
            edges.append(float(ec.sum()))
    value = sum(edges) / sum(times) / 1e9
    sample = (f"each step: {nthreads} concurrent single-threaded level-synchronous BFS runs "
              f"(run_bfs_cpu restatement) from distinct roots of RMAT-{a.scale}/EF{a.edge_factor}")
    out = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
           "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": round(1e3 * sum(times) / len(times), 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u32",
           "data": "synthetic (seeded R-MAT, the oracle's host generator)",
           "config": {"workload": workload(a), "vertices": g.n_cols, "edges": g.nnz,
                      "graph_gen_s": round(gen_s, 2)},
           "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": nthreads,
                            "kind": "port", "sample": sample},
           "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
