"""Trains the learned per-level scheduler on a GB300 and evaluates its regret.

Training data are per-level timings that the engine records itself
(bfs_sched_record: every level of a BFS, every one of the 9 explore arms,
same starting state) over seeded synthetic graphs:
  R-MAT scales 18-22 with edge factors 8/16/32, 4-neighbour grids
  1024^2-2048^2 with 5 % of edges deleted, Erdos-Renyi graphs,
  seeds 10-29 (one graph of each family per seed).
Held-out evaluation: R-MAT scale 25 / EF16 seed 5 and R-MAT scale 23 / EF16
seed 2.  Regret of a level = explore time of the chosen arm - best arm's.

Writes sched_weights.f32 (1545 little-endian float32, the layout of
include/bfs_gb300.h) and sched_weights.json (training set, loss, regret)
next to this file, and the recorded samples to --out.

Usage:  python bfs-gpu-sycl_gb300/train_sched.py [--out DIR] [--quick]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, PKG)
import bfs_gb300 as B  # noqa: E402

WEIGHTS = os.path.join(PKG, "sched_weights.f32")
REPORT = os.path.join(PKG, "sched_weights.json")
FIXED_LLB = 1  # arm index of LLB / 256 threads


def training_graphs(quick):
    seeds = range(10, 30) if not quick else range(10, 13)
    for s in seeds:
        scale = 18 + (s % 5)
        ef = (8, 16, 32)[s % 3]
        yield f"rmat{scale}_ef{ef}_s{s}", ("rmat", scale, ef, s)
        side = (1024, 1536, 2048)[s % 3]
        yield f"grid{side}_s{s}", ("grid", side, s)
        yield f"er{20 + s % 3}_d{(8, 16)[s % 2]}_s{s}", ("er", 20 + s % 3, (8, 16)[s % 2], s)


def make_graph(spec):
    kind = spec[0]
    if kind == "rmat":
        _, scale, ef, s = spec
        return B.Graph.gen_rmat_device(scale, ef, seed=s), None
    if kind == "grid":
        _, side, s = spec
        h = B.gen_grid(side, side, 0.05, s)
    else:
        _, lg, deg, s = spec
        h = B.gen_er(1 << lg, float(deg), s)
    return B.Graph.upload(h, validate=False), h


def record(dg, roots, reps, max_per_root=None):
    feats, times, meta = [], [], []
    for r in roots:
        samples = dg.sched_record(int(r), ipt=4, reps=reps)
        f, t, m = B.samples_to_arrays(samples)
        if max_per_root and len(f) > max_per_root:
            keep = np.linspace(0, len(f) - 1, max_per_root).astype(int)
            f, t, m = f[keep], t[keep], m[keep]
        feats.append(f)
        times.append(t)
        meta.append(m)
    return np.concatenate(feats), np.concatenate(times), np.concatenate(meta)


def regret_report(weights, f, t):
    arms, conf = B.sched_predict(weights, f)
    best = t.min(axis=1)
    chosen = t[np.arange(len(t)), arms]
    llb = t[:, FIXED_LLB]
    return {
        "levels": int(len(t)),
        "explore_ms_best": float(best.sum()),
        "explore_ms_learned": float(chosen.sum()),
        "explore_ms_fixed_llb256": float(llb.sum()),
        "regret_ms": float((chosen - best).sum()),
        "regret_frac_of_best": float((chosen - best).sum() / best.sum()),
        "speedup_vs_fixed_llb": float(llb.sum() / chosen.sum()),
        "levels_with_best_arm": float((chosen <= best * 1.0 + 1e-9).mean()),
        "arm_histogram": {B.ARM_NAMES[a]: int((arms == a).sum()) for a in range(9)
                          if (arms == a).any()},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None, help="directory for the recorded samples")
    ap.add_argument("--quick", action="store_true", help="3 seeds instead of 20")
    ap.add_argument("--epochs", type=int, default=3000)
    a = ap.parse_args()
    import torch
    torch.cuda.set_device(0)
    t0 = time.time()
    F, T, M, names = [], [], [], []
    for name, spec in training_graphs(a.quick):
        dg, h = make_graph(spec)
        host = h if h is not None else dg.download()
        is_grid = spec[0] == "grid"
        roots = B.sample_roots(host, 1 if is_grid else 2, spec[-1])
        f, t, m = record(dg, roots, reps=2 if is_grid else 3,
                         max_per_root=200 if is_grid else None)
        F.append(f)
        T.append(t)
        M.append(m)
        names.append((name, len(f)))
        dg.free()
        print(f"recorded {name}: {len(f)} levels", flush=True)
    F, T, M = np.concatenate(F), np.concatenate(T), np.concatenate(M)
    rec_s = time.time() - t0
    if a.out:
        os.makedirs(a.out, exist_ok=True)
        np.savez_compressed(os.path.join(a.out, "sched_train_samples.npz"), features=F,
                            arm_ms=T, meta=M)
    t1 = time.time()
    w, loss = B.sched_train(F, T, epochs=a.epochs, lr=3e-3, seed=1)
    train_s = time.time() - t1
    train_rep = regret_report(w, F, T)
    print("train", json.dumps(train_rep), flush=True)

    held = {}
    for name, spec in (("rmat25_ef16_s5", ("rmat", 25, 16, 5)),
                       ("rmat23_ef16_s2", ("rmat", 23, 16, 2))):
        dg, _ = make_graph(spec)
        host = dg.download()
        roots = B.sample_roots(host, 3, spec[-1] + 100)
        f, t, m = record(dg, roots, reps=3)
        held[name] = regret_report(w, f, t)
        # end-to-end: learned vs fixed LLB/256 in the device level loop
        lv = torch.empty(dg.n_cols, dtype=torch.int32, device="cuda")
        dg.sched_attach(w)
        res = {}
        for label, o in (("learned", B.options("learned")), ("fixed_llb256", B.options("llb"))):
            dg.run_device(int(roots[0]), lv.data_ptr(), opts=o)
            ms = [dg.run_device(int(r), lv.data_ptr(), opts=o).device_ms for r in roots]
            res[label + "_bfs_ms"] = float(np.mean(ms))
        res["bfs_speedup_learned_vs_llb"] = res["fixed_llb256_bfs_ms"] / res["learned_bfs_ms"]
        held[name].update(res)
        if a.out:
            np.savez_compressed(os.path.join(a.out, f"sched_eval_{name}.npz"), features=f,
                                arm_ms=t, meta=m)
        dg.free()
        print("held-out", name, json.dumps(held[name]), flush=True)

    w.astype("<f4").tofile(WEIGHTS)
    report = {"params": int(w.size), "layout": "W1[32][5] b1[32] W2[32][32] b2[32] W3[9][32] b3[9]",
              "arms": B.ARM_NAMES, "train_graphs": names, "train_levels": int(len(F)),
              "epochs": a.epochs, "final_loss": loss, "record_s": rec_s, "train_s": train_s,
              "train": train_rep, "held_out": held}
    with open(REPORT, "w") as fh:
        json.dump(report, fh, indent=1)
    print(json.dumps({"final_loss": loss, "train_s": train_s, "record_s": rec_s}))


if __name__ == "__main__":
    main()
