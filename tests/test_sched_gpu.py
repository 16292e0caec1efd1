"""Learned per-level scheduler: recorder, device inference against a PyTorch
fp32 reference of the same MLP, training kernels, and BFS parity whatever the
scheduler picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def torch_mlp(w, x):
    """PyTorch fp32 reference of the scheduler MLP (layout of bfs_gb300.h)."""
    import torch
    w = torch.as_tensor(w, dtype=torch.float32)
    x = torch.as_tensor(x, dtype=torch.float32)
    o = 0
    W1 = w[o:o + 160].view(32, 5); o += 160
    b1 = w[o:o + 32]; o += 32
    W2 = w[o:o + 1024].view(32, 32); o += 1024
    b2 = w[o:o + 32]; o += 32
    W3 = w[o:o + 288].view(9, 32); o += 288
    b3 = w[o:o + 9]; o += 9
    h1 = torch.relu(x @ W1.T + b1)
    h2 = torch.relu(h1 @ W2.T + b2)
    return torch.softmax(h2 @ W3.T + b3, dim=1)


def test_predict_matches_torch_fp32_reference(B):
    torch_cuda()
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.5, B.SCHED_PARAMS).astype(np.float32)
    x = rng.uniform(0, 1, (4096, 5)).astype(np.float32)
    arms, conf = B.sched_predict(w, x)
    p = torch_mlp(w, x).numpy()
    ref_arm = p.argmax(axis=1)
    ref_conf = p.max(axis=1)
    # tolerance: fp32 sums in a different order; argmax may differ only on
    # near ties
    assert np.allclose(conf, ref_conf, rtol=1e-4, atol=1e-5)
    mism = arms != ref_arm
    if mism.any():
        srt = np.sort(p[mism], axis=1)
        assert np.all(srt[:, -1] - srt[:, -2] < 1e-4)


def test_training_learns_a_separable_rule(B):
    """Synthetic per-level costs: arm 4 is fastest when x1 > 0.5, else arm 1."""
    torch_cuda()
    rng = np.random.default_rng(1)
    n = 2000
    x = rng.uniform(0, 1, (n, 5)).astype(np.float32)
    t = np.full((n, 9), 2.0, np.float32)
    good = np.where(x[:, 1] > 0.5, 4, 1)
    t[np.arange(n), good] = 1.0
    w, loss = B.sched_train(x, t, epochs=800, lr=1e-2, seed=3)
    assert np.all(np.isfinite(w))
    arms, _ = B.sched_predict(w, x)
    assert (arms == good).mean() > 0.95
    assert loss < 0.2


def test_recorder_levels_and_times(B):
    torch_cuda()
    g = B.gen_rmat(15, 16, seed=4)
    dg = B.Graph.upload(g)
    r = int(B.sample_roots(g, 1, 4)[0])
    samples = dg.sched_record(r, reps=2)
    f, t, m = B.samples_to_arrays(samples)
    _, _, st = dg.run(r, B.options("glb", 256, record=1))
    tab = st.levels_table()
    fr = [x for x in tab["frontier"] if x > 0]
    assert m[:, 1].tolist() == fr
    assert np.all(t > 0) and np.all(np.isfinite(t))
    assert np.all((f >= 0) & (f <= 1.0))
    # the recorder leaves the BFS result intact: levels equal a plain run
    lv_plain, _, _ = dg.run(r)
    samples = dg.sched_record(r, reps=1)
    lv_after, _, _ = dg.run(r)
    assert np.array_equal(lv_plain, lv_after)
    dg.free()


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_learned_schedule_levels_bit_exact(B, O, loop):
    torch_cuda()
    rng = np.random.default_rng(7)
    g = B.gen_rmat(16, 16, seed=8)
    dg = B.Graph.upload(g)
    roots = B.sample_roots(g, 3, 8)
    # untrained: every level falls back to LLB/256
    lv, _, st = dg.run(int(roots[0]), B.options("learned", loop=loop, record=1))
    ref, ec = O.oracle_bfs(g.indptr, g.inds, int(roots[0]))
    assert np.array_equal(lv, ref) and st.edges_count == ec
    arms = [a for a, f in zip(st.levels_table()["arm"], st.levels_table()["frontier"]) if f]
    assert set(arms) == {1}
    # random weights: arbitrary arms, same levels
    for trial in range(3):
        w = rng.normal(0, 1.0, B.SCHED_PARAMS).astype(np.float32)
        dg.sched_attach(w)
        for r in roots:
            lv, pa, st = dg.run(int(r), B.options("learned", loop=loop, record=1), parents=True)
            ref, ec = O.oracle_bfs(g.indptr, g.inds, int(r))
            assert np.array_equal(lv, ref) and st.edges_count == ec
        tab = st.levels_table()
        used = [a for a, f in zip(tab["arm"], tab["frontier"]) if f]
        assert all(0 <= a < 9 for a in used)
    # a confidence threshold above 1 forces the fallback arm
    dg.sched_attach(w, min_confidence=1.5)
    lv, _, st = dg.run(int(roots[0]), B.options("learned", loop=loop, record=1))
    tab = st.levels_table()
    assert set(a for a, f in zip(tab["arm"], tab["frontier"]) if f) == {1}
    dg.free()


def test_device_choice_equals_batch_prediction(B):
    """The arms picked inside the level loop are the MLP's argmax on the
    level's features (recorded independently)."""
    torch_cuda()
    rng = np.random.default_rng(9)
    g = B.gen_rmat(16, 8, seed=10)
    dg = B.Graph.upload(g)
    r = int(B.sample_roots(g, 1, 10)[0])
    w = rng.normal(0, 1.0, B.SCHED_PARAMS).astype(np.float32)
    samples = dg.sched_record(r, reps=1)
    f, _, m = B.samples_to_arrays(samples)
    pred, _ = B.sched_predict(w, f)
    dg.sched_attach(w)
    _, _, st = dg.run(r, B.options("learned", record=1))
    tab = st.levels_table()
    used = [a for a, fr in zip(tab["arm"], tab["frontier"]) if fr]
    assert used == pred.tolist()
    dg.free()


def test_graph_loop_runs_every_arm_exactly(B, O):
    """A model whose output bias forces one arm runs that arm on every level
    of the CUDA-graph loop (the one kernel that serves any arm), with and
    without parents; levels, edge counts and parents are exact."""
    torch_cuda()
    graphs = [B.gen_rmat(15, 16, seed=21), B.gen_grid(96, 64, 0.05, 22)]
    b3 = B.SCHED_PARAMS - B.SCHED_ARMS  # output bias offset (last 9 parameters)
    for g in graphs:
        dg = B.Graph.upload(g)
        roots = B.sample_roots(g, 2, 23)
        refs = [O.oracle_bfs(g.indptr, g.inds, int(r)) for r in roots]
        for arm in range(B.SCHED_ARMS):
            w = np.zeros(B.SCHED_PARAMS, np.float32)
            w[b3 + arm] = 10.0
            dg.sched_attach(w)
            for r, (ref, ec) in zip(roots, refs):
                lv, pa, st = dg.run(int(r), B.options("learned", record=1), parents=True)
                assert np.array_equal(lv, ref) and st.edges_count == ec, (arm, int(r))
                tab = st.levels_table()
                assert set(a for a, f in zip(tab["arm"], tab["frontier"]) if f) == {arm}
                reached = lv >= 0
                assert pa[int(r)] == int(r)
                kids = np.flatnonzero(reached & (lv > 0))
                assert np.all(lv[pa[kids]] == lv[kids] - 1)
                lv2, _, _ = dg.run(int(r), B.options("learned"))
                assert np.array_equal(lv2, ref)
        dg.free()
