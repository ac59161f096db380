"""GPU tests of the schedule selector.

* The CUDA forward and backward kernels against the FP64 CPU oracle
  (oracle/mlp.py), and the determinism of the gradient reduction.
* Training on the GPU lowers the loss.
* Schedules chosen by the network never change a result: BFS levels and
  SSSP distances stay bit-identical to the oracle's.
* The trained network gains over the plain schedule on held-out traces.
"""
import numpy as np
import pytest

import oracle
from oracle import mlp as omlp
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg, selector

pytestmark = pytest.mark.gpu


def _rand_problem(n, seed):
    rng = np.random.default_rng(seed)
    p = omlp.init(seed, shift=rng.normal(0, 1, 12), scale=rng.uniform(0.5, 2, 12))
    x = rng.normal(0, 1.5, (n, 12)).astype(np.float32)
    t = rng.normal(0, 1, (n, 6)).astype(np.float32)
    m = (rng.random((n, 6)) < 0.6).astype(np.float32)
    return p, x, t, m


def test_forward_matches_oracle(ctx):
    p, x, _, _ = _rand_problem(301, 1)
    got = ctx.mlp_forward(p, x)
    want = omlp.forward(p, x)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("n", [1, 33, 1000])
def test_gradient_matches_oracle(ctx, n):
    p, x, t, m = _rand_problem(n, 2 + n)
    m[0, 0] = 1.0
    loss, g = ctx.mlp_loss_grad(p, x, t, m)
    want_loss, want_g = omlp.loss_grad(p, x, t, m)
    assert abs(loss - want_loss) <= 1e-4 * max(1.0, abs(want_loss))
    assert np.all(g[:24] == 0)
    err = np.linalg.norm(g - want_g) / max(np.linalg.norm(want_g), 1e-12)
    assert err < 1e-4, err
    np.testing.assert_allclose(g, want_g, rtol=1e-3, atol=1e-5)


def test_gradient_is_deterministic(ctx):
    p, x, t, m = _rand_problem(777, 9)
    _, g1 = ctx.mlp_loss_grad(p, x, t, m)
    _, g2 = ctx.mlp_loss_grad(p, x, t, m)
    assert np.array_equal(g1, g2)


def test_training_lowers_the_loss(ctx):
    rng = np.random.default_rng(4)
    x = rng.normal(0, 1, (2000, 12)).astype(np.float32)
    t = np.zeros((2000, 6), np.float32)
    t[:, 0] = x[:, 0] * 2 - x[:, 3]
    t[:, 1] = np.abs(x[:, 1]) + 0.5 * x[:, 5]
    m = np.zeros_like(t)
    m[:, :2] = 1
    p0 = selector.init_params(1, np.zeros(12, np.float32), np.ones(12, np.float32))
    l0, _ = ctx.mlp_loss_grad(p0, x, t, m)
    p, _ = ctx.mlp_train(p0, x, t, m, epochs=1500, lr=3e-3)
    l1, _ = ctx.mlp_loss_grad(p, x, t, m)
    assert l1 < 0.05 * l0, (l0, l1)
    # the trained blob evaluates the same on the device as in the oracle
    np.testing.assert_allclose(ctx.mlp_forward(p, x[:50]), omlp.forward(p, x[:50]), rtol=1e-4, atol=1e-4)


@pytest.fixture(scope="module")
def trained():
    """Traces of small synthetic graphs, a network trained on the GPU from
    them, and held-out traces."""
    graphs = selector.training_graphs(small=True)
    fit = [g for i, g in enumerate(graphs) if i % 4 != 3]
    held = [g for i, g in enumerate(graphs) if i % 4 == 3]
    with gdb.Ctx() as c:
        bfs_fit, sssp_fit = selector.collect(c, fit)
        bfs_held, sssp_held = selector.collect(c, held)
        settle_fit = selector.collect_settle(c, fit)
        X, T, M = selector.dataset(bfs_fit, sssp_fit, settle_fit)
        p, info = selector.train(c, X, T, M, epochs=2000)
    return p, info, (bfs_fit, sssp_fit), (bfs_held, sssp_held)


def test_settle_traces_are_schedule_independent(ctx):
    """Every settle superstep pushed or every one pulled: the same
    distances, the same settle supersteps and features (decision kind 3)."""
    g = gg.rmat(1 << 14, 16, seed=7)
    w = gg.uniform_weights(g, 1, 255, seed=2)
    want = oracle.sssp_worklist(g.with_weights(w), 3)
    with gdb.Ctx(schedule=gdb.SCHED_ADAPTIVE) as c:
        G = c.graph(g.row_ptr, g.col, w)
        d0, x0, m0, us0 = c.sssp_trace(G, 3, 0)
        d1, x1, m1, us1 = c.sssp_trace(G, 3, 1)
    assert np.array_equal(d0, want) and np.array_equal(d1, want)
    assert len(x0) == len(x1) > 0
    np.testing.assert_array_equal(x0, x1)
    assert np.all(x0[:, 9] == 3)
    assert np.all(m0 == 0) and np.all(m1 == 1)
    assert np.all(us0 > 0) and np.all(us1 > 0)


def test_learned_settle_keeps_distances():
    """The shipped network decides every settle direction inside the
    kernel; distances stay exact on R-MAT (split on) and grids."""
    p = selector.load()
    assert p is not None, "selector_weights.json missing"
    with gdb.Ctx(schedule=gdb.SCHED_LEARNED) as c:
        c.selector_set(p)
        for g, hi in ((gg.rmat(1 << 15, 16, seed=12), 255), (gg.grid(200, 150), 1000),
                      (gg.rmat(5000, 8, seed=3), 255)):
            w = gg.uniform_weights(g, 1, hi, seed=5)
            G = c.graph(g.row_ptr, g.col, w, symmetric=True)
            for s in (0, g.V // 3):
                assert np.array_equal(c.sssp(G, s), oracle.sssp_worklist(g.with_weights(w), s))
            _, x, modes, _ = c.sssp_trace(G, 0, 2)
            assert len(modes) == len(x)


def test_settle_selector_is_bounded_by_the_rule():
    """The shipped network on the settle supersteps of graphs outside its
    training set: its push / pull choices cost at most a little more than
    the fixed rule's (timing noise on microsecond supersteps allowed)."""
    p = selector.load()
    assert p is not None, "selector_weights.json missing"
    graphs = []
    for sc, ef, seed in ((17, 16, 991), (18, 8, 992)):
        g = gg.rmat_scale(sc, ef, seed=seed)
        graphs.append((f"rmat{sc}", g.with_weights(gg.uniform_weights(g, 1, 255, seed=seed)),
                       [int(x) for x in gg.sources(g, 2, seed=seed)]))
    with gdb.Ctx() as c:
        traces = selector.collect_settle(c, graphs, reps=3)
        r = selector.settle_regret(c, p, traces)
    assert r["supersteps"] > 0, r
    assert r["selector_us"] <= 1.10 * r["rule_us"] + 2.0 * r["supersteps"] ** 0.5, r


def test_trace_features_are_schedule_independent(ctx):
    g = gg.rmat(1 << 13, 16, seed=3)
    G = ctx.graph(g.row_ptr, g.col)
    d0, x0, m0, us0 = ctx.bfs_trace(G, 5, 0)
    d1, x1, m1, us1 = ctx.bfs_trace(G, 5, 1)
    assert np.array_equal(d0, oracle.bfs(g, 5)) and np.array_equal(d1, d0)
    assert len(x0) == len(x1) == int(d0[d0 != gdb.LONESTAR_INF].max()) + 1
    assert np.all(m0 == 0) and np.all(m1 == 1)
    np.testing.assert_array_equal(x0[:, [0, 1, 2, 3, 4, 6, 7, 8]], x1[:, [0, 1, 2, 3, 4, 6, 7, 8]])
    assert np.all(us0 > 0) and np.all(us1 > 0)


def test_training_fits_the_traces(trained):
    _, info, _, _ = trained
    assert info["loss_final"] < 0.25 * info["loss_init"], info


def test_learned_schedules_keep_results(trained):
    p = trained[0]
    graphs = [gg.rmat(1 << 14, 16, seed=41), gg.grid(128, 96), gg.rmat(3000, 9, seed=2)]
    with gdb.Ctx(schedule=gdb.SCHED_LEARNED) as c:
        c.selector_set(p)
        for g in graphs:
            w = gg.uniform_weights(g, 1, 255, seed=3)
            G = c.graph(g.row_ptr, g.col, w)
            for s in (0, g.V // 2):
                assert np.array_equal(c.bfs(G, s), oracle.bfs(g, s))
                assert np.array_equal(c.sssp(G, s), oracle.sssp_worklist(g.with_weights(w), s))
        # the batched form under the learned schedule
        members = gg.mixed_batch(6, 200, 4000, seed=13)
        U = c.graph_batch(members)
        off = U.vertex_offset
        srcs = [m.meta["source"] for m in members]
        with c.batch(U, [int(off[i]) + s for i, s in enumerate(srcs)]) as B:
            B.run()
            res = B.results()
        for i, m in enumerate(members):
            assert np.array_equal(res["bfs"][off[i]:off[i + 1]], oracle.bfs(m, srcs[i]))
            assert np.array_equal(res["sssp"][off[i]:off[i + 1]], oracle.sssp_worklist(m, srcs[i]))


def test_learned_needs_a_selector():
    g = gg.grid(8, 8)
    with gdb.Ctx(schedule=gdb.SCHED_LEARNED) as c:
        G = c.graph(g.row_ptr, g.col)
        with pytest.raises(gdb.GdbError):
            c.bfs(G, 0)


def test_selector_gains_over_plain(trained):
    p, _, _, (bfs_held, sssp_held) = trained
    with gdb.Ctx() as c:
        r = selector.regret(c, p, bfs_held, sssp_held)
    b, s = r["bfs"], r["sssp"]
    # on held-out graphs the network is never meaningfully slower than the
    # plain schedule, and where the per-level (per-run) optimum offers a
    # clear gain over it, takes at least half of that gain (the small
    # graphs' runs take about a millisecond: gains of a few per cent are
    # within the timing noise, and a held-out SSSP run of ~1 ms varies by
    # up to ~7 % from one trace collection to the next)
    for d, t_sel, t_plain, t_opt, slack in ((b, "selector_us", "plain_us", "optimal_us", 1.05),
                                            (s, "selector_ms", "plain_ms", "optimal_ms", 1.10)):
        assert d[t_sel] <= slack * d[t_plain], r
        if d[t_plain] > 1.15 * d[t_opt]:
            assert d[t_plain] - d[t_sel] >= 0.5 * (d[t_plain] - d[t_opt]), r
    assert b["regret"] < 0.5, r


def test_learned_bfs_inspects_fewer_arcs():
    """Online, with the shipped network on a graph outside its training set:
    pull levels chosen by the network skip most arcs of the big middle
    levels.  (The network the tests above train on small graphs alone has
    seen too few levels where pull pays to be held to this.)"""
    p = selector.load()
    assert p is not None, "selector_weights.json missing"
    g = gg.rmat(1 << 17, 16, seed=1234)
    with gdb.Ctx() as c:
        c.selector_set(p)
        G = c.graph(g.row_ptr, g.col)
        c.bfs(G, 1)
        plain = c.last_stats()["edges_processed"]
        c.set_options(schedule=gdb.SCHED_LEARNED)
        got = c.bfs(G, 1)
        learned = c.last_stats()["edges_processed"]
    assert np.array_equal(got, oracle.bfs(g, 1))
    assert learned < 0.7 * plain, (learned, plain)


@pytest.mark.parametrize("schedule", [gdb.SCHED_ADAPTIVE, gdb.SCHED_LEARNED])
def test_bounded_degree_graphs_run_push_only(schedule):
    """On a graph whose vertices have at most 8 arcs the direction-optimising
    schedules run the plain push kernel (a pull level can pay only in the
    last few levels, while the hooked kernel costs extra on every level):
    the same arcs inspected as the plain schedule, the same levels."""
    p = selector.load()
    assert p is not None, "selector_weights.json missing"
    g = gg.grid(300, 200)
    with gdb.Ctx() as c:
        c.selector_set(p)
        G = c.graph(g.row_ptr, g.col)
        want = c.bfs(G, 0)
        plain = c.last_stats()["edges_processed"]
        c.set_options(schedule=schedule)
        got = c.bfs(G, 0)
        assert c.last_stats()["edges_processed"] == plain
    assert np.array_equal(got, want)
