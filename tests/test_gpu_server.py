"""GPU tests of the request loop (continuous batching).

Each result computed in the mix -- many requests in flight on several
slots, admitted as slots and pool memory free up -- must equal the same
request run alone: BFS levels and SSSP distances bit-exact (and equal to
the oracle), BC scores within 1e-4 relative (float atomics make their
summation order vary).
"""
import time

import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def _graphs(ctx, n, seed, vmax=20000):
    members = gg.mixed_batch(n, 300, vmax, seed=seed)
    return members, [ctx.graph(m.row_ptr, m.col, m.w) for m in members]


def _alone(ctx, G, app, src):
    if app == gdb.APP_BFS:
        return ctx.bfs(G, src)
    if app == gdb.APP_SSSP:
        return ctx.sssp(G, src)
    return ctx.bc(G, [src])


def _same(app, got, want):
    if app == gdb.APP_BC:
        # float32 path counts overflow on long grids (as in the reference):
        # non-finite entries must match, finite ones agree within RTOL
        fin = np.isfinite(want)
        if not np.array_equal(fin, np.isfinite(got)):
            return False
        g, w = got[fin].astype(np.float64), want[fin].astype(np.float64)
        if w.size == 0:
            return True
        scale = np.maximum(np.abs(w), 1e-6 * max(1.0, float(np.abs(w).max())))
        return bool(np.all(np.abs(g - w) <= RTOL * scale + 1e-6))
    return bool(np.array_equal(got, want))


def test_results_alone_equal_results_in_the_mix(ctx):
    members, Gs = _graphs(ctx, 8, seed=21)
    rng = np.random.default_rng(5)
    reqs = []
    for _ in range(60):
        i = int(rng.integers(len(members)))
        app = int(rng.integers(1, 4))
        reqs.append((i, app, int(rng.integers(members[i].V))))
    with ctx.server(slots=6, pool_bytes=256 << 20) as srv:
        ids = [srv.add_graph(G) for G in Gs]
        sub = {}
        for i, app, s in reqs:
            rid, out = srv.submit(ids[i], app, s)
            sub[rid] = (i, app, s, out)
        srv.drain(120.0)
        done = srv.poll(1000)
    assert len(done) == len(reqs)
    slots = set()
    for d in done:
        assert d["status"] == 0, d
        i, app, s, out = sub[d["id"]]
        slots.add(d["slot"])
        want = _alone(ctx, Gs[i], app, s)
        assert _same(app, out, want), (members[i].name, app, s)
        if app == gdb.APP_BFS:
            assert np.array_equal(out, oracle.bfs(members[i], s))
        elif app == gdb.APP_SSSP:
            assert np.array_equal(out, oracle.sssp_worklist(members[i], s))
    assert len(slots) > 1  # requests really ran on several slots


def test_requests_overlap_on_the_device(ctx):
    members, Gs = _graphs(ctx, 4, seed=8, vmax=200000)
    with ctx.server(slots=8) as srv:
        ids = [srv.add_graph(G) for G in Gs]
        t0 = time.perf_counter()
        sub = {}
        for k in range(32):
            i = k % len(members)
            rid, _ = srv.submit(ids[i], gdb.APP_BFS, members[i].meta["source"])
            sub[rid] = time.perf_counter() - t0
        srv.drain(120.0)
        done = srv.poll(100)
    spans = sorted((sub[d["id"]] * 1e3 + d["queue_ms"], sub[d["id"]] * 1e3 + d["total_ms"]) for d in done)
    overlaps = sum(1 for a, b in zip(spans, spans[1:]) if b[0] < a[1])
    assert overlaps > 0


def test_admission_by_footprint(ctx):
    members, Gs = _graphs(ctx, 1, seed=4)
    m, G = members[0], Gs[0]
    with ctx.server(slots=1) as probe:
        gid = probe.add_graph(G)
        probe.submit(gid, gdb.APP_SSSP, 0)
        probe.drain(60.0)
        fp = probe.poll(1)[0]["footprint"]
    # room for one request at a time: four slots, but admission waits for memory
    with ctx.server(slots=4, pool_bytes=fp * 3 // 2) as srv:
        gid = srv.add_graph(G)
        t0 = time.perf_counter()
        sub = {}
        for k in range(8):
            rid, out = srv.submit(gid, gdb.APP_SSSP, k)
            sub[rid] = (k, out, time.perf_counter() - t0)
        srv.drain(120.0)
        done = srv.poll(100)
        assert len(done) == 8
        spans = []
        for d in done:
            k, out, ts = sub[d["id"]]
            assert d["status"] == 0 and d["footprint"] == fp
            assert np.array_equal(out, oracle.sssp_worklist(m, k))
            spans.append((ts * 1e3 + d["queue_ms"], ts * 1e3 + d["total_ms"]))
        spans.sort()
        assert all(b[0] >= a[1] - 0.05 for a, b in zip(spans, spans[1:]))
        # a request larger than the whole pool is refused at submission
        big = gg.grid(512, 512)
        big = big.with_weights(gg.uniform_weights(big, 1, 9, seed=1))
        Gb = ctx.graph(big.row_ptr, big.col, big.w)
        bid = srv.add_graph(Gb)
        with pytest.raises(gdb.GdbError) as e:
            srv.submit(bid, gdb.APP_BC, 0)
        assert e.value.status == -5


def test_server_learned_schedule(ctx):
    from gpu_discovery_barrier_gb300 import selector

    p = selector.load()
    if p is None:
        pytest.skip("no trained selector weights")
    members, _ = _graphs(ctx, 4, seed=31)
    with gdb.Ctx(schedule=gdb.SCHED_LEARNED) as c:
        c.selector_set(p)
        Gs = [c.graph(m.row_ptr, m.col, m.w) for m in members]
        with c.server(slots=3) as srv:
            ids = [srv.add_graph(G) for G in Gs]
            sub = {}
            for i, m in enumerate(members):
                for app in (gdb.APP_BFS, gdb.APP_SSSP):
                    rid, out = srv.submit(ids[i], app, m.meta["source"])
                    sub[rid] = (i, app, out)
            srv.drain(60.0)
            for d in srv.poll(100):
                i, app, out = sub[d["id"]]
                s = members[i].meta["source"]
                want = oracle.bfs(members[i], s) if app == gdb.APP_BFS else oracle.sssp_worklist(members[i], s)
                assert d["status"] == 0 and np.array_equal(out, want)
