"""GPU tests of the multi-source and batched forms.

A batch packs member graphs into one disjoint union and runs one
multi-source BFS and SSSP over it; every member's slice of the result must
be bit-exact with the oracle's single-graph answer from that member's
source, on the first run and on every replay of the captured CUDA graph.
"""
import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

pytestmark = pytest.mark.gpu


def _weighted_rmat(V, ef, seed):
    g = gg.rmat(V, ef, seed=seed)
    return g.with_weights(gg.uniform_weights(g, 1, 255, seed))


@pytest.mark.parametrize("barrier", [gdb.BARRIER_XF, gdb.BARRIER_XF_FIXED, gdb.BARRIER_GRID_SYNC])
def test_multi_source_is_min_over_sources(barrier):
    g = _weighted_rmat(1 << 13, 12, 21)
    srcs = [int(s) for s in gg.sources(g, 5, seed=4)] + [7, 7]   # duplicates are harmless
    with gdb.Ctx(barrier=barrier) as c:
        G = c.graph(g.row_ptr, g.col, g.w)
        want_b = np.minimum.reduce([oracle.bfs(g, s) for s in srcs])
        want_s = np.minimum.reduce([oracle.sssp_worklist(g, s) for s in srcs])
        assert np.array_equal(c.bfs_multi(G, srcs), want_b)
        assert np.array_equal(c.sssp_multi(G, srcs), want_s)


def test_multi_source_needs_persistent_barrier():
    g = _weighted_rmat(1 << 10, 8, 2)
    with gdb.Ctx(barrier=gdb.BARRIER_RELAUNCH_GRAPH) as c:
        G = c.graph(g.row_ptr, g.col, g.w)
        with pytest.raises(gdb.GdbError) as e:
            c.sssp_multi(G, [0, 1])
        assert e.value.status == -7
        with pytest.raises(gdb.GdbError) as e:
            c.bfs_multi(G, [0, 1])
        assert e.value.status == -7


def _member_checks(batch_graphs, off, res, srcs):
    for i, g in enumerate(batch_graphs):
        a, b = int(off[i]), int(off[i + 1])
        want_b = oracle.bfs(g, srcs[i])
        want_s = oracle.sssp_worklist(g, srcs[i])
        # unreached stays GDB_LONESTAR_INF; reached levels are member-local
        assert np.array_equal(res["bfs"][a:b], want_b), (i, g.name)
        assert np.array_equal(res["sssp"][a:b], want_s), (i, g.name)


@pytest.mark.parametrize("schedule", [gdb.SCHED_PLAIN, gdb.SCHED_ADAPTIVE])
def test_batch_matches_single_graph_runs(schedule):
    members = gg.mixed_batch(24, 50, 20000, seed=3)
    srcs = [g.meta["source"] for g in members]
    with gdb.Ctx(schedule=schedule) as c:
        U = c.graph_batch(members)
        off = U.vertex_offset
        assert int(off[-1]) == sum(g.V for g in members)
        usrc = [int(off[i]) + s for i, s in enumerate(srcs)]
        with c.batch(U, usrc) as B:
            for _ in range(3):  # first run and replays of the captured graph
                ms = B.run()
                assert ms > 0
                _member_checks(members, off, B.results(), srcs)
            arcs_b, steps_b = B.app_stats(gdb.BATCH_BFS)
            assert arcs_b > 0 and steps_b >= 1
        # the same members through the single-graph entry points
        for i in (0, 1, 5):
            G = c.graph(members[i].row_ptr, members[i].col, members[i].w)
            assert np.array_equal(c.bfs(G, srcs[i]), oracle.bfs(members[i], srcs[i]))
            assert np.array_equal(c.sssp(G, srcs[i]), oracle.sssp_worklist(members[i], srcs[i]))


def test_batch_set_sources_and_single_app():
    members = gg.mixed_batch(8, 200, 5000, seed=11)
    with gdb.Ctx() as c:
        U = c.graph_batch(members)
        off = U.vertex_offset
        srcs = [g.meta["source"] for g in members]
        with c.batch(U, [int(off[i]) + s for i, s in enumerate(srcs)], apps=gdb.BATCH_BFS) as B:
            B.run()
            res = B.results()
            assert "sssp" not in res
            for i, g in enumerate(members):
                assert np.array_equal(res["bfs"][off[i]:off[i + 1]], oracle.bfs(g, srcs[i]))
            srcs2 = [g.V - 1 for g in members]
            B.set_sources([int(off[i]) + s for i, s in enumerate(srcs2)])
            B.run()
            res = B.results()
            for i, g in enumerate(members):
                assert np.array_equal(res["bfs"][off[i]:off[i + 1]], oracle.bfs(g, srcs2[i]))


def test_batch_rejects_bad_arguments():
    members = gg.mixed_batch(4, 100, 400, seed=5)
    with gdb.Ctx() as c:
        U = c.graph_batch(members)
        with pytest.raises(gdb.GdbError):
            c.batch(U, [U.V])               # source out of range
        with pytest.raises(gdb.GdbError):
            c.batch(U, [0], apps=4)         # unknown app bit
        Unw = c.graph_batch(members, weights=False)
        with pytest.raises(gdb.GdbError):
            c.batch(Unw, [0], apps=gdb.BATCH_SSSP)   # SSSP without weights


def test_full_mixed_batch_sampled_members():
    """The benchmark's own batch at full size (512 members, V log-uniform
    in [1e3, 1e6]): one captured replay, then every 16th member and the
    last one against the oracle, BFS and SSSP bit-exact."""
    members = gg.mixed_batch(512, 1000, 1_000_000, seed=1)
    srcs = [g.meta["source"] for g in members]
    with gdb.Ctx() as c:
        U = c.graph_batch(members)
        off = U.vertex_offset
        with c.batch(U, [int(off[i]) + s for i, s in enumerate(srcs)]) as B:
            B.run()
            B.run()  # a replay of the captured graph
            res = B.results()
    sample = sorted(set(range(0, len(members), 16)) | {len(members) - 1})
    for i in sample:
        g, a, b = members[i], int(off[i]), int(off[i + 1])
        assert np.array_equal(res["bfs"][a:b], oracle.bfs(g, srcs[i])), (i, g.name)
        assert np.array_equal(res["sssp"][a:b], oracle.sssp_worklist(g, srcs[i])), (i, g.name)
