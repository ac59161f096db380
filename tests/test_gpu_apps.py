"""GPU parity of every application entry point against the CPU oracle.

Integer results (BFS levels, SSSP distances, MIS set, colours, MST weight /
edge count / edge set) must be bit-exact; BC float32 scores must be within
1e-4 relative of the oracle's float32 restatement and of the FP64 Brandes
oracle (RTOL below).  Calls go through the C ABI (gdb.Ctx -> libgdb.so).
"""
import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

pytestmark = pytest.mark.gpu

RTOL = 1e-4  # BC tolerance stated by the parity contract


def graphs():
    out = [
        ("grid16", gg.grid(16, 16)),
        ("grid256x256", gg.grid(256, 256)),
        ("rmat12", gg.rmat(1 << 12, 16, seed=5)),
        ("rmat14_hubs", gg.rmat(1 << 14, 32, seed=6)),
        ("grid3x1000", gg.grid(3, 1000)),
    ]
    # star: one hub of degree 3000 (heavy chunks) plus isolated vertices
    V = 5000
    pairs = [(0, i) for i in range(1, 3001)] + [(3001, 3002), (3002, 3003)]
    out.append(("star_isolated", gg.from_edges(V, pairs)))
    out.append(("path", gg.from_edges(400, [(i, i + 1) for i in range(399)])))
    out.append(("single", gg.from_edges(1, [])))
    out.append(("pair", gg.from_edges(2, [(0, 1)])))
    return out


GRAPHS = graphs()
IDS = [n for n, _ in GRAPHS]


def bc_close(got, want):
    scale = np.maximum(np.abs(want), 1e-6 * max(1.0, float(np.max(np.abs(want))) if want.size else 1.0))
    return np.all(np.abs(got.astype(np.float64) - want) <= RTOL * scale + 1e-6)


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_bfs(ctx, name, g):
    G = ctx.graph(g.row_ptr, g.col)
    for src in sorted(set([0, g.V - 1] + list(gg.sources(g, 3, seed=7)))):
        got = ctx.bfs(G, int(src))
        assert np.array_equal(got, oracle.bfs(g, int(src))), (name, src)


@pytest.mark.parametrize("barrier", [gdb.BARRIER_XF, gdb.BARRIER_GRID_SYNC, gdb.BARRIER_RELAUNCH,
                                     gdb.BARRIER_RELAUNCH_GRAPH])
@pytest.mark.parametrize("schedule", [gdb.SCHED_PLAIN, gdb.SCHED_ADAPTIVE])
def test_bfs_barrier_kinds(barrier, schedule):
    if barrier in (gdb.BARRIER_RELAUNCH, gdb.BARRIER_RELAUNCH_GRAPH) and schedule == gdb.SCHED_ADAPTIVE:
        pytest.skip("adaptive needs a persistent barrier")
    g = gg.rmat(1 << 13, 16, seed=9)
    with gdb.Ctx(barrier=barrier, schedule=schedule) as c:
        G = c.graph(g.row_ptr, g.col)
        for src in gg.sources(g, 3, seed=1):
            assert np.array_equal(c.bfs(G, int(src)), oracle.bfs(g, int(src)))


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_sssp_worklist(ctx, name, g):
    w = gg.uniform_weights(g, 1, 255, seed=1)
    gw = g.with_weights(w)
    G = ctx.graph(g.row_ptr, g.col, w)
    for src in sorted(set([0] + list(gg.sources(g, 2, seed=3)))):
        got = ctx.sssp(G, int(src))
        assert np.array_equal(got, oracle.sssp_worklist(gw, int(src))), (name, src)


@pytest.mark.parametrize("barrier", [gdb.BARRIER_XF, gdb.BARRIER_GRID_SYNC, gdb.BARRIER_RELAUNCH,
                                     gdb.BARRIER_RELAUNCH_GRAPH])
def test_sssp_barrier_kinds(barrier):
    g = gg.grid(64, 64)
    w = gg.uniform_weights(g, 1, 1000, seed=1)
    with gdb.Ctx(barrier=barrier) as c:
        G = c.graph(g.row_ptr, g.col, w)
        assert np.array_equal(c.sssp(G, 0), oracle.sssp_worklist(g.with_weights(w), 0))


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
@pytest.mark.parametrize("delta", [1, 37, 300, 1 << 20])
@pytest.mark.parametrize("split", [0, -1, 1])
def test_sssp_near_far(name, g, delta, split):
    """The near-far schedule reaches the same distances for every bucket
    width, with and without the light/heavy arc split."""
    w = gg.uniform_weights(g, 1, 255, seed=1)
    gw = g.with_weights(w)
    with gdb.Ctx(sssp_delta=delta, sssp_split=split) as c:
        G = c.graph(g.row_ptr, g.col, w)
        for src in sorted(set([0] + list(gg.sources(g, 2, seed=3)))):
            got = c.sssp(G, int(src))
            assert np.array_equal(got, oracle.sssp_worklist(gw, int(src))), (name, src, delta)
            st = c.last_stats()
            assert st["sssp_delta"] == delta
            # automatic: split only when some arc is at least as heavy as the width
            on = split == 1 or (split == 0 and g.E > 0 and delta <= int(w.max()))
            assert st["sssp_light"] == (delta if on else 0)


@pytest.mark.parametrize("split", [-1, 1])
def test_sssp_split_skips_heavy_rework(split):
    """On R-MAT with U[1,255] weights the split relaxes far fewer arcs than
    plain near-far at the same width (heavy arcs once per vertex)."""
    g = gg.rmat(1 << 15, 16, seed=21)
    w = gg.uniform_weights(g, 1, 255, seed=4)
    want = oracle.sssp_worklist(g.with_weights(w), 3)
    with gdb.Ctx(sssp_delta=32, sssp_split=split) as c:
        G = c.graph(g.row_ptr, g.col, w)
        assert np.array_equal(c.sssp(G, 3), want)
        st = c.last_stats()
    reached = int(np.diff(g.row_ptr.astype(np.int64))[want < gdb.LONESTAR_INF].sum())
    if split == 1:
        assert st["edges_processed"] < 1.5 * reached, (st, reached)
    else:
        assert st["edges_processed"] > 1.5 * reached, (st, reached)


def test_sssp_split_on_a_declared_symmetric_graph():
    """A graph declared symmetric (one weight per undirected edge) pulls
    over its own heavy half instead of a transposed copy: the same
    distances, and undeclaring rebuilds the partition with the transpose."""
    g = gg.rmat(1 << 14, 16, seed=31)
    w = gg.uniform_weights(g, 1, 255, seed=6)
    gw = g.with_weights(w)
    with gdb.Ctx(schedule=gdb.SCHED_ADAPTIVE) as c:
        G = c.graph(g.row_ptr, g.col, w, symmetric=True)
        for delta in (8, 32, 0):
            c.set_options(sssp_delta=delta)
            for src in (0, 17):
                assert np.array_equal(c.sssp(G, src), oracle.sssp_worklist(gw, src)), (delta, src)
        G.set_symmetric(False)
        assert np.array_equal(c.sssp(G, 3), oracle.sssp_worklist(gw, 3))
        G.set_symmetric(True)
        assert np.array_equal(c.sssp(G, 3), oracle.sssp_worklist(gw, 3))


def test_sssp_split_zero_and_infinite_weights():
    """Weight-0 arcs are light, arcs of weight >= 1e9 are never relaxed --
    in near and settle supersteps alike."""
    g = gg.rmat(1 << 12, 12, seed=5)
    rng = np.random.default_rng(6)
    w = rng.integers(0, 400, g.E).astype(np.uint32)
    w[rng.random(g.E) < 0.1] = 0
    w[rng.random(g.E) < 0.05] = gdb.LONESTAR_INF
    w[rng.random(g.E) < 0.02] = 4_000_000_000
    gw = g.with_weights(w)
    for delta in (1, 16, 200):
        with gdb.Ctx(sssp_delta=delta, sssp_split=1) as c:
            G = c.graph(g.row_ptr, g.col, w)
            for src in (0, 7, 100):
                assert np.array_equal(c.sssp(G, src), oracle.sssp_worklist(gw, src)), (delta, src)


@pytest.mark.parametrize("barrier", [gdb.BARRIER_XF, gdb.BARRIER_GRID_SYNC])
def test_sssp_near_far_auto_width(barrier):
    g = gg.grid(96, 80)
    w = gg.uniform_weights(g, 1, 1000, seed=1)
    with gdb.Ctx(barrier=barrier, schedule=gdb.SCHED_ADAPTIVE) as c:
        G = c.graph(g.row_ptr, g.col, w)
        got = c.sssp(G, 0)
        st = c.last_stats()
        assert np.array_equal(got, oracle.sssp_worklist(g.with_weights(w), 0))
        # 32 x mean weight (~500) / mean degree (~4)
        assert 2000 < st["sssp_delta"] < 6000
        assert st["phases"] > 1
        # weights replaced: the width follows the new mean
        w2 = gg.uniform_weights(g, 1, 10, seed=2)
        G.set_weights(w2)
        assert np.array_equal(c.sssp(G, 5), oracle.sssp_worklist(g.with_weights(w2), 5))
        assert c.last_stats()["sssp_delta"] < 100


def test_sssp_near_far_multi_source():
    g = gg.rmat(1 << 12, 16, seed=8)
    w = gg.uniform_weights(g, 1, 255, seed=8)
    srcs = [int(s) for s in gg.sources(g, 4, seed=1)]
    want = np.minimum.reduce([oracle.sssp_worklist(g.with_weights(w), s) for s in srcs])
    for split in (-1, 1):
        with gdb.Ctx(sssp_delta=50, sssp_split=split) as c:
            G = c.graph(g.row_ptr, g.col, w)
            assert np.array_equal(c.sssp_multi(G, srcs), want)


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_sssp_jacobi(ctx, name, g):
    w = gg.uniform_weights(g, 1, 100, seed=2)
    gw = g.with_weights(w)
    G = ctx.graph(g.row_ptr, g.col, w)
    got = ctx.sssp_jacobi(G, 0)
    assert np.array_equal(got, oracle.sssp_jacobi(gw, 0, literal=True)), name


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_mis(ctx, name, g):
    prio = gg.priorities(g.V, seed=4)
    G = ctx.graph(g.row_ptr, g.col)
    got = ctx.mis(G, prio)
    want, _ = oracle.mis(g, prio)
    assert np.array_equal(got, want), name


STUCK_MIS = [
    # adjacent vertices of equal priority: neither is below the other
    ("equal_pair", gg.from_edges(2, [(0, 1)]), [0.5, 0.5]),
    # equal priorities in a triangle, next to a path that does finish
    ("equal_triangle", gg.from_edges(6, [(0, 1), (1, 2), (2, 0), (3, 4), (4, 5)]),
     [0.25, 0.25, 0.25, 0.1, 0.2, 0.3]),
    # a NaN priority, of either sign, never wins: an isolated vertex with
    # one stays undecided (a neighbour's win would decide it)
    ("nan", gg.from_edges(3, [(1, 2)]), np.array([0x7FC00000, 0x3E99999A, 0x3E4CCCCD], np.uint32).view(np.float32)),
    ("negative_nan", gg.from_edges(3, [(1, 2)]),
     np.array([0xFFC00000, 0x3E99999A, 0x3E4CCCCD], np.uint32).view(np.float32)),
    # a priority of BIGNUM (99999999) or above never wins
    ("bignum", gg.from_edges(3, [(0, 1), (1, 2)]), [5e8, 99999999.0, 2e8]),
]


@pytest.mark.parametrize("kind", [gdb.BARRIER_XF, gdb.BARRIER_RELAUNCH, gdb.BARRIER_RELAUNCH_GRAPH],
                         ids=["xf", "relaunch", "relaunch_graph"])
@pytest.mark.parametrize("name,g,prio", STUCK_MIS, ids=[n for n, _, _ in STUCK_MIS])
def test_mis_stops_when_a_round_chooses_nobody(ctx, kind, name, g, prio):
    """Inputs on which the reference's MIS loops forever (no vertex of some
    round is below all of its undecided neighbours) end the call with
    GDB_ERR_INVALID at that round, on every barrier form; the context stays
    usable."""
    ctx.set_options(barrier=kind)
    try:
        G = ctx.graph(g.row_ptr, g.col)
        with pytest.raises(gdb.GdbError) as e:
            ctx.mis(G, np.asarray(prio, np.float32))
        assert e.value.status == -1, str(e.value)
        ok = gg.priorities(g.V, seed=4)
        assert np.array_equal(ctx.mis(G, ok), oracle.mis(g, ok)[0])
    finally:
        ctx.set_options(barrier=gdb.BARRIER_XF)


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_color(ctx, name, g):
    prio = gg.priorities(g.V, seed=5)
    G = ctx.graph(g.row_ptr, g.col)
    got = ctx.color(G, prio)
    want, _ = oracle.color(g, prio)
    assert np.array_equal(got, want), name


def test_color_waiting_counts_around_chunk_size(ctx):
    """The colouring enters a coloured vertex as chunks (kChunk = 128
    arcs) when more than 128 neighbours wait for it, else as one light
    entry.  Hubs of degree 300 whose waiting neighbours number 1, 127, 128,
    129, 255, 256, 257 and 299 (each neighbour also has a second arc, to a
    shared anchor, so that it looks at its neighbours)."""
    ks = [1, 127, 128, 129, 255, 256, 257, 299]
    deg = 300
    rng = np.random.default_rng(3)
    V = 1 + len(ks) * (deg + 1)
    pairs, prio = [], np.zeros(V, np.float32)
    # distinct even integers below 2**24 for every vertex, so that each
    # hub's priority can sit strictly between two of its neighbours'
    vals = 2 * rng.permutation(V).astype(np.int64)
    prio[:] = vals
    for i, k in enumerate(ks):
        h = 1 + i * (deg + 1)
        us = np.arange(h + 1, h + 1 + deg)
        pairs += [(h, int(u)) for u in us] + [(int(u), 0) for u in us]
        pu = np.sort(vals[us])
        prio[h] = np.float32(pu[k - 1] + 1) if k < deg else np.float32(pu[-1] + 1)
    assert len(np.unique(prio)) == V
    g = gg.from_edges(V, pairs)
    G = ctx.graph(g.row_ptr, g.col)
    got = ctx.color(G, prio)
    want, _ = oracle.color(g, prio)
    assert np.array_equal(got, want)
    for i, k in enumerate(ks):
        h = 1 + i * (deg + 1)
        us = np.arange(h + 1, h + 1 + deg)
        assert int((prio[us] <= prio[h]).sum()) == k


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_bc(ctx, name, g):
    """Path counts are float32 as in the reference (bc_kernel.cl rho); on
    long grids they overflow (C(510,255) ~ 1e152 on 256x256), making the
    reference's own scores inf/NaN.  Where the float32 oracle is finite the
    GPU must be within RTOL of it and of the FP64 oracle; where it is not,
    the GPU result must not be finite either."""
    srcs = gg.sources(g, 4, seed=8) if g.E else np.array([0], dtype=np.uint32)
    G = ctx.graph(g.row_ptr, g.col)
    got = ctx.bc(G, srcs)
    want32 = oracle.bc_f32(g, g, srcs).astype(np.float64)
    want64 = oracle.bc_f64(g, srcs)
    fin = np.isfinite(want32)
    assert bc_close(got[fin], want64[fin]), name
    assert bc_close(got[fin], want32[fin]), name
    assert not np.any(np.isfinite(got[~fin])), name


@pytest.mark.parametrize("n", [1, 3, 7, 17])
@pytest.mark.parametrize("schedule", [gdb.SCHED_PLAIN, gdb.SCHED_ADAPTIVE])
def test_many_sources_on_lanes(n, schedule):
    """Independent runs of several sources on concurrent lanes: row i is the
    single-source answer of sources[i] (17 sources: more than the 8 lanes of
    BFS and the 16 of SSSP, so lanes run several sources in turn)."""
    g = gg.rmat(1 << 13, 16, seed=41)
    w = gg.uniform_weights(g, 1, 255, seed=7)
    gw = g.with_weights(w)
    srcs = [int(x) for x in gg.sources(g, n, seed=5)]
    with gdb.Ctx(schedule=schedule) as c:
        G = c.graph(g.row_ptr, g.col, w, symmetric=True)
        for _ in range(2):  # lanes are reused
            lv = c.bfs_sources(G, srcs)
            ds = c.sssp_sources(G, srcs)
            for i, s in enumerate(srcs):
                assert np.array_equal(lv[i], oracle.bfs(g, s)), (i, s)
                assert np.array_equal(ds[i], oracle.sssp_worklist(gw, s)), (i, s)
        assert c.last_stats()["launches"] == n


def test_many_sources_device_form_ignores_out_of_range():
    import torch

    g = gg.grid(40, 30)
    w = gg.uniform_weights(g, 1, 9, seed=2)
    with gdb.Ctx() as c:
        G = c.graph(g.row_ptr, g.col, w)
        src = torch.tensor([0, g.V + 5, 17], dtype=torch.int32, device="cuda")
        out = torch.zeros((3, g.V), dtype=torch.int32, device="cuda")
        c.sssp_sources_device(G, src.data_ptr(), 3, out.data_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        gw = g.with_weights(w)
        assert np.array_equal(got[0], oracle.sssp_worklist(gw, 0))
        assert np.all(got[1] == gdb.LONESTAR_INF)
        assert np.array_equal(got[2], oracle.sssp_worklist(gw, 17))
        with pytest.raises(gdb.GdbError):
            c.sssp_sources(G, [0, g.V])


def test_bc_device_form_ignores_out_of_range_sources(ctx):
    """gdb_bc_device skips a source >= V (it adds nothing), as the BFS and
    SSSP device forms do; gdb_bc refuses one."""
    import torch

    g = gg.rmat(1 << 12, 16, seed=5)
    G = ctx.graph(g.row_ptr, g.col)
    want = ctx.bc(G, [0, 3, 77])
    for srcs in ([0, g.V + 5, 3, 77], [g.V, 0, 3, 77, 0xFFFFFFFF]):
        d_src = torch.tensor(np.array(srcs, np.uint32).view(np.int32), device="cuda")
        out = torch.zeros(g.V, dtype=torch.float32, device="cuda")
        ctx.bc_device(G, d_src.data_ptr(), len(srcs), out.data_ptr())
        torch.cuda.synchronize()
        assert bc_close(out.cpu().numpy(), want.astype(np.float64)), srcs
    with pytest.raises(gdb.GdbError):
        ctx.bc(G, [0, g.V])


@pytest.mark.parametrize("case", ["column_out_of_range", "row_decreases"])
@pytest.mark.parametrize("device", [False, True], ids=["host_arrays", "device_arrays"])
def test_graph_refuses_a_malformed_csr(ctx, case, device):
    """A CSR that the kernels would read or write out of bounds -- a column
    naming a vertex >= V, or a row pointer that decreases (row_ptr[0] = 0
    and row_ptr[V] = E still hold) -- is refused at creation with
    GDB_ERR_INVALID; the context stays usable."""
    import torch

    if case == "column_out_of_range":
        row = np.array([0, 2, 3, 4], np.uint32)
        col = np.array([1, 2, 0, 3], np.uint32)   # vertex 3 of V = 3
    else:
        row = np.array([0, 3, 1, 4], np.uint32)   # 3 > 1
        col = np.array([1, 2, 0, 0], np.uint32)
    with pytest.raises(gdb.GdbError) as e:
        if device:
            d_row = torch.tensor(row.view(np.int32), device="cuda")
            d_col = torch.tensor(col.view(np.int32), device="cuda")
            gdb.Graph(ctx, (d_row.data_ptr(), len(row)), (d_col.data_ptr(), len(col)), device=True)
        else:
            ctx.graph(row, col)
    assert e.value.status == -1, str(e.value)
    g = gg.grid(8, 8)
    assert np.array_equal(ctx.bfs(ctx.graph(g.row_ptr, g.col), 0), oracle.bfs(g, 0))


@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_mst(ctx, name, g):
    uw = gg.unique_weights(g, seed=9)
    gu = g.with_weights(uw)
    G = ctx.graph(g.row_ptr, g.col, uw)
    got = ctx.mst(G, with_arcs=True)
    want = oracle.mst(gu)
    assert got["weight64"] == want["weight64"], name
    assert got["weight32"] == want["weight32"], name
    assert got["edges"] == want["edges"] and got["components"] == want["components"], name
    assert oracle.mst_edge_set(g, got["arc_in_mst"]) == oracle.mst_edge_set(g, want["arc_in_mst"])


def _forest(g, arc_in_mst) -> tuple[int, bool]:
    """(undirected edges chosen, whether they form a forest)."""
    edges = oracle.mst_edge_set(g, arc_in_mst)
    parent = list(range(g.V))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for u, v in edges:
        ru, rv = find(u), find(v)
        if ru == rv:
            return len(edges), False
        parent[ru] = rv
    return len(edges), True


def _csr(V, adj):
    """CSR from adjacency lists kept in the given order."""
    row = np.zeros(V + 1, np.uint32)
    row[1:] = np.cumsum([len(a) for a in adj])
    return row, np.array([u for a in adj for u in a], np.uint32)


TIED_MST = [
    ("rmat12_ones", gg.rmat(1 << 12, 16, seed=5), "ones"),
    ("rmat14_hubs_1to3", gg.rmat(1 << 14, 32, seed=6), "1to3"),
    ("grid64_ones", gg.grid(64, 64), "ones"),
    ("grid64_1to3", gg.grid(64, 64), "1to3"),
    ("star_isolated_ones", dict(GRAPHS)["star_isolated"], "ones"),
]


@pytest.mark.parametrize("name,g,kind", TIED_MST, ids=[n for n, _, _ in TIED_MST])
def test_mst_tied_weights(ctx, name, g, kind):
    """Equal weights on different edges: the forest is not unique, so the
    call must give one of the minimum forests -- the oracle's weight, edge
    and component counts, and chosen edges that form a forest."""
    if kind == "ones":
        w = np.ones(g.E, np.uint32)
    else:
        w = (gg.unique_weights(g, seed=13) % 3 + 1).astype(np.uint32)  # one per edge
    G = ctx.graph(g.row_ptr, g.col, w)
    got = ctx.mst(G, with_arcs=True)
    want = oracle.mst(g.with_weights(w))
    assert got["weight64"] == want["weight64"], name
    assert got["edges"] == want["edges"] and got["components"] == want["components"], name
    n, forest = _forest(g, got["arc_in_mst"])
    assert forest and n == got["edges"], name


@pytest.mark.parametrize("adj", [
    [[1, 2], [2, 0], [0, 1]],                       # triangle, each vertex's first arc goes round
    [[1, 3], [2, 0], [3, 1], [0, 2]],               # square, the same way round
], ids=["triangle", "square"])
def test_mst_equal_weights_in_a_ring_order(ctx, adj):
    """Every vertex's lowest arc index points the same way round the ring:
    with equal weights, hooks by arc index alone would close the ring."""
    V = len(adj)
    row, col = _csr(V, adj)
    w = np.full(len(col), 7, np.uint32)
    G = ctx.graph(row, col, w)
    got = ctx.mst(G, with_arcs=True)
    assert got["edges"] == V - 1 and got["components"] == 1
    assert got["weight64"] == 7 * (V - 1)


@pytest.mark.parametrize("name", ["rmat14_hubs", "star_isolated", "grid256x256"])
def test_mst_never_chosen_weights(ctx, name):
    """Arcs of weight >= 1e9 are never chosen (mst_common.cl:84-88): lift
    the heavier half of the unique weights past 1e9, so that components
    whose remaining arcs are all of that kind stop hooking while others
    still do, and every light vertex and heavy chunk meets arcs it must
    skip in every round."""
    g = dict(GRAPHS)[name]
    uw = gg.unique_weights(g, seed=11).astype(np.uint64)
    half = uw > (uw.max() // 2 if len(uw) else 0)
    uw = np.where(half, uw + 1_000_000_000, uw).astype(np.uint32)
    gu = g.with_weights(uw)
    G = ctx.graph(g.row_ptr, g.col, uw)
    got = ctx.mst(G, with_arcs=True)
    want = oracle.mst(gu)
    assert got["weight64"] == want["weight64"], name
    assert got["weight32"] == want["weight32"], name
    assert got["edges"] == want["edges"] and got["components"] == want["components"], name
    assert oracle.mst_edge_set(g, got["arc_in_mst"]) == oracle.mst_edge_set(g, want["arc_in_mst"])
    assert want["edges"] < g.V - 1, "some components must stay apart"
