"""Relaunch forms of the Pannotia apps: one launch per superstep.

The reference's multi-kernel apps run every superstep as its own launch and
read a stop flag back after it (pannotia/graph_app/sssp/sssp.cpp:290-344,
mis/mis.cpp:314-364, color/color.cpp:294-334, bc/bc.cpp:322-420).  Under
GDB_BARRIER_RELAUNCH (host loop with a stop read-back) and
GDB_BARRIER_RELAUNCH_GRAPH (a CUDA-graph WHILE node) Jacobi SSSP, MIS,
colouring and BC run the persistent kernels' superstep code once per
launch; their results must equal the oracle's and the persistent run's --
bit for bit for the integer apps, BC within the 1e-4 relative tolerance.
"""
import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

pytestmark = pytest.mark.gpu

RTOL = 1e-4
KINDS = [gdb.BARRIER_RELAUNCH, gdb.BARRIER_RELAUNCH_GRAPH]
KIND_IDS = ["relaunch", "relaunch_graph"]


def _graphs():
    V = 3000
    pairs = [(0, i) for i in range(1, 2001)] + [(2001, 2002), (2002, 2003)]
    return [
        ("grid16", gg.grid(16, 16)),
        ("rmat12", gg.rmat(1 << 12, 16, seed=5)),
        ("rmat14_hubs", gg.rmat(1 << 14, 32, seed=6)),
        ("star_isolated", gg.from_edges(V, pairs)),
        ("path", gg.from_edges(300, [(i, i + 1) for i in range(299)])),
        ("single", gg.from_edges(1, [])),
        ("pair", gg.from_edges(2, [(0, 1)])),
    ]


GRAPHS = _graphs()
IDS = [n for n, _ in GRAPHS]


def _bc_close(got, want):
    scale = np.maximum(np.abs(want), 1e-6 * max(1.0, float(np.max(np.abs(want))) if want.size else 1.0))
    return np.all(np.abs(got.astype(np.float64) - want) <= RTOL * scale + 1e-6)


@pytest.mark.parametrize("kind", KINDS, ids=KIND_IDS)
@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_jacobi_relaunch(kind, name, g):
    w = gg.uniform_weights(g, 1, 100, seed=2)
    want = oracle.sssp_jacobi(g.with_weights(w), 0, literal=True)
    with gdb.Ctx(barrier=kind) as c:
        G = c.graph(g.row_ptr, g.col, w)
        got = c.sssp_jacobi(G, 0)
        st = c.last_stats()
    assert np.array_equal(got, want), name
    if g.V >= 2 and kind == gdb.BARRIER_RELAUNCH:
        assert st["launches"] == st["supersteps"] + 1  # init + one per iteration


@pytest.mark.parametrize("kind", KINDS, ids=KIND_IDS)
@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_mis_relaunch(kind, name, g):
    prio = gg.priorities(g.V, seed=4)
    want, _ = oracle.mis(g, prio)
    with gdb.Ctx(barrier=kind) as c:
        G = c.graph(g.row_ptr, g.col)
        got = c.mis(G, prio)
    assert np.array_equal(got, want), name


@pytest.mark.parametrize("kind", KINDS, ids=KIND_IDS)
@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_color_relaunch(kind, name, g):
    prio = gg.priorities(g.V, seed=5)
    want, _ = oracle.color(g, prio)
    with gdb.Ctx() as c:
        c.color(c.graph(g.row_ptr, g.col), prio)
        rounds = c.last_stats()["supersteps"]
    with gdb.Ctx(barrier=kind) as c:
        G = c.graph(g.row_ptr, g.col)
        got = c.color(G, prio)
        st = c.last_stats()
    assert np.array_equal(got, want), name
    assert st["supersteps"] == rounds
    if kind == gdb.BARRIER_RELAUNCH:
        # init, count pass, colour 1, then one launch per round
        assert st["launches"] == rounds + 3


@pytest.mark.parametrize("kind", KINDS, ids=KIND_IDS)
@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_bc_relaunch(kind, name, g):
    srcs = gg.sources(g, 3, seed=8) if g.E else np.array([0], dtype=np.uint32)
    want32 = oracle.bc_f32(g, g, srcs).astype(np.float64)
    want64 = oracle.bc_f64(g, srcs)
    with gdb.Ctx(barrier=kind) as c:
        G = c.graph(g.row_ptr, g.col)
        got = c.bc(G, srcs)
    fin = np.isfinite(want32)
    assert _bc_close(got[fin], want64[fin]), name
    assert _bc_close(got[fin], want32[fin]), name
    assert not np.any(np.isfinite(got[~fin])), name


@pytest.mark.parametrize("kind", KINDS, ids=KIND_IDS)
def test_relaunch_equals_persistent_on_rmat16(kind):
    """The same supersteps as the persistent kernels: identical integer
    results, the same superstep counts, BC within the tolerance."""
    g = gg.rmat(1 << 16, 16, seed=23)
    w = gg.uniform_weights(g, 1, 100, seed=3)
    prio = gg.priorities(g.V, seed=6)
    srcs = [int(s) for s in gg.sources(g, 4, seed=2)]
    out = {}
    for k in (gdb.BARRIER_XF, kind):
        with gdb.Ctx(barrier=k) as c:
            G = c.graph(g.row_ptr, g.col, w)
            r = {}
            r["jacobi"] = c.sssp_jacobi(G, srcs[0])
            r["jacobi_steps"] = c.last_stats()["supersteps"]
            r["mis"] = c.mis(G, prio)
            r["mis_steps"] = c.last_stats()["supersteps"]
            r["color"] = c.color(G, prio)
            r["color_steps"] = c.last_stats()["supersteps"]
            r["bc"] = c.bc(G, srcs)
            r["bc_steps"] = c.last_stats()["supersteps"]
            out[k] = r
    a, b = out[gdb.BARRIER_XF], out[kind]
    for key in ("jacobi", "mis", "color"):
        assert np.array_equal(a[key], b[key]), key
    for key in ("jacobi_steps", "mis_steps", "color_steps"):
        assert a[key] == b[key], (key, a[key], b[key])
    fin = np.isfinite(a["bc"])
    assert _bc_close(b["bc"][fin], a["bc"][fin].astype(np.float64))
