"""Frontier bitmaps of the direction-optimising BFS.

Each level's frontier is kept as a V-bit bitmap beside its queue; a
bottom-up (pull) level tests a neighbour's bit instead of loading its level,
with the bitmap's lowest ids staged in every CTA's shared memory.  The
levels must equal the oracle's (lonestar/apps/bfs/kernel/bfs_port_kernel.cl:146-192
semantics) for every stage size:
  * -1: no bitmap (pull levels test the level array);
  * 1 KB: a stage smaller than the bitmap, so probes past it read the
    bitmap from L2;
  * 0: automatic (16 KB for a traversal alone on the GPU, none for
    traversals sharing it on lanes);
  * 64 KB: the largest, clipped to the bitmap on small graphs;
under the threshold schedule, the learned one, every level forced pull
(level 0's bitmap built from the level array, every later one written by
the pull level before it), push and pull alternating level by level (every
pull level builds its bitmap from the level array), and many sources at
once (one multi-source run, and independent runs on lanes).
"""
import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg, selector

pytestmark = pytest.mark.gpu

STAGES = [-1, 1, 0, 64]
STAGE_IDS = ["none", "1kb", "default", "64kb"]


def _graphs():
    V = 3000
    star = [(0, i) for i in range(1, 2001)] + [(2001, 2002), (2002, 2003)]
    # two components joined by nothing, ids interleaved
    two = [(2 * i, 2 * i + 2) for i in range(400)] + [(2 * i + 1, 2 * i + 3) for i in range(400)]
    return [
        ("rmat14", gg.rmat(1 << 14, 16, seed=5)),
        ("rmat16", gg.rmat(1 << 16, 16, seed=23)),
        ("star_isolated", gg.from_edges(V, star)),
        ("two_components", gg.from_edges(803, two)),
        ("path", gg.from_edges(300, [(i, i + 1) for i in range(299)])),
        ("grid32", gg.grid(32, 32)),
        ("v1000", gg.rmat(1000, 6, seed=3)),
        ("tiny", gg.from_edges(5, [(0, 1), (1, 2), (3, 4)])),
        ("single", gg.from_edges(1, [])),
    ]


GRAPHS = _graphs()
IDS = [n for n, _ in GRAPHS]


def _src(g):
    return int(gg.sources(g, 1, seed=3)[0]) if g.E else 0


@pytest.mark.parametrize("kb", STAGES, ids=STAGE_IDS)
@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_forced_pull_levels(kb, name, g):
    """Every level bottom-up: the bitmap carries the whole traversal."""
    s = _src(g)
    want = oracle.bfs(g, s)
    with gdb.Ctx(pull_bitmap_kb=kb) as c:
        G = c.graph(g.row_ptr, g.col)
        got, _, modes, _ = c.bfs_trace(G, s, mode=1)
    assert np.array_equal(got, want), name
    assert np.all(modes == 1)


@pytest.mark.parametrize("kb", STAGES, ids=STAGE_IDS)
@pytest.mark.parametrize("name,g", GRAPHS, ids=IDS)
def test_threshold_schedule(kb, name, g):
    s = _src(g)
    want = oracle.bfs(g, s)
    with gdb.Ctx(schedule=gdb.SCHED_ADAPTIVE, pull_bitmap_kb=kb) as c:
        G = c.graph(g.row_ptr, g.col)
        got = c.bfs(G, s)
    assert np.array_equal(got, want), name


@pytest.mark.parametrize("kb", STAGES, ids=STAGE_IDS)
@pytest.mark.parametrize("name,g", GRAPHS[:5], ids=IDS[:5])
def test_alternating_push_and_pull(kb, name, g):
    """pull_alpha 10^6 switches a push level to pull as soon as its frontier
    has an arc, push_beta 1 switches back at once: the levels alternate."""
    s = _src(g)
    with gdb.Ctx(schedule=gdb.SCHED_ADAPTIVE, pull_alpha=10**6, push_beta=1, pull_bitmap_kb=kb) as c:
        G = c.graph(g.row_ptr, g.col)
        got = c.bfs(G, s)
    assert np.array_equal(got, oracle.bfs(g, s)), name


@pytest.mark.parametrize("kb", STAGES, ids=STAGE_IDS)
def test_learned_schedule_and_lanes(kb):
    """The shipped network's push/pull choices over bitmap levels, one
    source per call and 16 sources on concurrent lanes."""
    p = selector.load()
    if p is None:
        pytest.skip("no shipped selector weights")
    g = gg.rmat(1 << 17, 16, seed=11)
    srcs = [int(x) for x in gg.sources(g, 16, seed=5)]
    want = np.stack([oracle.bfs(g, s) for s in srcs])
    with gdb.Ctx(schedule=gdb.SCHED_LEARNED, pull_bitmap_kb=kb) as c:
        c.selector_set(p)
        G = c.graph(g.row_ptr, g.col)
        assert np.array_equal(c.bfs(G, srcs[0]), want[0])
        assert np.array_equal(c.bfs_sources(G, srcs), want)


@pytest.mark.parametrize("kb", STAGES, ids=STAGE_IDS)
def test_multi_source_seed_bits(kb):
    """One run from many sources (repeated ones included): level 0's bitmap
    holds every source."""
    g = gg.rmat(1 << 13, 12, seed=21)
    srcs = [int(s) for s in gg.sources(g, 5, seed=4)] + [7, 7]
    want = np.minimum.reduce([oracle.bfs(g, s) for s in srcs])
    with gdb.Ctx(schedule=gdb.SCHED_ADAPTIVE, pull_bitmap_kb=kb) as c:
        G = c.graph(g.row_ptr, g.col)
        assert np.array_equal(c.bfs_multi(G, srcs), want)


def test_grid_sync_barrier_with_bitmap():
    g = gg.rmat(1 << 15, 16, seed=9)
    s = _src(g)
    with gdb.Ctx(barrier=gdb.BARRIER_GRID_SYNC, pull_bitmap_kb=16) as c:
        G = c.graph(g.row_ptr, g.col)
        got, _, _, _ = c.bfs_trace(G, s, mode=1)
    assert np.array_equal(got, oracle.bfs(g, s))
