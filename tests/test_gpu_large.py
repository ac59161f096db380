"""Full-size checks: BFS levels on the 4096x4096 grid are the Manhattan
distance from the corner (8,190 supersteps); SSSP from that corner with
the grid workload's U[1,1000] weights passes the reference's own validity
check (dverifysolution: no arc can still relax it, sssp_common.cl:41-56)
and equals the oracle's distances under every schedule; the 1024x1024 grid
likewise."""
import functools

import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("barrier", [gdb.BARRIER_XF, gdb.BARRIER_GRID_SYNC])
def test_grid4096_bfs_levels(barrier):
    R = C = 4096
    g = gg.grid(R, C)
    with gdb.Ctx(barrier=barrier) as c:
        G = c.graph(g.row_ptr, g.col)
        d = c.bfs(G, 0)
        assert c.last_stats()["supersteps"] == R + C - 1
    r, col = np.divmod(np.arange(g.V, dtype=np.int64), C)
    assert np.array_equal(d.astype(np.int64), r + col)


@pytest.mark.parametrize("schedule", [gdb.SCHED_PLAIN, gdb.SCHED_ADAPTIVE])
def test_grid1024_sssp_valid_and_exact(schedule):
    g = gg.grid(1024, 1024)
    w = gg.uniform_weights(g, 1, 1000, seed=1)
    with gdb.Ctx(schedule=schedule) as c:
        G = c.graph(g.row_ptr, g.col, w)
        d = c.sssp(G, 0)
    gw = g.with_weights(w)
    assert oracle.verify_dist(gw, d, weighted=True) == 0
    assert np.array_equal(d, oracle.sssp_worklist(gw, 0))


@functools.lru_cache(maxsize=1)
def _grid4096_weighted():
    g = gg.grid(4096, 4096)
    w = gg.uniform_weights(g, 1, 1000, seed=1)
    gw = g.with_weights(w)
    return gw, oracle.sssp_worklist(gw, 0)


@pytest.mark.parametrize("schedule", [gdb.SCHED_PLAIN, gdb.SCHED_ADAPTIVE])
def test_grid4096_sssp_from_corner_exact(schedule):
    gw, want = _grid4096_weighted()
    with gdb.Ctx(schedule=schedule) as c:
        G = c.graph(gw.row_ptr, gw.col, gw.w, symmetric=True)
        d = c.sssp(G, 0)
        st = c.last_stats()
    assert st["supersteps"] > 1000
    assert oracle.verify_dist(gw, d, weighted=True) == 0
    assert np.array_equal(d, want)
