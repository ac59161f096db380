"""Delaunay mesh refinement (LonestarGPU DMR): the CPU restatement.

The restatement (oracle/oracle_dmr.c) is pinned against the reference's own
kernels (dmr_port_kernel.cl, run through oracle/refshim) on meshes where the
reference's refinement terminates, and shown to stop with a capacity error
where the reference's runs past its arrays.  The GPU kernel
(gdb_dmr_refine) is held to this restatement bit for bit in
tests/test_gpu_dmr.py.
"""
import numpy as np
import pytest

import oracle as O
from gpu_discovery_barrier_gb300 import meshgen

# isotropic jittered grids the reference refines to completion (2 to 54
# refinements)
PIN_MESHES = [(20, 20, 0.2), (30, 30, 0.2), (40, 25, 0.15)]


def _mesh(nx, ny, jitter, hy=1.0):
    return meshgen.grid_mesh(nx, ny, hy=hy, jitter=jitter, seed=1)


def test_grid_mesh_layout():
    m = _mesh(5, 4, 0.2)
    assert m.ntriangles == 2 * 4 * 3 and m.nsegments == 2 * (4 + 3)
    tri = m.elements[: m.ntriangles].astype(np.int64)
    a, b, c = tri.T
    area = ((m.x[b] - m.x[a]) * (m.y[c] - m.y[a]) - (m.y[b] - m.y[a]) * (m.x[c] - m.x[a])) / 2
    assert (area > 0).all()  # counter-clockwise
    assert np.isclose(area.sum(), 4.0 * 3.0)
    assert (m.elements[m.ntriangles:, 2] == meshgen.SEGMENT).all()
    nb = O.dmr_neighbours(m.elements)
    # every triangle has three neighbours (segments on the border)
    assert (nb[: m.ntriangles] != meshgen.SEGMENT).all()


@pytest.mark.skipif(not O.ref_available(), reason="reference kernels not built here")
@pytest.mark.parametrize("nx,ny,jitter", PIN_MESHES)
def test_dmr_restatement_matches_the_reference(nx, ny, jitter):
    m = _mesh(nx, ny, jitter)
    ours = O.dmr_refine(m, chunk=1)
    ref = O.ref_dmr(m)
    for k in ("x", "y", "elements", "neighbours", "isdel"):
        assert np.array_equal(ours[k], ref[k]), k
    assert ours["rounds"] == ref["rounds"]


def _live_triangles(r):
    el = r["elements"]
    live = (r["isdel"] == 0) & (el[:, 2] != meshgen.SEGMENT)
    return el[live].astype(np.int64), live


@pytest.mark.parametrize("chunk", [1, 7, 64])
def test_dmr_chunked_schedule_refines_completely(chunk):
    m = _mesh(30, 30, 0.2)
    r = O.dmr_refine(m, chunk=chunk)
    assert r["refined"] > 0
    assert O.dmr_count_bad(r["x"], r["y"], r["elements"], r["isdel"]) == 0
    tri, live = _live_triangles(r)
    x, y = r["x"], r["y"]
    a, b, c = tri.T
    area = ((x[b] - x[a]) * (y[c] - y[a]) - (y[b] - y[a]) * (x[c] - x[a])) / 2
    assert (area > 0).all()
    assert np.isclose(area.sum(), 29.0 * 29.0)  # the rectangle is tiled
    # neighbour links among live elements are mutual
    nb = r["neighbours"]
    ids = np.flatnonzero(live | ((r["isdel"] == 0) & (r["elements"][:, 2] == meshgen.SEGMENT)))
    for t in ids[:2000]:
        for n in nb[t]:
            if n != meshgen.SEGMENT:
                assert t in nb[n]


def test_dmr_runaway_is_reported_not_overrun():
    # anisotropic cells: the reference's segment test keeps splitting a
    # border segment (and writes past its arrays); the restatement stops at
    # the capacity (maxfactor) with an error
    m = _mesh(6, 6, 0.03, hy=0.3)
    with pytest.raises(RuntimeError, match="-3"):
        O.dmr_refine(m, chunk=1, maxfactor=40)
