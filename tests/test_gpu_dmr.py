"""Delaunay mesh refinement on the GPU (gdb_dmr_refine) against the CPU
restatement of the reference's refinement (oracle/oracle_dmr.c), which the
reference's own kernels pin with a chunk of one item.

The GPU kernel runs the oracle's deterministic chunked schedule: for every
chunk size the refined mesh must be the same bits -- node coordinates
(doubles), elements, neighbour triples, deleted flags -- and the same
round, chunk and refinement counts.  Meshes: isotropic jittered grids,
which the reference refines to completion.
"""
import numpy as np
import pytest

import oracle as O
from gpu_discovery_barrier_gb300 import gdb, meshgen

pytestmark = pytest.mark.gpu

# (nx, ny, jitter, seed): 10, 54, 2, 127, 163 and 381-382 refinements;
# each refines to completion under every chunk size tested
MESHES = [(20, 20, 0.2, 1), (30, 30, 0.2, 1), (40, 25, 0.15, 1), (50, 50, 0.2, 2), (60, 60, 0.2, 2),
          (60, 40, 0.25, 1)]


@pytest.mark.parametrize("nx,ny,jitter,seed", MESHES)
@pytest.mark.parametrize("chunk", [1, 7, 64, 4096])
def test_dmr_gpu_equals_the_schedule_bit_for_bit(ctx, nx, ny, jitter, seed, chunk):
    m = meshgen.grid_mesh(nx, ny, hy=1.0, jitter=jitter, seed=seed)
    want = O.dmr_refine(m, chunk=chunk)
    got = ctx.dmr_refine(m, chunk=chunk)
    for k in ("rounds", "chunks", "refined"):
        assert got[k] == want[k], (k, got[k], want[k])
    for k in ("x", "y", "elements", "neighbours", "isdel"):
        assert got[k].shape == want[k].shape, k
        assert np.array_equal(got[k].view(np.uint8), want[k].view(np.uint8)), k


def test_dmr_gpu_leaves_no_bad_triangle(ctx):
    m = meshgen.grid_mesh(60, 40, hy=1.0, jitter=0.25, seed=1)
    r = ctx.dmr_refine(m, chunk=64)
    assert r["refined"] > 0
    assert O.dmr_count_bad(r["x"], r["y"], r["elements"], r["isdel"]) == 0


def test_dmr_gpu_reports_runaway_as_capacity(ctx):
    # anisotropic cells: refinement keeps splitting a border segment until
    # the node / element capacity runs out; the GPU stops with an error
    m = meshgen.grid_mesh(6, 6, hy=0.3, jitter=0.03, seed=1)
    with pytest.raises(gdb.GdbError) as e:
        ctx.dmr_refine(m, chunk=1, maxfactor=40)
    assert e.value.status == -5  # GDB_ERR_CAPACITY


def test_dmr_cavity_capacity_matches_the_restatement(ctx):
    # with 4,096 items a chunk, this mesh grows a cavity past its slot
    # (256 elements / 1,024 boundary words): both report it
    m = meshgen.grid_mesh(40, 40, hy=1.0, jitter=0.25, seed=1)
    with pytest.raises(RuntimeError, match="-5"):
        O.dmr_refine(m, chunk=4096)
    with pytest.raises(gdb.GdbError) as e:
        ctx.dmr_refine(m, chunk=4096)
    assert e.value.status == -5  # GDB_ERR_CAPACITY


def test_dmr_rejects_bad_input(ctx):
    m = meshgen.grid_mesh(5, 5, hy=1.0, jitter=0.1, seed=2)
    bad = meshgen.Mesh(m.x, m.y, m.elements.copy(), m.ntriangles, m.nsegments)
    bad.elements[0, 0] = m.nnodes + 5
    with pytest.raises(gdb.GdbError):
        ctx.dmr_refine(bad, chunk=8)
    with pytest.raises(gdb.GdbError):
        ctx.dmr_refine(m, chunk=0)


def test_dmr_obtuse_triangle_facing_no_neighbour_is_rejected(ctx):
    # here refinement reaches an obtuse triangle whose facing neighbour is
    # missing, where the reference reads past its element array; the
    # restatement and the GPU both stop with an error instead
    m = meshgen.grid_mesh(60, 60, hy=1.0, jitter=0.2, seed=3)
    with pytest.raises(RuntimeError, match="-6"):
        O.dmr_refine(m, chunk=64)
    with pytest.raises(gdb.GdbError) as e:
        ctx.dmr_refine(m, chunk=64)
    assert e.value.status == -1  # GDB_ERR_INVALID
