"""Oracle restatement against the reference's kernels run live through the
shim, on random graphs (only where oracle/_ref was built, i.e. where the
reference checkout exists)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from gpu_discovery_barrier_gb300 import graphgen as gg

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="oracle/_ref not built here")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_rmat(seed):
    R = O.ref()
    g = gg.rmat(700 + 97 * seed, 6 + seed, seed=seed)
    w = gg.uniform_weights(g, 1, 50, seed=seed)
    s = int(gg.sources(g, 1, seed=seed)[0])
    d = np.empty(g.V, np.uint32)
    R.ref_bfs_lonestar(g.V, g.row_ptr, O._nz(g.col), s, d)
    assert np.array_equal(d, O.bfs(g, s))
    R.ref_sssp_lonestar(g.V, g.row_ptr, O._nz(g.col), O._nz(w), s, d)
    assert np.array_equal(d, O.sssp_worklist(g.with_weights(w), s))
    p = gg.priorities(g.V, seed=seed)
    m = np.empty(g.V, np.int32)
    R.ref_mis_pannotia(g.V, g.row_ptr, O._nz(g.col), p, m)
    assert np.array_equal(m, O.mis(g, p)[0])
    R.ref_color_pannotia(g.V, g.row_ptr, O._nz(g.col), p, m)
    assert np.array_equal(m, O.color(g, p)[0])
    uw = gg.unique_weights(g, seed=seed)
    a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
    R.ref_mst_lonestar(g.V, g.row_ptr, O._nz(g.col), O._nz(uw), C.byref(a), C.byref(b), C.byref(c))
    o = O.mst(g.with_weights(uw))
    assert (a.value, b.value, c.value) == (o["weight32"], o["components"], o["edges"])


@pytest.mark.parametrize("groups", [1, 4, 16])
def test_reference_discovery_on_threads(groups):
    """The reference's discovery protocol + XF barrier on host threads:
    participants get the ids 0..P-1, the barrier holds, and the last group
    re-arms the context (discovery.cl:32-36)."""
    R = O.ref()
    ids = np.empty(groups, np.int32)
    n, ok, err = C.c_int(), C.c_int(), C.c_int()
    R.ref_discovery_threads(groups, 5, ids, C.byref(n), C.byref(ok), C.byref(err))
    got = sorted(int(i) for i in ids if i >= 0)
    assert got == list(range(n.value)) and n.value >= 1
    assert ok.value == 1 and err.value == 0
