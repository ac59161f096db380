"""The CPU oracle against the golden fixtures made by the reference's own
kernels (tests/golden/make_golden.py).  Integer outputs bit-exact; the
float32 BC restatement follows the reference's sequential order, so it is
compared bit-exact too, and the FP64 oracle within 1e-4 relative."""
import numpy as np
import pytest

import oracle as O
from golden_io import load, names

NAMES = names()


@pytest.mark.parametrize("name", NAMES)
def test_bfs_sssp(name):
    g, w, _, _, fx, meta = load(name)
    gw = g.with_weights(w)
    for i, s in enumerate(fx["sources"]):
        assert np.array_equal(O.bfs(g, int(s)), fx[f"bfs_{i}"]), (name, s)
        assert np.array_equal(O.par_bfs(g, int(s)), fx[f"bfs_{i}"]), (name, s)
        assert np.array_equal(O.sssp_worklist(gw, int(s)), fx[f"sssp_{i}"]), (name, s)
        # dverifysolution: no arc can still relax the answer
        assert O.verify_dist(g, fx[f"bfs_{i}"], weighted=False) == 0
        assert O.verify_dist(gw, fx[f"sssp_{i}"], weighted=True) == 0


@pytest.mark.parametrize("name", [n for n in NAMES if not n.endswith("_C1")])
def test_jacobi_mis_color(name):
    g, w, _, prio, fx, _ = load(name)
    gw = g.with_weights(w)
    assert np.array_equal(O.sssp_jacobi(gw, 0, literal=True), fx["jacobi_0"])
    # the Dijkstra form has the same fixed point unless the V-1 iteration cap
    # binds (a shortest path with V-1 or more arcs, e.g. a path from one end)
    lv = O.bfs(g, 0)
    if lv[lv != O.LONESTAR_INF].max() < g.V - 2:
        assert np.array_equal(O.sssp_jacobi(gw, 0), fx["jacobi_0"])
    assert np.array_equal(O.mis(g, prio)[0], fx["mis"])
    assert np.array_equal(O.color(g, prio)[0], fx["color"])


@pytest.mark.parametrize("name", [n for n in NAMES if not n.endswith("_C1")])
def test_bc(name):
    g, _, _, _, fx, _ = load(name)
    got = O.bc_f32(g, g, fx["bc_sources"])
    assert np.array_equal(got, fx["bc"]), name
    f64 = O.bc_f64(g, fx["bc_sources"])
    assert np.allclose(f64, fx["bc"], rtol=1e-4, atol=1e-6)
    if "bc_all" in fx:
        allsrc = np.arange(g.V, dtype=np.uint32)
        assert np.array_equal(O.bc_f32(g, g, allsrc), fx["bc_all"])


@pytest.mark.parametrize("name", [n for n in NAMES if not n.endswith("_C1")])
def test_mst(name):
    g, _, uw, _, fx, _ = load(name)
    m = O.mst(g.with_weights(uw))
    assert [m["weight32"], m["components"], m["edges"]] == fx["mst"].tolist()
