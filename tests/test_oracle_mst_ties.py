"""The CPU oracle's MST under equal weights (no GPU).  The GPU tests with
tied weights compare the forest's weight and edge count with the oracle's,
so the oracle is pinned here against an independent minimum spanning
forest: every minimum forest has the same weight and edge count."""
import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import graphgen as gg

sp = pytest.importorskip("scipy.sparse")
csgraph = pytest.importorskip("scipy.sparse.csgraph")


def _scipy_forest(g, w):
    rows = np.repeat(np.arange(g.V), np.diff(g.row_ptr.astype(np.int64)))
    m = sp.csr_matrix((w.astype(np.float64), (rows, g.col.astype(np.int64))), shape=(g.V, g.V))
    t = csgraph.minimum_spanning_tree(m)
    return int(round(t.sum())), int(t.nnz)


@pytest.mark.parametrize("name,g", [
    ("rmat12", gg.rmat(1 << 12, 16, seed=5)),
    ("grid48", gg.grid(48, 48)),
    ("star", gg.from_edges(600, [(0, i) for i in range(1, 400)] + [(400, 401)])),
], ids=["rmat12", "grid48", "star"])
@pytest.mark.parametrize("kind", ["ones", "1to3"])
def test_oracle_mst_with_tied_weights(name, g, kind):
    if kind == "ones":
        w = np.ones(g.E, np.uint32)
    else:
        w = (gg.unique_weights(g, seed=13) % 3 + 1).astype(np.uint32)  # one per edge
    got = oracle.mst(g.with_weights(w))
    weight, edges = _scipy_forest(g, w)
    assert got["weight64"] == weight, name
    assert got["edges"] == edges and got["components"] == g.V - edges, name
