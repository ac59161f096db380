"""Properties of the synthetic graph generators (CPU)."""
import numpy as np
import pytest

from gpu_discovery_barrier_gb300 import graphgen as gg


def check_csr(g):
    rp, col = g.row_ptr.astype(np.int64), g.col
    assert rp[0] == 0 and rp[-1] == g.E
    assert np.all(np.diff(rp) >= 0)
    src = np.repeat(np.arange(g.V), np.diff(rp))
    assert np.all(col < g.V)
    assert not np.any(src == col), "self loop"
    # rows strictly ascending: sorted and no duplicate arcs
    same_row = src[1:] == src[:-1]
    assert np.all(col[1:][same_row] > col[:-1][same_row])
    # symmetric
    fwd = set(zip(src.tolist(), col.tolist())) if g.E < 300000 else None
    if fwd is not None:
        assert all((b, a) in fwd for (a, b) in fwd)


@pytest.mark.parametrize("r,c", [(1, 1), (1, 7), (5, 1), (16, 16), (256, 256), (3, 1000)])
def test_grid(r, c):
    g = gg.grid(r, c)
    assert g.V == r * c
    assert g.E == 2 * (r * (c - 1) + c * (r - 1))
    check_csr(g)


def test_grid_c1_arc_count():
    # the 256x256 parity grid has 261,120 arcs (not 260,096)
    assert gg.grid(256, 256).E == 261120


def test_rmat_deterministic_and_valid():
    a = gg.rmat(1 << 12, 16, seed=5)
    b = gg.rmat(1 << 12, 16, seed=5)
    c = gg.rmat(1 << 12, 16, seed=6)
    assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)
    assert not np.array_equal(a.col[: min(a.E, c.E)], c.col[: min(a.E, c.E)])
    check_csr(a)
    # skewed degrees (R-MAT), isolated vertices allowed
    d = a.degrees()
    assert d.max() > 20 * d.mean()


def test_rmat_non_power_of_two():
    g = gg.rmat(1000, 8, seed=2)
    assert g.V == 1000
    check_csr(g)


def test_weights_symmetric_and_unique():
    g = gg.rmat(2048, 8, seed=3)
    w = gg.uniform_weights(g, 1, 255, seed=1)
    assert w.min() >= 1 and w.max() <= 255
    uw = gg.unique_weights(g, seed=9)
    src = np.repeat(np.arange(g.V), g.degrees())
    fw = {(int(a), int(b)): int(x) for a, b, x in zip(src, g.col, w)}
    fu = {(int(a), int(b)): int(x) for a, b, x in zip(src, g.col, uw)}
    assert all(fw[(a, b)] == fw[(b, a)] for (a, b) in fw)
    assert all(fu[(a, b)] == fu[(b, a)] for (a, b) in fu)
    und = sorted(v for (a, b), v in fu.items() if a < b)
    assert und == list(range(1, g.E // 2 + 1))


def test_priorities_and_sources():
    p = gg.priorities(1000, seed=4)
    assert sorted(p.astype(int).tolist()) == list(range(1000))
    g = gg.rmat(4096, 4, seed=1)
    s = gg.sources(g, 16, seed=2)
    assert len(set(s.tolist())) == 16
    assert np.all(g.degrees()[s] > 0)


def test_transpose_of_symmetric_is_identity():
    g = gg.rmat(512, 8, seed=8)
    t = gg.transpose(g)
    assert np.array_equal(t.row_ptr, g.row_ptr) and np.array_equal(t.col, g.col)
