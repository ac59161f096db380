"""Graph file readers (CPU only): .gr v1, DIMACS and METIS.

Checked against hand-written files whose CSR is known, round trips through
the .gr writer, error reporting, and -- where the reference checkout is
built (oracle/_ref) -- the reference's own Pannotia readers (parseCOO,
parseMetis) on the same files.
"""
import ctypes as C
import struct

import numpy as np
import pytest

import oracle
from gpu_discovery_barrier_gb300 import gdb, graphgen as gg


def _gr_bytes(row_end, dst, w=None):
    """A .gr v1 file laid out by hand from the format's description."""
    V, E = len(row_end), len(dst)
    b = struct.pack("<4Q", 1, 4 if w is not None else 0, V, E)
    b += struct.pack(f"<{V}Q", *row_end) + struct.pack(f"<{E}I", *dst)
    if E % 2:
        b += b"\0" * 4
    if w is not None:
        b += struct.pack(f"<{E}I", *w)
    return b


def test_gr_hand_built(tmp_path):
    p = tmp_path / "g.gr"
    # 4 vertices, 5 arcs (odd: padded), vertex 2 without arcs
    p.write_bytes(_gr_bytes([2, 4, 4, 5], [1, 3, 0, 3, 0], [7, 8, 9, 10, 11]))
    g = gdb.read_graph(p)
    assert g.row_ptr.tolist() == [0, 2, 4, 4, 5]
    assert g.col.tolist() == [1, 3, 0, 3, 0]
    assert g.w.tolist() == [7, 8, 9, 10, 11]
    p.write_bytes(_gr_bytes([1, 2], [1, 0]))
    g = gdb.read_graph(p)
    assert g.w is None and g.col.tolist() == [1, 0]


@pytest.mark.parametrize("weighted", [False, True])
def test_gr_round_trip(tmp_path, weighted):
    g = gg.rmat(3000, 7, seed=4)
    if weighted:
        g = g.with_weights(gg.uniform_weights(g, 1, 255, seed=2))
    if g.E % 2 == 0:  # exercise the pad
        g = gg.from_edges(5, [(0, 1), (1, 2), (2, 3)], weights=[3, 4, 5] if weighted else None,
                          symmetric=False)
    p = tmp_path / "r.gr"
    gdb.write_gr(p, g)
    h = gdb.read_graph(p)
    assert np.array_equal(h.row_ptr, g.row_ptr) and np.array_equal(h.col, g.col)
    assert (h.w is None) == (not weighted)
    if weighted:
        assert np.array_equal(h.w, g.w)


DIMACS = """c a small road-like graph
p sp 5 6
a 1 2 10
a 2 3 20
c comment between arcs
a 1 3 5
a 3 4 7
a 4 5 1
a 5 1 2
"""


def test_dimacs_directed_and_undirected(tmp_path):
    p = tmp_path / "g.dimacs"
    p.write_text(DIMACS)
    d = gdb.read_graph(p, directed=True)
    assert d.row_ptr.tolist() == [0, 2, 3, 4, 5, 6]
    assert d.col.tolist() == [1, 2, 2, 3, 4, 0]
    assert d.w.tolist() == [10, 5, 20, 7, 1, 2]
    u = gdb.read_graph(p, directed=False)
    # every arc and its reverse, grouped by source in file order
    assert u.row_ptr.tolist() == [0, 3, 5, 8, 10, 12]
    assert u.col.tolist() == [1, 2, 4, 0, 2, 1, 0, 3, 2, 4, 3, 0]
    assert u.w.tolist() == [10, 5, 2, 10, 20, 20, 5, 7, 7, 1, 1, 2]


METIS = """% a 6-vertex graph, vertex 6 isolated
6 5
2 3
1 3
1 2 4
3 5
4

"""

METIS_W = """6 5 001
2 4 3 9
1 4 3 1
1 9 2 1 4 6
3 6 5 2
4 2

"""


def test_metis(tmp_path):
    p = tmp_path / "g.graph"
    p.write_text(METIS)
    g = gdb.read_graph(p)
    assert g.row_ptr.tolist() == [0, 2, 4, 7, 9, 10, 10]
    assert g.col.tolist() == [1, 2, 0, 2, 0, 1, 3, 2, 4, 3]
    assert g.w is None
    p.write_text(METIS_W)
    h = gdb.read_graph(p)
    assert np.array_equal(h.row_ptr, g.row_ptr) and np.array_equal(h.col, g.col)
    assert h.w.tolist() == [4, 9, 4, 1, 9, 1, 6, 6, 2, 2]


@pytest.mark.parametrize("text,fmt,needle", [
    ("p sp 3 1\na 1 4 2\n", gdb.FMT_DIMACS, "out of range"),
    ("a 1 2 3\n", gdb.FMT_DIMACS, "before the problem line"),
    ("2 1\n2\n", gdb.FMT_METIS, "fewer lines"),
    ("2 1\n3\n1\n", gdb.FMT_METIS, "out of range"),
    ("2 1 011\n2 1\n1 1\n", gdb.FMT_METIS, "vertex weights"),
])
def test_errors_are_reported(tmp_path, text, fmt, needle):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(gdb.GdbError) as e:
        gdb.read_graph(p, fmt=fmt)
    assert e.value.status == -1 and needle in str(e.value)


def test_gr_errors(tmp_path):
    p = tmp_path / "bad.gr"
    p.write_bytes(_gr_bytes([1, 2], [1, 5]))
    with pytest.raises(gdb.GdbError) as e:
        gdb.read_graph(p)
    assert "out of range" in str(e.value)
    p.write_bytes(struct.pack("<4Q", 2, 0, 1, 0) + struct.pack("<Q", 0))
    with pytest.raises(gdb.GdbError):
        gdb.read_graph(p)


def _ref_parse(path, metis, directed):
    L = oracle.ref()
    ip = C.POINTER(C.c_int)
    L.ref_parse.argtypes = [C.c_char_p, C.c_int, C.c_int, ip, ip, ip, C.POINTER(ip), C.POINTER(ip),
                            C.POINTER(ip)]
    n, e, r = C.c_int(), C.c_int(), C.c_int()
    ra, ca, da = ip(), ip(), ip()
    assert L.ref_parse(str(path).encode(), metis, directed, C.byref(n), C.byref(e), C.byref(r),
                       C.byref(ra), C.byref(ca), C.byref(da)) == 0
    out = (n.value, [ra[i] for i in range(r.value + 1)], [ca[i] for i in range(e.value)],
           [da[i] for i in range(e.value)])
    L.ref_parse_free(ra, ca, da)
    return out


@pytest.mark.skipif(not oracle.ref_available(), reason="reference readers not built here")
@pytest.mark.parametrize("directed", [0, 1])
def test_dimacs_matches_the_reference_reader(tmp_path, directed):
    g = gg.rmat(500, 6, seed=9)
    w = gg.uniform_weights(g, 1, 99, seed=1)
    src = np.repeat(np.arange(g.V), np.diff(g.row_ptr.astype(np.int64)))
    keep = src < g.col  # one line per undirected edge, in a shuffled order
    order = np.random.default_rng(3).permutation(int(keep.sum()))
    us, vs, ws = src[keep][order], g.col[keep][order], w[keep][order]
    # every vertex has an arc (the reference drops rows without arcs)
    lines = [f"p sp {g.V} {len(us) + g.V}"] + [f"a {u + 1} {v + 1} {x}" for u, v, x in zip(us, vs, ws)]
    lines += [f"a {v + 1} {(v + 1) % g.V + 1} 1" for v in range(g.V)]
    p = tmp_path / "r.dimacs"
    p.write_text("\n".join(lines) + "\n")
    V, rows, col, data = _ref_parse(p, 0, directed)
    ours = gdb.read_graph(p, directed=bool(directed))
    assert V == ours.V and len(rows) == ours.V + 1
    assert rows == ours.row_ptr.tolist() and col == ours.col.tolist() and data == ours.w.tolist()


@pytest.mark.skipif(not oracle.ref_available(), reason="reference readers not built here")
def test_metis_matches_the_reference_reader(tmp_path):
    g = gg.rmat(400, 5, seed=12)
    deg = np.diff(g.row_ptr.astype(np.int64))
    keep = np.nonzero(deg > 0)[0]  # the reference drops rows without arcs
    sub = {int(v): i for i, v in enumerate(keep)}
    lines = [f"{len(keep)} {int(deg[keep].sum()) // 2}"]
    for v in keep:
        nb = g.col[g.row_ptr[v]:g.row_ptr[v + 1]]
        lines.append(" ".join(str(sub[int(u)] + 1) for u in nb))
    p = tmp_path / "r.graph"
    p.write_text("\n".join(lines) + "\n")
    V, rows, col, _ = _ref_parse(p, 1, 0)
    ours = gdb.read_graph(p)
    assert V == ours.V
    assert rows == ours.row_ptr.tolist() and col == ours.col.tolist()
