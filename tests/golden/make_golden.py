"""Generate the golden fixtures from the reference's own kernels.

Runs the reference's OpenCL C kernels, compiled as C++ through
oracle/refshim (oracle/_ref/libgdbref.so, built from the reference checkout
by ``python -m gpu_discovery_barrier_gb300.build ref``), on small seeded
graphs and writes one compressed .npz per graph into this folder.  The
fixtures carry their inputs (or, for the 256x256 grid, the generator
parameters plus a SHA-256 of the arrays) so tests on any machine can check
the oracle and the GPU path against them without the reference.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from gpu_discovery_barrier_gb300 import graphgen as gg  # noqa: E402


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def ref_bfs(R, g, s):
    d = np.empty(g.V, np.uint32)
    assert R.ref_bfs_lonestar(g.V, g.row_ptr, O._nz(g.col), s, d) == 0
    return d


def ref_sssp(R, g, w, s):
    d = np.empty(g.V, np.uint32)
    assert R.ref_sssp_lonestar(g.V, g.row_ptr, O._nz(g.col), O._nz(w), s, d) == 0
    return d


def ref_jacobi(R, g, w, s):
    d = np.empty(g.V, np.int32)
    assert R.ref_sssp_pannotia(g.V, g.row_ptr, O._nz(g.col), O._nz(w), s, d) == 0
    return d


def ref_mis(R, g, p):
    d = np.empty(g.V, np.int32)
    assert R.ref_mis_pannotia(g.V, g.row_ptr, O._nz(g.col), p, d) == 0
    return d


def ref_color(R, g, p):
    d = np.empty(g.V, np.int32)
    assert R.ref_color_pannotia(g.V, g.row_ptr, O._nz(g.col), p, d) == 0
    return d


def ref_bc_sources(R, g, srcs):
    d = np.empty(g.V, np.float32)
    s = np.ascontiguousarray(srcs, np.uint32)
    assert R.ref_bc_pannotia_sources(g.V, g.row_ptr, O._nz(g.col), g.row_ptr, O._nz(g.col),
                                     O._nz(s), len(s), d) == 0
    return d


def ref_bc_all(R, g):
    d = np.empty(g.V, np.float32)
    assert R.ref_bc_pannotia_gb(g.V, g.row_ptr, O._nz(g.col), g.row_ptr, O._nz(g.col), d) == 0
    return d


def ref_mst(R, g, w):
    a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
    assert R.ref_mst_lonestar(g.V, g.row_ptr, O._nz(g.col), O._nz(w), C.byref(a), C.byref(b),
                              C.byref(c)) == 0
    return np.array([a.value, b.value, c.value], dtype=np.uint32)


def cases():
    star_pairs = [(0, i) for i in range(1, 1501)] + [(1501, 1502), (1503, 1504)]
    return [
        ("grid16x16", gg.grid(16, 16), True),
        ("rmat1024_ef16", gg.rmat(1024, 16, seed=3), True),
        ("rmat300_ef5", gg.rmat(300, 5, seed=7), True),
        ("grid4x300", gg.grid(4, 300), True),
        ("star1500_isolated", gg.from_edges(1600, star_pairs), True),
        ("path200", gg.from_edges(200, [(i, i + 1) for i in range(199)]), True),
        ("two_triangles_isolated", gg.from_edges(9, [(0, 1), (1, 2), (2, 0), (4, 5), (5, 6), (6, 4)]),
         True),
        ("grid256x256_C1", gg.grid(256, 256), False),
    ]


def make(R, name, g, store_inputs):
    w = gg.uniform_weights(g, 1, 100, seed=1)
    uw = gg.unique_weights(g, seed=9)
    prio = gg.priorities(g.V, seed=4)
    srcs = sorted(set([0] + [int(x) for x in gg.sources(g, 3, seed=7)]))
    out = {"sources": np.array(srcs, np.uint32)}
    for i, s in enumerate(srcs):
        out[f"bfs_{i}"] = ref_bfs(R, g, s)
        out[f"sssp_{i}"] = ref_sssp(R, g, w, s)
    meta = {"name": name, "V": g.V, "E": g.E, "sources": srcs,
            "weights": "uniform_weights(1, 100, seed=1)", "mst_weights": "unique_weights(seed=9)",
            "priorities": "priorities(seed=4)", "input_sha256": sha(g.row_ptr, g.col, w, uw, prio)}
    if name.endswith("_C1"):
        meta["generator"] = {"kind": "grid", "rows": 256, "cols": 256}
        # the 256x256 grid of the parity config: BFS and SSSP from vertex 0
        out = {"sources": np.array([0], np.uint32), "bfs_0": ref_bfs(R, g, 0),
               "sssp_0": ref_sssp(R, g, w, 0)}
    else:
        out["jacobi_0"] = ref_jacobi(R, g, w, 0)
        out["mis"] = ref_mis(R, g, prio)
        out["color"] = ref_color(R, g, prio)
        bsrc = np.array(srcs, np.uint32)
        out["bc_sources"] = bsrc
        out["bc"] = ref_bc_sources(R, g, bsrc)
        if g.V <= 2048:
            out["bc_all"] = ref_bc_all(R, g)
        out["mst"] = ref_mst(R, g, uw)
    if store_inputs:
        out.update(row_ptr=g.row_ptr, col=g.col, w=w, uw=uw, prio=prio)
    np.savez_compressed(HERE / f"{name}.npz", meta=np.array(json.dumps(meta)), **out)
    print(name, g.V, g.E, "ok")


def main():
    if not O.ref_available():
        from gpu_discovery_barrier_gb300 import build
        if build.build_reference() is None:
            sys.exit("reference checkout not found: cannot build oracle/_ref")
    R = O.ref()
    for name, g, store in cases():
        make(R, name, g, store)


if __name__ == "__main__":
    main()
