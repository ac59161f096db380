"""Deterministic synthetic graphs (symmetric uint32 CSR) for the workloads.

Thin ctypes layer over ``lib/libgdbgen.so`` (csrc/graphgen.cpp).  The
generators are counter-based, so a graph depends only on its parameters and
seed -- identical on x86_64 and aarch64 and for any thread count.

The reference reads external datasets (DIMACS road graphs, rmat22, 2-D
grids; pannotia/graph_parser/parse.cpp, lonestar_gpu_opencl/include/graph.h);
these seeded graphs of the same shapes stand in for them.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_LIB = None
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def _lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = Path(__file__).resolve().parent / "lib" / "libgdbgen.so"
        if not path.exists():
            from . import build
            build.build_graphgen()
        lib = C.CDLL(str(path))
        lib.gdbgen_grid_arcs.restype = C.c_uint64
        lib.gdbgen_grid_arcs.argtypes = [C.c_uint32, C.c_uint32]
        lib.gdbgen_grid.restype = C.c_int
        lib.gdbgen_grid.argtypes = [C.c_uint32, C.c_uint32, _u32p, _u32p]
        lib.gdbgen_rmat.restype = C.c_int
        lib.gdbgen_rmat.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_uint64, C.POINTER(C.POINTER(C.c_uint32)),
                                    C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_uint64)]
        lib.gdbgen_free.argtypes = [C.c_void_p]
        lib.gdbgen_uniform_weights.argtypes = [C.c_uint32, _u32p, _u32p, C.c_uint64,
                                               C.c_uint32, C.c_uint32, _u32p]
        lib.gdbgen_permutation.argtypes = [C.c_uint32, C.c_uint64, _u32p]
        lib.gdbgen_unique_weights.restype = C.c_uint64
        lib.gdbgen_unique_weights.argtypes = [C.c_uint32, _u32p, _u32p, C.c_uint64, _u32p]
        lib.gdbgen_sources.restype = C.c_uint32
        lib.gdbgen_sources.argtypes = [C.c_uint32, _u32p, C.c_uint64, C.c_uint32, _u32p]
        lib.gdbgen_transpose.argtypes = [C.c_uint32, _u32p, _u32p, C.c_void_p, _u32p, _u32p,
                                         C.c_void_p]
        lib.gdbgen_splitmix64.restype = C.c_uint64
        lib.gdbgen_splitmix64.argtypes = [C.c_uint64]
        _LIB = lib
    return _LIB


@dataclass
class CSR:
    """Symmetric CSR graph: row_ptr[V+1], col[E] (uint32), optional w[E]."""

    row_ptr: np.ndarray
    col: np.ndarray
    w: np.ndarray | None = None
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def V(self) -> int:
        return int(self.row_ptr.shape[0] - 1)

    @property
    def E(self) -> int:
        return int(self.col.shape[0])

    def degrees(self) -> np.ndarray:
        return np.diff(self.row_ptr.astype(np.int64))

    def with_weights(self, w: np.ndarray) -> "CSR":
        return CSR(self.row_ptr, self.col, np.ascontiguousarray(w, dtype=np.uint32), self.name,
                   dict(self.meta))


def grid(rows: int, cols: int) -> CSR:
    """rows x cols 4-neighbour grid, vertex (r, c) = r*cols + c."""
    lib = _lib()
    V = rows * cols
    E = int(lib.gdbgen_grid_arcs(rows, cols))
    rp = np.empty(V + 1, dtype=np.uint32)
    col = np.empty(max(E, 1), dtype=np.uint32)
    if lib.gdbgen_grid(rows, cols, rp, col) != 0:
        raise ValueError(f"grid {rows}x{cols} too large for uint32 CSR")
    return CSR(rp, col[:E], None, f"grid{rows}x{cols}", {"rows": rows, "cols": cols})


def rmat(V: int, edge_factor: float, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1) -> CSR:
    """Seeded R-MAT over V vertices, symmetrised, deduplicated, no self loops."""
    lib = _lib()
    rp_p = C.POINTER(C.c_uint32)()
    col_p = C.POINTER(C.c_uint32)()
    E = C.c_uint64()
    rc = lib.gdbgen_rmat(V, edge_factor, a, b, c, seed, C.byref(rp_p), C.byref(col_p), C.byref(E))
    if rc != 0:
        raise ValueError(f"rmat generation failed ({rc})")
    try:
        rp = np.ctypeslib.as_array(rp_p, shape=(V + 1,)).copy()
        col = np.ctypeslib.as_array(col_p, shape=(max(E.value, 1),))[: E.value].copy()
    finally:
        lib.gdbgen_free(rp_p)
        lib.gdbgen_free(col_p)
    return CSR(rp, col, None, f"rmat_V{V}_ef{edge_factor:g}",
               {"V": V, "edge_factor": edge_factor, "abc": (a, b, c), "seed": seed})


def rmat_scale(scale: int, edge_factor: float = 16, seed: int = 1) -> CSR:
    return rmat(1 << scale, edge_factor, seed=seed)


def uniform_weights(g: CSR, lo: int, hi: int, seed: int) -> np.ndarray:
    """One weight per undirected edge, uniform in [lo, hi]."""
    w = np.empty(max(g.E, 1), dtype=np.uint32)
    _lib().gdbgen_uniform_weights(g.V, g.row_ptr, np.ascontiguousarray(g.col) if g.E else w,
                                  seed, lo, hi, w)
    return w[: g.E]


def unique_weights(g: CSR, seed: int) -> np.ndarray:
    """Seeded permutation of 1..E_undirected, same value on both arcs."""
    w = np.empty(max(g.E, 1), dtype=np.uint32)
    _lib().gdbgen_unique_weights(g.V, g.row_ptr, g.col if g.E else w, seed, w)
    return w[: g.E]


def permutation(n: int, seed: int) -> np.ndarray:
    out = np.empty(max(n, 1), dtype=np.uint32)
    _lib().gdbgen_permutation(n, seed, out)
    return out[:n]


def priorities(n: int, seed: int) -> np.ndarray:
    """Seeded permutation of 0..n-1 as exact float32 values (n <= 2**24)."""
    if n > (1 << 24):
        raise ValueError("priorities above 2**24 are not exact in float32")
    return permutation(n, seed).astype(np.float32)


def sources(g: CSR, count: int, seed: int) -> np.ndarray:
    out = np.empty(max(count, 1), dtype=np.uint32)
    got = _lib().gdbgen_sources(g.V, g.row_ptr, seed, count, out)
    return out[:got]


def transpose(g: CSR) -> CSR:
    lib = _lib()
    trp = np.empty(g.V + 1, dtype=np.uint32)
    tcol = np.empty(max(g.E, 1), dtype=np.uint32)
    tw = np.empty(max(g.E, 1), dtype=np.uint32) if g.w is not None else None
    lib.gdbgen_transpose(g.V, g.row_ptr, g.col if g.E else tcol,
                         g.w.ctypes.data if g.w is not None else None, trp, tcol,
                         tw.ctypes.data if tw is not None else None)
    return CSR(trp, tcol[: g.E], tw[: g.E] if tw is not None else None, g.name + "_T")


def from_edges(V: int, pairs, weights=None, symmetric: bool = True) -> CSR:
    """Small CSR from an edge list (tests): symmetrised, deduplicated, sorted.
    With weights, the weight of {u, v} is taken from its first occurrence."""
    arcs = {}
    for i, (u, v) in enumerate(pairs):
        if u == v:
            continue
        wt = int(weights[i]) if weights is not None else 1
        arcs.setdefault((u, v), wt)
        if symmetric:
            arcs.setdefault((v, u), arcs[(u, v)])
    keys = sorted(arcs)
    rp = np.zeros(V + 1, dtype=np.uint32)
    for (u, _v) in keys:
        rp[u + 1] += 1
    rp = np.cumsum(rp, dtype=np.uint64).astype(np.uint32)
    col = np.array([v for (_u, v) in keys], dtype=np.uint32)
    w = np.array([arcs[k] for k in keys], dtype=np.uint32) if weights is not None else None
    return CSR(rp, col, w, f"edges_V{V}")


def _splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def _unit(seed: int, i: int, k: int) -> float:
    """Counter-based uniform in [0, 1) for member i, draw k."""
    return (_splitmix64((seed << 40) ^ (i << 8) ^ k) >> 11) / float(1 << 53)


def mixed_batch_spec(n: int, vmin: int = 1000, vmax: int = 1_000_000, seed: int = 1,
                     max_aspect: float = 64.0) -> list[dict]:
    """The shape of every member of mixed_batch(n, ...) without building it:
    kind, V, edge factor (R-MAT) or rows x cols (grid), and the arcs the
    member will hold (grids exactly, R-MAT the 2 x ef x V pairs before
    de-duplication)."""
    out = []
    lo, hi = np.log(vmin), np.log(vmax)
    for i in range(n):
        V = int(round(np.exp(lo + _unit(seed, i, 0) * (hi - lo))))
        if i % 2 == 0:
            ef = 8 + int(_unit(seed, i, 1) * 25)
            out.append({"i": i, "kind": "rmat", "V": V, "ef": ef, "arcs": 2 * ef * V})
        else:
            aspect = float(np.exp(_unit(seed, i, 2) * np.log(max_aspect)))
            rows = max(1, int(round(np.sqrt(V / aspect))))
            cols = max(1, int(round(V / rows)))
            out.append({"i": i, "kind": "grid", "V": rows * cols, "rows": rows, "cols": cols,
                        "arcs": 2 * (rows * (cols - 1) + cols * (rows - 1))})
    return out


def mixed_batch(n: int, vmin: int = 1000, vmax: int = 1_000_000, seed: int = 1,
                max_aspect: float = 64.0, members=None) -> list[CSR]:
    """The mixed batch workload: n graphs with vertex counts log-uniform in
    [vmin, vmax]; even members are R-MAT (edge factor uniform in 8..32,
    (a,b,c,d) = (0.57,0.19,0.19,0.05)), odd members 2-D grids whose aspect
    ratio is log-uniform in [1, max_aspect].  Each member carries weights
    (R-MAT uniform [1,255], grid uniform [1,1000]) and meta["source"], one
    seeded non-isolated vertex.  `members`: build only these member indices
    (in the order given), each identical to its copy in the full batch."""
    out = []
    spec = mixed_batch_spec(n, vmin, vmax, seed, max_aspect)
    for i in (range(n) if members is None else members):
        m = spec[i]
        gseed = (seed << 20) + i
        if m["kind"] == "rmat":
            g = rmat(m["V"], m["ef"], seed=gseed)
            w = uniform_weights(g, 1, 255, gseed)
        else:
            g = grid(m["rows"], m["cols"])
            w = uniform_weights(g, 1, 1000, gseed)
        g = g.with_weights(w)
        s = sources(g, 1, gseed)
        g.meta["source"] = int(s[0]) if len(s) else 0
        g.meta["kind"] = m["kind"]
        g.meta["member"] = i
        out.append(g)
    return out
