"""CPU oracle for the discovery-barrier graph path -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs may
import this package, as the checker (or as the timed CPU baseline).  The
product path never does.

* ``oracle.c`` restates each reference kernel in plain C (citations inside).
* ``refshim/`` compiles the reference's own OpenCL C kernels as C++ into
  ``_ref/libgdbref.so`` where the reference checkout exists, to pin the
  restatement (tests/test_oracle_golden.py, tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LONESTAR_INF = 1_000_000_000
PANNOTIA_BIG = 99_999_999

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

_ORC = None
_REF = None


def _nz(a: np.ndarray, dtype=np.uint32) -> np.ndarray:
    """ctypes needs a non-empty buffer even for E == 0."""
    a = np.ascontiguousarray(a, dtype=dtype)
    return a if a.size else np.zeros(1, dtype=dtype)


def lib() -> C.CDLL:
    global _ORC
    if _ORC is None:
        path = HERE / "_build" / "liboracle.so"
        if not path.exists():
            import sys
            sys.path.insert(0, str(HERE.parent))
            from gpu_discovery_barrier_gb300 import build
            build.build_oracle()
        L = C.CDLL(str(path))
        U32, P = C.c_uint32, C.c_void_p
        L.orc_bfs.argtypes = [U32, _u32p, _u32p, U32, _u32p]
        L.orc_sssp_worklist.argtypes = [U32, _u32p, _u32p, _u32p, U32, _u32p]
        L.orc_sssp_jacobi.argtypes = [U32, _u32p, _u32p, _u32p, U32, _i32p, C.POINTER(U32)]
        L.orc_sssp_dijkstra_int.argtypes = [U32, _u32p, _u32p, _u32p, U32, _i32p]
        L.orc_mis.argtypes = [U32, _u32p, _u32p, _f32p, _i32p, C.POINTER(U32)]
        L.orc_color.argtypes = [U32, _u32p, _u32p, _f32p, _i32p, C.POINTER(U32)]
        L.orc_color_fast.argtypes = [U32, _u32p, _u32p, _f32p, _i32p, C.POINTER(U32)]
        L.orc_bc_f32.argtypes = [U32, _u32p, _u32p, _u32p, _u32p, _u32p, U32, _f32p]
        L.orc_bc_f64.argtypes = [U32, _u32p, _u32p, _u32p, U32, _f64p]
        L.orc_mst.argtypes = [U32, _u32p, _u32p, _u32p, C.POINTER(C.c_uint64), C.POINTER(U32),
                              C.POINTER(U32), C.POINTER(U32), P]
        L.orc_verify_dist.restype = C.c_uint64
        L.orc_verify_dist.argtypes = [U32, _u32p, _u32p, P, _u32p]
        L.orc_bfs_reached_arcs.restype = C.c_uint64
        L.orc_bfs_reached_arcs.argtypes = [U32, _u32p, _u32p, U32, C.POINTER(U32)]
        L.orc_dmr_neighbours.argtypes = [U32, _u32p, _u32p]
        L.orc_dmr_refine.argtypes = [_f64p, _f64p, U32, _u32p, U32, U32, U32, _f64p, _f64p, _u32p,
                                     _u32p, _u8p, _u32p]
        L.orc_dmr_count_bad.restype = U32
        L.orc_dmr_count_bad.argtypes = [_f64p, _f64p, U32, _u32p, _u8p]
        L.orc_par_threads.restype = C.c_int
        L.orc_par_bfs.argtypes = [U32, _u32p, _u32p, U32, _u32p]
        U64, PU32 = C.c_uint64, C.POINTER(C.POINTER(U32))
        L.orc_gen_rmat.argtypes = [U32, C.c_double, C.c_double, C.c_double, C.c_double, U64,
                                   PU32, PU32, C.POINTER(U64)]
        L.orc_gen_free.argtypes = [P]
        L.orc_gen_uniform_weights.argtypes = [U32, _u32p, _u32p, U64, U32, U32, _u32p]
        L.orc_gen_permutation.argtypes = [U32, U64, _u32p]
        L.orc_gen_unique_weights.restype = U64
        L.orc_gen_unique_weights.argtypes = [U32, _u32p, _u32p, U64, _u32p]
        L.orc_gen_sources.restype = U32
        L.orc_gen_sources.argtypes = [U32, _u32p, U64, U32, _u32p]
        _ORC = L
    return _ORC


class Graph:
    """Plain CSR holder for graphs the oracle generates itself."""

    def __init__(self, row_ptr: np.ndarray, col: np.ndarray, w: np.ndarray | None = None):
        self.row_ptr, self.col, self.w = row_ptr, col, w

    @property
    def V(self) -> int:
        return int(self.row_ptr.shape[0] - 1)

    @property
    def E(self) -> int:
        return int(self.col.shape[0])

    def degrees(self) -> np.ndarray:
        return np.diff(self.row_ptr.astype(np.int64))

    def with_weights(self, w: np.ndarray) -> "Graph":
        return Graph(self.row_ptr, self.col, np.ascontiguousarray(w, dtype=np.uint32))


def gen_rmat(V: int, edge_factor: float, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1) -> Graph:
    """The seeded R-MAT workload graph (oracle_gen.c), symmetric uint32 CSR."""
    rp_p, col_p = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)()
    E = C.c_uint64()
    _check(lib().orc_gen_rmat(V, edge_factor, a, b, c, seed, C.byref(rp_p), C.byref(col_p),
                              C.byref(E)), "gen_rmat")
    try:
        rp = np.ctypeslib.as_array(rp_p, shape=(V + 1,)).copy()
        col = np.ctypeslib.as_array(col_p, shape=(max(E.value, 1),))[: E.value].copy()
    finally:
        lib().orc_gen_free(rp_p)
        lib().orc_gen_free(col_p)
    return Graph(rp, col)


def gen_uniform_weights(g, lo: int, hi: int, seed: int) -> np.ndarray:
    w = np.empty(max(g.E, 1), dtype=np.uint32)
    lib().orc_gen_uniform_weights(g.V, g.row_ptr, _nz(g.col), seed, lo, hi, w)
    return w[: g.E]


def gen_unique_weights(g, seed: int) -> np.ndarray:
    w = np.empty(max(g.E, 1), dtype=np.uint32)
    lib().orc_gen_unique_weights(g.V, g.row_ptr, _nz(g.col), seed, w)
    return w[: g.E]


def gen_permutation(n: int, seed: int) -> np.ndarray:
    out = np.empty(max(n, 1), dtype=np.uint32)
    lib().orc_gen_permutation(n, seed, out)
    return out[:n]


def gen_priorities(n: int, seed: int) -> np.ndarray:
    return gen_permutation(n, seed).astype(np.float32)


def gen_sources(g, count: int, seed: int) -> np.ndarray:
    out = np.empty(max(count, 1), dtype=np.uint32)
    got = lib().orc_gen_sources(g.V, g.row_ptr, seed, count, out)
    return out[:got]


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with {rc}")


def bfs(g, src: int) -> np.ndarray:
    d = np.empty(g.V, dtype=np.uint32)
    _check(lib().orc_bfs(g.V, g.row_ptr, _nz(g.col), src, d), "bfs")
    return d


def par_bfs(g, src: int) -> np.ndarray:
    d = np.empty(g.V, dtype=np.uint32)
    _check(lib().orc_par_bfs(g.V, g.row_ptr, _nz(g.col), src, d), "par_bfs")
    return d


def par_threads() -> int:
    return int(lib().orc_par_threads())


def sssp_worklist(g, src: int) -> np.ndarray:
    d = np.empty(g.V, dtype=np.uint32)
    _check(lib().orc_sssp_worklist(g.V, g.row_ptr, _nz(g.col), _nz(g.w), src, d), "sssp")
    return d


def sssp_jacobi(g, src: int, literal: bool = False) -> np.ndarray:
    """Pannotia Jacobi SSSP costs; `literal` runs the iteration itself
    (O(diameter * E)), otherwise the same fixed point via Dijkstra."""
    c = np.empty(g.V, dtype=np.int32)
    if literal:
        it = C.c_uint32()
        _check(lib().orc_sssp_jacobi(g.V, g.row_ptr, _nz(g.col), _nz(g.w), src, c,
                                     C.byref(it)), "jacobi")
    else:
        _check(lib().orc_sssp_dijkstra_int(g.V, g.row_ptr, _nz(g.col), _nz(g.w), src, c),
               "jacobi")
    return c


def mis(g, prio: np.ndarray) -> tuple[np.ndarray, int]:
    s = np.empty(g.V, dtype=np.int32)
    r = C.c_uint32()
    _check(lib().orc_mis(g.V, g.row_ptr, _nz(g.col), np.ascontiguousarray(prio, np.float32), s,
                         C.byref(r)), "mis")
    return s, r.value


def color(g, prio: np.ndarray) -> tuple[np.ndarray, int]:
    c = np.empty(g.V, dtype=np.int32)
    r = C.c_uint32()
    _check(lib().orc_color(g.V, g.row_ptr, _nz(g.col), np.ascontiguousarray(prio, np.float32),
                           c, C.byref(r)), "color")
    return c, r.value


def color_fast(g, prio: np.ndarray) -> tuple[np.ndarray, int]:
    """Same colouring from its closed form (fast on large graphs)."""
    c = np.empty(g.V, dtype=np.int32)
    r = C.c_uint32()
    _check(lib().orc_color_fast(g.V, g.row_ptr, _nz(g.col), np.ascontiguousarray(prio, np.float32),
                                c, C.byref(r)), "color_fast")
    return c, r.value


def bc_f32(g, gt, srcs) -> np.ndarray:
    bc = np.zeros(g.V, dtype=np.float32)
    s = np.ascontiguousarray(srcs, dtype=np.uint32)
    _check(lib().orc_bc_f32(g.V, g.row_ptr, _nz(g.col), gt.row_ptr, _nz(gt.col), _nz(s), len(s),
                            bc), "bc_f32")
    return bc


def bc_f64(g, srcs) -> np.ndarray:
    bc = np.zeros(g.V, dtype=np.float64)
    s = np.ascontiguousarray(srcs, dtype=np.uint32)
    _check(lib().orc_bc_f64(g.V, g.row_ptr, _nz(g.col), _nz(s), len(s), bc), "bc_f64")
    return bc


def mst(g) -> dict:
    w64 = C.c_uint64()
    w32, comps, edges = C.c_uint32(), C.c_uint32(), C.c_uint32()
    flags = np.zeros(max(g.E, 1), dtype=np.uint8)
    _check(lib().orc_mst(g.V, g.row_ptr, _nz(g.col), _nz(g.w), C.byref(w64), C.byref(w32),
                         C.byref(comps), C.byref(edges), flags.ctypes.data), "mst")
    return {"weight64": w64.value, "weight32": w32.value, "components": comps.value,
            "edges": edges.value, "arc_in_mst": flags[: g.E]}


def verify_dist(g, dist: np.ndarray, weighted: bool) -> int:
    w = _nz(g.w) if weighted else None
    return int(lib().orc_verify_dist(g.V, g.row_ptr, _nz(g.col),
                                     w.ctypes.data if w is not None else None,
                                     np.ascontiguousarray(dist, np.uint32)))


def reached_arcs(g, dist: np.ndarray, inf: int) -> tuple[int, int]:
    r = C.c_uint32()
    arcs = lib().orc_bfs_reached_arcs(g.V, g.row_ptr, np.ascontiguousarray(dist, np.uint32),
                                      inf, C.byref(r))
    return int(arcs), r.value


def mst_edge_set(g, arc_flags: np.ndarray) -> set:
    """Normalised {(min, max)} undirected edge set from per-arc flags."""
    src = np.repeat(np.arange(g.V, dtype=np.uint32), np.diff(g.row_ptr.astype(np.int64)))
    sel = np.nonzero(arc_flags[: g.E])[0]
    a, b = src[sel], g.col[sel]
    return set(zip(np.minimum(a, b).tolist(), np.maximum(a, b).tolist()))


# ---------------------------------------------------------------- reference


def _dmr_out(nnodes: int, nelements: int, maxfactor: int):
    mn, me = (maxfactor // 2) * nnodes, maxfactor * nelements
    return (np.zeros(mn, np.float64), np.zeros(mn, np.float64), np.zeros(3 * me, np.uint32),
            np.zeros(3 * me, np.uint32), np.zeros(me, np.uint8), np.zeros(5, np.uint32))


def _dmr_result(x, y, el, nb, isdel, counts) -> dict:
    nn, ne = int(counts[0]), int(counts[1])
    return {"x": x[:nn], "y": y[:nn], "elements": el[:3 * ne].reshape(ne, 3),
            "neighbours": nb[:3 * ne].reshape(ne, 3), "isdel": isdel[:ne],
            "rounds": int(counts[2]), "chunks": int(counts[3]), "refined": int(counts[4])}


def dmr_neighbours(elements: np.ndarray) -> np.ndarray:
    """find_neighbours_cpu (dmr.h:55-104): neighbour triples per element."""
    el = np.ascontiguousarray(elements, np.uint32).reshape(-1)
    nb = np.zeros_like(el)
    _check(lib().orc_dmr_neighbours(el.size // 3, el, nb), "dmr_neighbours")
    return nb.reshape(-1, 3)


def dmr_refine(mesh, chunk: int, maxfactor: int = 20) -> dict:
    """Refine `mesh` (meshgen.Mesh) with `chunk` items per superstep."""
    out = _dmr_out(mesh.nnodes, mesh.nelements, maxfactor)
    _check(lib().orc_dmr_refine(np.ascontiguousarray(mesh.x, np.float64),
                                np.ascontiguousarray(mesh.y, np.float64), mesh.nnodes,
                                np.ascontiguousarray(mesh.elements, np.uint32).reshape(-1),
                                mesh.nelements, maxfactor, chunk, *out), "dmr_refine")
    return _dmr_result(*out)


def dmr_count_bad(x, y, elements, isdel) -> int:
    """Live triangles with an angle below 30 degrees (angleLT)."""
    el = np.ascontiguousarray(elements, np.uint32).reshape(-1)
    return int(lib().orc_dmr_count_bad(np.ascontiguousarray(x, np.float64),
                                       np.ascontiguousarray(y, np.float64), el.size // 3, el,
                                       np.ascontiguousarray(isdel, np.uint8)))


def ref_dmr(mesh, maxfactor: int = 20) -> dict:
    """The reference's check_triangles / refine (one work-item) on `mesh`."""
    out = _dmr_out(mesh.nnodes, mesh.nelements, maxfactor)
    _check(ref().ref_dmr_lonestar(np.ascontiguousarray(mesh.x, np.float64),
                                  np.ascontiguousarray(mesh.y, np.float64), mesh.nnodes,
                                  np.ascontiguousarray(mesh.elements, np.uint32).reshape(-1),
                                  mesh.nelements, maxfactor, *out), "ref_dmr")
    return _dmr_result(*out)


def ref_available() -> bool:
    return (HERE / "_ref" / "libgdbref.so").exists()


def ref() -> C.CDLL:
    """The reference's own kernels (oracle/_ref/libgdbref.so)."""
    global _REF
    if _REF is None:
        L = C.CDLL(str(HERE / "_ref" / "libgdbref.so"))
        U32 = C.c_uint32
        L.ref_bfs_lonestar.argtypes = [U32, _u32p, _u32p, U32, _u32p]
        L.ref_sssp_lonestar.argtypes = [U32, _u32p, _u32p, _u32p, U32, _u32p]
        L.ref_sssp_pannotia.argtypes = [U32, _u32p, _u32p, _u32p, U32, _i32p]
        L.ref_mis_pannotia.argtypes = [U32, _u32p, _u32p, _f32p, _i32p]
        L.ref_color_pannotia.argtypes = [U32, _u32p, _u32p, _f32p, _i32p]
        L.ref_bc_pannotia_gb.argtypes = [U32, _u32p, _u32p, _u32p, _u32p, _f32p]
        L.ref_bc_pannotia_sources.argtypes = [U32, _u32p, _u32p, _u32p, _u32p, _u32p, U32, _f32p]
        L.ref_mst_lonestar.argtypes = [U32, _u32p, _u32p, _u32p, C.POINTER(U32), C.POINTER(U32),
                                       C.POINTER(U32)]
        L.ref_dmr_lonestar.argtypes = [_f64p, _f64p, U32, _u32p, U32, U32, _f64p, _f64p, _u32p,
                                       _u32p, _u8p, _u32p]
        L.ref_discovery_threads.argtypes = [C.c_int, C.c_int, _i32p, C.POINTER(C.c_int),
                                            C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _REF = L
    return _REF
