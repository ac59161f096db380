"""ctypes mirror of the C ABI in include/gdb.h.

The names follow the reference's host API and kernels:

* discovery (code/discovery_protocol/api/discovery.h): ``init_discovery_kernel_ctx``,
  ``init_discovery_kernel_ctx_skip``, ``number_of_participating_groups``,
  ``time_protocol``; occupancy tests (occupancy_tests/src/occupancy_test.c);
* one call per reference app: ``bfs`` (LonestarGPU bfs drelax2), ``sssp``
  (LonestarGPU sssp drelax2), ``sssp_jacobi`` (Pannotia sssp mega_kernel),
  ``mis``, ``color``, ``bc`` (Pannotia mega-kernels), ``mst`` (LonestarGPU mst).

There is no CPU fallback: if ``lib/libgdb.so`` is missing or a call fails, a
``GdbError`` is raised.  Every call runs on the context's own CUDA stream and
returns when its result is ready.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libgdb.so"

ABI_VERSION = 10  # GDB_ABI_VERSION of include/gdb.h
LONESTAR_INF = 1_000_000_000
PANNOTIA_BIG = 99_999_999

LOCK_TICKET, LOCK_SPIN, LOCK_FREE = 0, 1, 2
BARRIER_XF, BARRIER_GRID_SYNC, BARRIER_RELAUNCH, BARRIER_XF_FIXED, BARRIER_RELAUNCH_GRAPH = range(5)
SCHED_PLAIN, SCHED_ADAPTIVE, SCHED_LEARNED = 0, 1, 2
MLP_FEATURES, MLP_OUTPUTS, MLP_PARAMS = 12, 6, 1694

STATUS = {0: "GDB_OK", -1: "GDB_ERR_INVALID", -2: "GDB_ERR_CUDA", -3: "GDB_ERR_OOM",
          -4: "GDB_ERR_TIMEOUT", -5: "GDB_ERR_CAPACITY", -6: "GDB_ERR_NOT_CORESIDENT",
          -7: "GDB_ERR_UNSUPPORTED"}


class GdbError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}" + (f" ({detail})" if detail else ""))


class Options(C.Structure):
    _fields_ = [("device", C.c_int), ("block_size", C.c_int), ("max_ctas", C.c_int),
                ("oversubscribe", C.c_int), ("lock", C.c_int), ("barrier", C.c_int),
                ("schedule", C.c_int), ("xf_release", C.c_int), ("timeout_ns", C.c_uint64),
                ("pull_alpha", C.c_uint32), ("push_beta", C.c_uint32), ("sssp_delta", C.c_uint32),
                ("sssp_split", C.c_int), ("pull_bitmap_kb", C.c_int)]


class RunStats(C.Structure):
    _fields_ = [("supersteps", C.c_uint32), ("participating", C.c_uint32),
                ("launched", C.c_uint32), ("launches", C.c_uint32),
                ("edges_processed", C.c_uint64), ("work_units", C.c_uint64),
                ("kernel_ms", C.c_double), ("phases", C.c_uint32), ("sssp_delta", C.c_uint32),
                ("sssp_light", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class MstResult(C.Structure):
    _fields_ = [("weight64", C.c_uint64), ("weight32", C.c_uint32), ("components", C.c_uint32),
                ("edges", C.c_uint32), ("rounds", C.c_uint32)]


class LevelTrace(C.Structure):
    _fields_ = [("x", C.c_float * 12), ("mode", C.c_uint32), ("us", C.c_float)]


class Csr(C.Structure):
    _fields_ = [("V", C.c_uint32), ("E", C.c_uint64), ("row_ptr", C.POINTER(C.c_uint32)),
                ("col", C.POINTER(C.c_uint32)), ("w", C.POINTER(C.c_uint32))]


class RequestInfo(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("app", C.c_uint32), ("graph", C.c_uint32),
                ("src", C.c_uint32), ("slot", C.c_uint32), ("queue_ms", C.c_double),
                ("run_ms", C.c_double), ("total_ms", C.c_double), ("footprint", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class DeviceInfo(C.Structure):
    _fields_ = [("device", C.c_int), ("sm_count", C.c_int), ("cc_major", C.c_int),
                ("cc_minor", C.c_int), ("total_mem", C.c_size_t), ("occupancy_per_sm", C.c_int),
                ("flag_capacity", C.c_int)]


_LIB = None
_P = C.c_void_p
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

# (name, restype, argtypes) for every symbol of include/gdb.h
SIGNATURES = [
    ("gdb_options_default", None, [C.POINTER(Options)]),
    ("gdb_ctx_create", C.c_int, [C.POINTER(Options), C.POINTER(_P)]),
    ("gdb_ctx_destroy", C.c_int, [_P]),
    ("gdb_ctx_set_options", C.c_int, [_P, C.POINTER(Options)]),
    ("gdb_ctx_get_options", C.c_int, [_P, C.POINTER(Options)]),
    ("gdb_ctx_stream", C.c_int, [_P, C.POINTER(_P)]),
    ("gdb_device_info_get", C.c_int, [_P, C.POINTER(DeviceInfo)]),
    ("gdb_status_string", C.c_char_p, [C.c_int]),
    ("gdb_last_error", C.c_char_p, [_P]),
    ("gdb_last_run_stats", C.c_int, [_P, C.POINTER(RunStats)]),
    ("gdb_abi_version", C.c_int, []),
    ("gdb_init_discovery_kernel_ctx", C.c_int, [_P]),
    ("gdb_init_discovery_kernel_ctx_skip", C.c_int, [_P, C.c_int]),
    ("gdb_number_of_participating_groups", C.c_int, [_P]),
    ("gdb_time_protocol", C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    ("gdb_occupancy_test", C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("gdb_api_occupancy", C.c_int, [_P, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("gdb_barrier_bench", C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                    C.POINTER(C.c_int)]),
    ("gdb_debug_stall_master", C.c_int, [_P, C.c_int]),
    ("gdb_graph_create", C.c_int, [_P, C.c_uint32, C.c_uint64, _P, _P, _P, C.POINTER(_P)]),
    ("gdb_graph_create_device", C.c_int, [_P, C.c_uint32, C.c_uint64, _P, _P, _P, C.POINTER(_P)]),
    ("gdb_graph_set_weights", C.c_int, [_P, _P]),
    ("gdb_graph_set_symmetric", C.c_int, [_P, C.c_int]),
    ("gdb_graph_destroy", C.c_int, [_P]),
    ("gdb_graph_info", C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_uint32)]),
    ("gdb_bfs", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_bfs_device", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_sssp", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_sssp_device", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_sssp_jacobi", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_sssp_jacobi_device", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_mis", C.c_int, [_P, _P, _P, _P]),
    ("gdb_mis_device", C.c_int, [_P, _P, _P, _P]),
    ("gdb_color", C.c_int, [_P, _P, _P, _P]),
    ("gdb_color_device", C.c_int, [_P, _P, _P, _P]),
    ("gdb_bc", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_bc_device", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_mst", C.c_int, [_P, _P, C.POINTER(MstResult), _P]),
    ("gdb_mst_device", C.c_int, [_P, _P, _P, _P]),
    ("gdb_csr_read", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(Csr)]),
    ("gdb_csr_free", None, [C.POINTER(Csr)]),
    ("gdb_csr_write_gr", C.c_int, [C.c_char_p, C.POINTER(Csr)]),
    ("gdb_io_last_error", C.c_char_p, []),
    ("gdb_selector_set", C.c_int, [_P, _P]),
    ("gdb_bfs_trace", C.c_int, [_P, _P, C.c_uint32, C.c_int, _P, _P, C.c_uint32,
                                C.POINTER(C.c_uint32)]),
    ("gdb_sssp_features", C.c_int, [_P, _P, C.c_uint32, _P]),
    ("gdb_sssp_trace", C.c_int, [_P, _P, C.c_uint32, C.c_int, _P, _P, C.c_uint32,
                                 C.POINTER(C.c_uint32)]),
    ("gdb_mlp_forward", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_mlp_loss_grad", C.c_int, [_P, _P, _P, _P, _P, C.c_uint32, _P, C.POINTER(C.c_double)]),
    ("gdb_mlp_train", C.c_int, [_P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_float, C.c_float,
                                C.POINTER(C.c_double)]),
    ("gdb_bfs_multi", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_bfs_sources", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_bfs_sources_device", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_sssp_sources", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_sssp_sources_device", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_bfs_multi_device", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_sssp_multi", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_sssp_multi_device", C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    ("gdb_graph_create_batch", C.c_int, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P, C.POINTER(_P)]),
    ("gdb_batch_create", C.c_int, [_P, _P, C.c_uint32, _P, C.c_uint32, C.POINTER(_P)]),
    ("gdb_batch_set_sources", C.c_int, [_P, _P]),
    ("gdb_batch_launch", C.c_int, [_P]),
    ("gdb_batch_wait", C.c_int, [_P, C.POINTER(C.c_double)]),
    ("gdb_batch_run", C.c_int, [_P, C.POINTER(C.c_double)]),
    ("gdb_batch_results", C.c_int, [_P, _P, _P]),
    ("gdb_batch_device_result", _P, [_P, C.c_uint32]),
    ("gdb_batch_app_stats", C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]),
    ("gdb_batch_destroy", C.c_int, [_P]),
    ("gdb_server_create", C.c_int, [_P, C.c_uint32, C.c_uint64, C.POINTER(_P)]),
    ("gdb_server_add_graph", C.c_int, [_P, _P, C.POINTER(C.c_uint32)]),
    ("gdb_server_submit", C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P, C.POINTER(C.c_uint64)]),
    ("gdb_server_poll", C.c_int, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    ("gdb_server_drain", C.c_int, [_P, C.c_double]),
    ("gdb_server_destroy", C.c_int, [_P]),
    ("gdb_bfs_noalloc", C.c_int, [_P, _P, C.c_uint32, C.c_uint64, C.c_uint32, _P, _P]),
    ("gdb_dmr_refine", C.c_int, [_P, _P, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, C.c_uint32,
                                 _P, _P, _P, _P, _P, _P]),
]

APP_BFS, APP_SSSP, APP_BC = 1, 2, 3
FMT_AUTO, FMT_GR, FMT_DIMACS, FMT_METIS = 0, 1, 2, 3


def read_graph(path, fmt: int = FMT_AUTO, directed: bool = False):
    """gdb_csr_read: a .gr / DIMACS / METIS file as a graphgen.CSR
    (weights in ``w`` when the file has them)."""
    from .graphgen import CSR

    c = Csr()
    L = lib()
    rc = L.gdb_csr_read(str(path).encode(), fmt, int(directed), C.byref(c))
    if rc != 0:
        raise GdbError(rc, "gdb_csr_read", L.gdb_io_last_error().decode())
    try:
        rp = np.ctypeslib.as_array(c.row_ptr, shape=(c.V + 1,)).copy()
        col = np.ctypeslib.as_array(c.col, shape=(max(c.E, 1),))[: c.E].copy()
        w = np.ctypeslib.as_array(c.w, shape=(max(c.E, 1),))[: c.E].copy() if c.w else None
    finally:
        L.gdb_csr_free(C.byref(c))
    return CSR(rp, col, w, Path(path).name)


def write_gr(path, g) -> None:
    """gdb_csr_write_gr: write a CSR (row_ptr, col, optional w) as .gr v1."""
    rp = np.ascontiguousarray(g.row_ptr, dtype=np.uint32)
    col = np.ascontiguousarray(g.col, dtype=np.uint32)
    w = None if g.w is None else np.ascontiguousarray(g.w, dtype=np.uint32)
    u32 = C.POINTER(C.c_uint32)
    c = Csr(rp.shape[0] - 1, col.shape[0], rp.ctypes.data_as(u32), col.ctypes.data_as(u32),
            w.ctypes.data_as(u32) if w is not None else None)
    L = lib()
    rc = L.gdb_csr_write_gr(str(path).encode(), C.byref(c))
    if rc != 0:
        raise GdbError(rc, "gdb_csr_write_gr", L.gdb_io_last_error().decode())

BATCH_BFS, BATCH_SSSP = 1, 2

NOALLOC_MAX_VERTICES = 1 << 20


def bfs_noalloc(d_row_ptr: int, d_col: int, V: int, E: int, src: int, d_dist: int,
                stream: int = 0) -> None:
    """gdb_bfs_noalloc: BFS from device pointers without any device
    allocation (see include/gdb.h); raises GdbError on failure."""
    rc = lib().gdb_bfs_noalloc(d_row_ptr, d_col, V, E, src, d_dist, stream)
    if rc != 0:
        raise GdbError(rc, "gdb_bfs_noalloc")


class DeviceArray:
    """A library-owned device array exposed through __cuda_array_interface__
    (zero copy), e.g. ``torch.as_tensor(DeviceArray(p, n), device="cuda")``."""

    def __init__(self, ptr: int, n: int, typestr: str = "<u4"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


def lib() -> C.CDLL:
    """Load lib/libgdb.so; raises when it has not been built."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise GdbError(-2, "libgdb", f"{LIB_PATH} missing -- run __graft_entry__.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.gdb_abi_version() != ABI_VERSION:
            raise GdbError(-1, "libgdb", f"ABI {L.gdb_abi_version()} != {ABI_VERSION}: rebuild")
        _LIB = L
    return _LIB


def default_options(**kw) -> Options:
    o = Options()
    lib().gdb_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _out(out, n: int, dtype) -> np.ndarray:
    """The result array of a call: a fresh one, or the caller's (checked)."""
    if out is None:
        return np.empty(n, dtype=dtype)
    if out.dtype != np.dtype(dtype) or out.shape != (n,) or not out.flags["C_CONTIGUOUS"] \
            or not out.flags["WRITEABLE"]:
        raise ValueError(f"out must be a writable contiguous {np.dtype(dtype).name}[{n}] array")
    return out


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


class Ctx:
    """A gdb_ctx: one CUDA stream, the discovery context, a workspace."""

    def __init__(self, **options):
        self._lib = lib()
        self.opt = default_options(**options)
        h = _P()
        rc = self._lib.gdb_ctx_create(C.byref(self.opt), C.byref(h))
        if rc != 0:
            raise GdbError(rc, "gdb_ctx_create")
        self.h = h

    # -- plumbing
    def check(self, rc: int, where: str) -> int:
        if rc < 0:
            raise GdbError(rc, where, self._lib.gdb_last_error(self.h).decode())
        return rc

    def close(self) -> None:
        if getattr(self, "h", None):
            self._lib.gdb_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_options(self, **kw) -> None:
        o = Options()
        self.check(self._lib.gdb_ctx_get_options(self.h, C.byref(o)), "gdb_ctx_get_options")
        for k, v in kw.items():
            setattr(o, k, v)
        self.check(self._lib.gdb_ctx_set_options(self.h, C.byref(o)), "gdb_ctx_set_options")
        self.opt = o

    def stream(self) -> int:
        s = _P()
        self.check(self._lib.gdb_ctx_stream(self.h, C.byref(s)), "gdb_ctx_stream")
        return s.value or 0

    def device_info(self) -> dict:
        d = DeviceInfo()
        self.check(self._lib.gdb_device_info_get(self.h, C.byref(d)), "gdb_device_info_get")
        return {k: getattr(d, k) for k, _ in d._fields_}

    def last_stats(self) -> dict:
        s = RunStats()
        self.check(self._lib.gdb_last_run_stats(self.h, C.byref(s)), "gdb_last_run_stats")
        return s.as_dict()

    # -- discovery protocol / barrier (discovery.h)
    def init_discovery_kernel_ctx(self, skip: int | None = None) -> None:
        if skip is None:
            self.check(self._lib.gdb_init_discovery_kernel_ctx(self.h), "init_discovery_kernel_ctx")
        else:
            self.check(self._lib.gdb_init_discovery_kernel_ctx_skip(self.h, int(skip)),
                       "init_discovery_kernel_ctx_skip")

    def number_of_participating_groups(self) -> int:
        return self.check(self._lib.gdb_number_of_participating_groups(self.h),
                          "number_of_participating_groups")

    def time_protocol(self, upper_bound: int, wgs: int) -> float:
        ns = C.c_double()
        self.check(self._lib.gdb_time_protocol(self.h, upper_bound, wgs, C.byref(ns)), "time_protocol")
        return ns.value

    def occupancy_test(self, wgc: int, wgs: int, lms: int = 0) -> int:
        n = C.c_int()
        self.check(self._lib.gdb_occupancy_test(self.h, wgc, wgs, lms, C.byref(n)), "occupancy_test")
        return n.value

    def api_occupancy(self, wgs: int, lms: int = 0) -> int:
        n = C.c_int()
        self.check(self._lib.gdb_api_occupancy(self.h, wgs, lms, C.byref(n)), "api_occupancy")
        return n.value

    def barrier_bench(self, kind: int, wgs: int = 0, iters: int = 1000) -> tuple[float, int]:
        ns, groups = C.c_double(), C.c_int()
        self.check(self._lib.gdb_barrier_bench(self.h, kind, wgs, iters, C.byref(ns), C.byref(groups)),
                   "barrier_bench")
        return ns.value, groups.value

    def debug_stall_master(self, after_barriers: int) -> None:
        self.check(self._lib.gdb_debug_stall_master(self.h, after_barriers), "debug_stall_master")

    # -- graphs
    def graph(self, row_ptr: np.ndarray, col: np.ndarray, w: np.ndarray | None = None,
              symmetric: bool = False) -> "Graph":
        return Graph(self, row_ptr, col, w, symmetric=symmetric)

    # -- applications (host buffers)
    def bfs(self, g: "Graph", src: int, out: np.ndarray | None = None) -> np.ndarray:
        """BFS levels from src.  `out`: an optional caller-owned result
        array (V uint32); page-locked host memory makes the read-back a
        direct DMA instead of a staged copy."""
        out = _out(out, g.V, np.uint32)
        self.check(self._lib.gdb_bfs(self.h, g.h, src, _ptr(out)), "gdb_bfs")
        return out

    def sssp(self, g: "Graph", src: int, out: np.ndarray | None = None) -> np.ndarray:
        out = _out(out, g.V, np.uint32)
        self.check(self._lib.gdb_sssp(self.h, g.h, src, _ptr(out)), "gdb_sssp")
        return out

    def sssp_jacobi(self, g: "Graph", src: int) -> np.ndarray:
        out = np.empty(g.V, dtype=np.int32)
        self.check(self._lib.gdb_sssp_jacobi(self.h, g.h, src, _ptr(out)), "gdb_sssp_jacobi")
        return out

    def mis(self, g: "Graph", node_value: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        nv = np.ascontiguousarray(node_value, dtype=np.float32)
        out = _out(out, g.V, np.int32)
        self.check(self._lib.gdb_mis(self.h, g.h, _ptr(nv), _ptr(out)), "gdb_mis")
        return out

    def color(self, g: "Graph", node_value: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        nv = np.ascontiguousarray(node_value, dtype=np.float32)
        out = _out(out, g.V, np.int32)
        self.check(self._lib.gdb_color(self.h, g.h, _ptr(nv), _ptr(out)), "gdb_color")
        return out

    def bc(self, g: "Graph", sources, out: np.ndarray | None = None) -> np.ndarray:
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = _out(out, g.V, np.float32)
        self.check(self._lib.gdb_bc(self.h, g.h, _ptr(s), len(s), _ptr(out)), "gdb_bc")
        return out

    def mst(self, g: "Graph", with_arcs: bool = False) -> dict:
        r = MstResult()
        flags = np.zeros(max(g.E, 1), dtype=np.uint8) if with_arcs else None
        self.check(self._lib.gdb_mst(self.h, g.h, C.byref(r), _ptr(flags)), "gdb_mst")
        out = {k: getattr(r, k) for k, _ in r._fields_}
        if with_arcs:
            out["arc_in_mst"] = flags[: g.E]
        return out

    def dmr_refine(self, mesh, chunk: int, maxfactor: int = 20) -> dict:
        """Delaunay mesh refinement of `mesh` (meshgen.Mesh: x, y, elements)
        with `chunk` items per superstep; the refined mesh and its counts."""
        x = np.ascontiguousarray(mesh.x, np.float64)
        y = np.ascontiguousarray(mesh.y, np.float64)
        el = np.ascontiguousarray(mesh.elements, np.uint32).reshape(-1)
        nn, ne = x.size, el.size // 3
        mn, me = (maxfactor // 2) * nn, maxfactor * ne
        xo, yo = np.zeros(mn, np.float64), np.zeros(mn, np.float64)
        elo, nbo = np.zeros(3 * me, np.uint32), np.zeros(3 * me, np.uint32)
        delo, counts = np.zeros(me, np.uint8), np.zeros(5, np.uint32)
        self.check(self._lib.gdb_dmr_refine(self.h, _ptr(x), _ptr(y), nn, _ptr(el), ne, maxfactor, chunk,
                                            _ptr(xo), _ptr(yo), _ptr(elo), _ptr(nbo), _ptr(delo),
                                            _ptr(counts)), "gdb_dmr_refine")
        n, e = int(counts[0]), int(counts[1])
        return {"x": xo[:n], "y": yo[:n], "elements": elo[:3 * e].reshape(e, 3),
                "neighbours": nbo[:3 * e].reshape(e, 3), "isdel": delo[:e], "rounds": int(counts[2]),
                "chunks": int(counts[3]), "refined": int(counts[4])}

    # -- schedule selector (no reference counterpart)
    def selector_set(self, params: np.ndarray | None) -> None:
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        if p is not None and p.size != MLP_PARAMS:
            raise GdbError(-1, "gdb_selector_set", f"{p.size} parameters, want {MLP_PARAMS}")
        self.check(self._lib.gdb_selector_set(self.h, _ptr(p)), "gdb_selector_set")
        self.has_selector = p is not None

    def bfs_trace(self, g: "Graph", src: int, mode: int, cap: int = 1 << 16):
        """BFS with every level pushed (0), pulled (1) or chosen by the
        selector (2); returns (levels, features[L, 12], modes[L], us[L])."""
        rec = (LevelTrace * max(cap, 1))()
        dist = np.empty(g.V, dtype=np.uint32)
        n = C.c_uint32()
        self.check(self._lib.gdb_bfs_trace(self.h, g.h, src, mode, _ptr(dist), rec, cap, C.byref(n)),
                   "gdb_bfs_trace")
        L = min(n.value, cap)
        arr = np.frombuffer(rec, dtype=np.float32, count=14 * max(cap, 1)).reshape(-1, 14)[:L]
        modes = np.frombuffer(rec, dtype=np.uint32, count=14 * max(cap, 1)).reshape(-1, 14)[:L, 12]
        return dist, arr[:, :12].copy(), modes.copy(), arr[:, 13].copy()

    def sssp_trace(self, g: "Graph", src: int, mode: int, cap: int = 1 << 14):
        """SSSP with every settle superstep pushed (0), pulled (1) or chosen
        by the selector (2); returns (dist, features[S, 12], modes[S], us[S])
        over the S settle supersteps."""
        rec = (LevelTrace * max(cap, 1))()
        dist = np.empty(g.V, dtype=np.uint32)
        n = C.c_uint32()
        self.check(self._lib.gdb_sssp_trace(self.h, g.h, src, mode, _ptr(dist), rec, cap, C.byref(n)),
                   "gdb_sssp_trace")
        S = min(n.value, cap)
        arr = np.frombuffer(rec, dtype=np.float32, count=14 * max(cap, 1)).reshape(-1, 14)[:S]
        modes = np.frombuffer(rec, dtype=np.uint32, count=14 * max(cap, 1)).reshape(-1, 14)[:S, 12]
        return dist, arr[:, :12].copy(), modes.copy(), arr[:, 13].copy()

    def sssp_features(self, g: "Graph", nsrc: int = 1) -> np.ndarray:
        x = np.empty(MLP_FEATURES, dtype=np.float32)
        self.check(self._lib.gdb_sssp_features(self.h, g.h, nsrc, _ptr(x)), "gdb_sssp_features")
        return x

    def mlp_forward(self, params: np.ndarray, x: np.ndarray) -> np.ndarray:
        p = np.ascontiguousarray(params, dtype=np.float32)
        xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_FEATURES)
        y = np.empty((xx.shape[0], MLP_OUTPUTS), dtype=np.float32)
        self.check(self._lib.gdb_mlp_forward(self.h, _ptr(p), _ptr(xx), xx.shape[0], _ptr(y)),
                   "gdb_mlp_forward")
        return y

    def mlp_loss_grad(self, params, x, t, m) -> tuple[float, np.ndarray]:
        p = np.ascontiguousarray(params, dtype=np.float32)
        xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_FEATURES)
        tt = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, MLP_OUTPUTS)
        mm = np.ascontiguousarray(m, dtype=np.float32).reshape(-1, MLP_OUTPUTS)
        g = np.empty(MLP_PARAMS, dtype=np.float32)
        loss = C.c_double()
        self.check(self._lib.gdb_mlp_loss_grad(self.h, _ptr(p), _ptr(xx), _ptr(tt), _ptr(mm),
                                               xx.shape[0], _ptr(g), C.byref(loss)), "gdb_mlp_loss_grad")
        return loss.value, g

    def mlp_train(self, params, x, t, m, epochs: int, lr: float = 1e-2, wd: float = 0.0):
        p = np.array(params, dtype=np.float32, copy=True)
        xx = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_FEATURES)
        tt = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, MLP_OUTPUTS)
        mm = np.ascontiguousarray(m, dtype=np.float32).reshape(-1, MLP_OUTPUTS)
        loss = C.c_double()
        self.check(self._lib.gdb_mlp_train(self.h, _ptr(p), _ptr(xx), _ptr(tt), _ptr(mm), xx.shape[0],
                                           epochs, lr, wd, C.byref(loss)), "gdb_mlp_train")
        return p, loss.value

    # -- multi-source and batched forms (no reference counterpart)
    def bfs_multi(self, g: "Graph", sources) -> np.ndarray:
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = np.empty(g.V, dtype=np.uint32)
        self.check(self._lib.gdb_bfs_multi(self.h, g.h, _ptr(s), len(s), _ptr(out)), "gdb_bfs_multi")
        return out

    def sssp_multi(self, g: "Graph", sources) -> np.ndarray:
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = np.empty(g.V, dtype=np.uint32)
        self.check(self._lib.gdb_sssp_multi(self.h, g.h, _ptr(s), len(s), _ptr(out)), "gdb_sssp_multi")
        return out

    def graph_batch(self, graphs, weights: bool = True) -> "Graph":
        """Disjoint union of CSR graphs (objects with row_ptr, col and w);
        the result's ``vertex_offset`` maps member i to its vertex range."""
        return Graph.batch(self, graphs, weights)

    def batch(self, g: "Graph", sources, apps: int = 3) -> "Batch":
        return Batch(self, g, sources, apps)

    def server(self, slots: int = 8, pool_bytes: int = 1 << 30) -> "Server":
        return Server(self, slots, pool_bytes)

    # -- applications on device buffers (integer device pointers)
    def bfs_device(self, g: "Graph", src: int, d_dist: int) -> None:
        self.check(self._lib.gdb_bfs_device(self.h, g.h, src, d_dist), "gdb_bfs_device")

    def sssp_device(self, g: "Graph", src: int, d_dist: int) -> None:
        self.check(self._lib.gdb_sssp_device(self.h, g.h, src, d_dist), "gdb_sssp_device")

    def sssp_jacobi_device(self, g: "Graph", src: int, d_cost: int) -> None:
        self.check(self._lib.gdb_sssp_jacobi_device(self.h, g.h, src, d_cost), "gdb_sssp_jacobi_device")

    def mis_device(self, g: "Graph", d_prio: int, d_s: int) -> None:
        self.check(self._lib.gdb_mis_device(self.h, g.h, d_prio, d_s), "gdb_mis_device")

    def color_device(self, g: "Graph", d_prio: int, d_color: int) -> None:
        self.check(self._lib.gdb_color_device(self.h, g.h, d_prio, d_color), "gdb_color_device")

    def bc_device(self, g: "Graph", d_sources: int, nsrc: int, d_bc: int) -> None:
        self.check(self._lib.gdb_bc_device(self.h, g.h, d_sources, nsrc, d_bc), "gdb_bc_device")

    def mst_device(self, g: "Graph", d_result: int, d_flags: int | None = None) -> None:
        self.check(self._lib.gdb_mst_device(self.h, g.h, d_result, d_flags), "gdb_mst_device")

    def bfs_sources(self, g: "Graph", sources, out: np.ndarray | None = None) -> np.ndarray:
        """Independent BFS from each source: row i = levels from sources[i]."""
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = _out(None if out is None else out.reshape(-1), len(s) * g.V, np.uint32)
        self.check(self._lib.gdb_bfs_sources(self.h, g.h, _ptr(s), len(s), _ptr(out)), "gdb_bfs_sources")
        return out.reshape(len(s), g.V)

    def sssp_sources(self, g: "Graph", sources, out: np.ndarray | None = None) -> np.ndarray:
        """Independent SSSP from each source: row i = distances from sources[i]."""
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = _out(None if out is None else out.reshape(-1), len(s) * g.V, np.uint32)
        self.check(self._lib.gdb_sssp_sources(self.h, g.h, _ptr(s), len(s), _ptr(out)),
                   "gdb_sssp_sources")
        return out.reshape(len(s), g.V)

    def bfs_sources_device(self, g: "Graph", d_sources: int, n: int, d_dist: int) -> None:
        self.check(self._lib.gdb_bfs_sources_device(self.h, g.h, d_sources, n, d_dist),
                   "gdb_bfs_sources_device")

    def sssp_sources_device(self, g: "Graph", d_sources: int, n: int, d_dist: int) -> None:
        self.check(self._lib.gdb_sssp_sources_device(self.h, g.h, d_sources, n, d_dist),
                   "gdb_sssp_sources_device")

    def bfs_multi_device(self, g: "Graph", d_sources: int, nsrc: int, d_dist: int) -> None:
        self.check(self._lib.gdb_bfs_multi_device(self.h, g.h, d_sources, nsrc, d_dist),
                   "gdb_bfs_multi_device")

    def sssp_multi_device(self, g: "Graph", d_sources: int, nsrc: int, d_dist: int) -> None:
        self.check(self._lib.gdb_sssp_multi_device(self.h, g.h, d_sources, nsrc, d_dist),
                   "gdb_sssp_multi_device")


class Graph:
    """A gdb_graph: CSR copied from host arrays (or borrowed device arrays)."""

    def __init__(self, ctx: Ctx, row_ptr, col, w=None, device: bool = False,
                 symmetric: bool = False):
        """symmetric: declare that arc u -> v of weight w exists exactly when
        v -> u of weight w does (gdb_graph_set_symmetric)."""
        self.ctx = ctx
        h = _P()
        if device:
            # row_ptr/col/w are (pointer, length) device buffers
            (rp, V1), (cp, E) = row_ptr, col
            wp = w[0] if w is not None else None
            self.V, self.E = V1 - 1, E
            ctx.check(ctx._lib.gdb_graph_create_device(ctx.h, self.V, self.E, rp, cp, wp, C.byref(h)),
                      "gdb_graph_create_device")
        else:
            self._rp = np.ascontiguousarray(row_ptr, dtype=np.uint32)
            self._col = np.ascontiguousarray(col, dtype=np.uint32)
            if self._col.size == 0:
                self._col = np.zeros(1, dtype=np.uint32)
            self._w = None if w is None else np.ascontiguousarray(w, dtype=np.uint32)
            if self._w is not None and self._w.size == 0:
                self._w = np.zeros(1, dtype=np.uint32)
            self.V = int(self._rp.shape[0] - 1)
            self.E = int(np.asarray(col).shape[0])
            ctx.check(ctx._lib.gdb_graph_create(ctx.h, self.V, self.E, _ptr(self._rp), _ptr(self._col),
                                                _ptr(self._w), C.byref(h)), "gdb_graph_create")
        self.h = h
        if symmetric:
            self.set_symmetric(True)

    def set_symmetric(self, symmetric: bool) -> None:
        self.ctx.check(self.ctx._lib.gdb_graph_set_symmetric(self.h, int(bool(symmetric))),
                       "gdb_graph_set_symmetric")

    @classmethod
    def batch(cls, ctx: Ctx, graphs, weights: bool = True) -> "Graph":
        n = len(graphs)
        rps = [np.ascontiguousarray(g.row_ptr, dtype=np.uint32) for g in graphs]
        cols = [np.ascontiguousarray(g.col, dtype=np.uint32) for g in graphs]
        ws = [np.ascontiguousarray(g.w, dtype=np.uint32) for g in graphs] if weights else None
        Vs = np.array([r.shape[0] - 1 for r in rps], dtype=np.uint32)
        Es = np.array([c.shape[0] for c in cols], dtype=np.uint64)
        arr = lambda xs: (C.c_void_p * n)(*[x.ctypes.data for x in xs])  # noqa: E731
        rp_a, col_a = arr(rps), arr(cols)
        w_a = arr(ws) if weights else None
        off = np.empty(n + 1, dtype=np.uint32)
        h = _P()
        ctx.check(ctx._lib.gdb_graph_create_batch(ctx.h, n, _ptr(Vs), _ptr(Es), rp_a, col_a, w_a,
                                                  _ptr(off), C.byref(h)), "gdb_graph_create_batch")
        self = cls.__new__(cls)
        self.ctx, self.h = ctx, h
        self.V, self.E = int(off[n]), int(Es.sum())
        self.vertex_offset = off
        return self

    def set_weights(self, w: np.ndarray) -> None:
        self._w = np.ascontiguousarray(w, dtype=np.uint32)
        self.ctx.check(self.ctx._lib.gdb_graph_set_weights(self.h, _ptr(self._w)), "gdb_graph_set_weights")

    def info(self) -> dict:
        V, E, hv = C.c_uint32(), C.c_uint64(), C.c_uint32()
        self.ctx.check(self.ctx._lib.gdb_graph_info(self.h, C.byref(V), C.byref(E), C.byref(hv)),
                       "gdb_graph_info")
        return {"V": V.value, "E": E.value, "heavy": hv.value}

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx._lib.gdb_graph_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """A gdb_batch: BFS and/or SSSP from one source per member graph of a
    batch union, captured once into a CUDA graph and replayed by run()."""

    def __init__(self, ctx: Ctx, g: Graph, sources, apps: int = BATCH_BFS | BATCH_SSSP):
        self.ctx, self.g, self.apps = ctx, g, apps
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        self.nsrc = len(s)
        h = _P()
        ctx.check(ctx._lib.gdb_batch_create(ctx.h, g.h, apps, _ptr(s), len(s), C.byref(h)),
                  "gdb_batch_create")
        self.h = h

    def set_sources(self, sources) -> None:
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        if len(s) != self.nsrc:
            raise GdbError(-1, "gdb_batch_set_sources", "source count differs from the batch's")
        self.ctx.check(self.ctx._lib.gdb_batch_set_sources(self.h, _ptr(s)), "gdb_batch_set_sources")

    def run(self) -> float:
        ms = C.c_double()
        self.ctx.check(self.ctx._lib.gdb_batch_run(self.h, C.byref(ms)), "gdb_batch_run")
        return ms.value

    def launch(self) -> None:
        self.ctx.check(self.ctx._lib.gdb_batch_launch(self.h), "gdb_batch_launch")

    def wait(self) -> float:
        ms = C.c_double()
        self.ctx.check(self.ctx._lib.gdb_batch_wait(self.h, C.byref(ms)), "gdb_batch_wait")
        return ms.value

    def results(self) -> dict:
        out = {}
        b = np.empty(self.g.V, dtype=np.uint32) if self.apps & BATCH_BFS else None
        s = np.empty(self.g.V, dtype=np.uint32) if self.apps & BATCH_SSSP else None
        self.ctx.check(self.ctx._lib.gdb_batch_results(self.h, _ptr(b), _ptr(s)), "gdb_batch_results")
        if b is not None:
            out["bfs"] = b
        if s is not None:
            out["sssp"] = s
        return out

    def device_result(self, app: int) -> int:
        return self.ctx._lib.gdb_batch_device_result(self.h, app) or 0

    def app_stats(self, app: int) -> tuple[int, int]:
        arcs, steps = C.c_uint64(), C.c_uint32()
        self.ctx.check(self.ctx._lib.gdb_batch_app_stats(self.h, app, C.byref(arcs), C.byref(steps)),
                       "gdb_batch_app_stats")
        return arcs.value, steps.value

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx._lib.gdb_batch_destroy(self.h)
        self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A gdb_server: requests over resident graphs, continuously batched
    into slots.  submit() returns the request id and the numpy array the
    result is written into (uint32 levels / distances, float32 BC)."""

    def __init__(self, ctx: Ctx, slots: int = 8, pool_bytes: int = 1 << 30):
        self.ctx = ctx
        self._out: dict[int, np.ndarray] = {}
        self.graphs: list[Graph] = []
        h = _P()
        ctx.check(ctx._lib.gdb_server_create(ctx.h, slots, pool_bytes, C.byref(h)), "gdb_server_create")
        self.h = h

    def add_graph(self, g: Graph) -> int:
        gid = C.c_uint32()
        self.ctx.check(self.ctx._lib.gdb_server_add_graph(self.h, g.h, C.byref(gid)), "gdb_server_add_graph")
        self.graphs.append(g)
        return gid.value

    def submit(self, graph: int, app: int, src: int) -> tuple[int, np.ndarray]:
        V = self.graphs[graph].V
        out = np.empty(V, dtype=np.float32 if app == APP_BC else np.uint32)
        rid = C.c_uint64()
        self.ctx.check(self.ctx._lib.gdb_server_submit(self.h, graph, app, src, _ptr(out), C.byref(rid)),
                       "gdb_server_submit")
        self._out[rid.value] = out
        return rid.value, out

    def poll(self, max_n: int = 1024) -> list[dict]:
        buf = (RequestInfo * max_n)()
        n = C.c_uint32()
        self.ctx.check(self.ctx._lib.gdb_server_poll(self.h, buf, max_n, C.byref(n)), "gdb_server_poll")
        out = []
        for i in range(n.value):
            d = buf[i].as_dict()
            d["result"] = self._out.pop(d["id"], None)
            out.append(d)
        return out

    def drain(self, timeout_s: float = 0.0) -> None:
        self.ctx.check(self.ctx._lib.gdb_server_drain(self.h, timeout_s), "gdb_server_drain")

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx._lib.gdb_server_destroy(self.h)
        self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
