"""The C-ABI library loads and exports every symbol include/*.h declares
(no GPU needed: only symbol resolution, no compute calls)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(gdb_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_abi():
    syms = declared_symbols()
    for must in ["gdb_init_discovery_kernel_ctx", "gdb_init_discovery_kernel_ctx_skip",
                 "gdb_number_of_participating_groups", "gdb_time_protocol", "gdb_bfs", "gdb_sssp",
                 "gdb_sssp_jacobi", "gdb_mis", "gdb_color", "gdb_bc", "gdb_mst", "gdb_barrier_bench"]:
        assert must in syms


def test_library_exports_every_declared_symbol():
    from gpu_discovery_barrier_gb300 import gdb

    if not gdb.LIB_PATH.exists():
        from gpu_discovery_barrier_gb300 import build
        build.build_cuda()
    lib = ctypes.CDLL(str(gdb.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the Python mirror binds exactly the declared C ABI
    bound = {name for name, _, _ in gdb.SIGNATURES}
    assert bound == set(declared_symbols())


def test_no_compute_calls_needed_for_abi_version():
    from gpu_discovery_barrier_gb300 import gdb

    assert gdb.lib().gdb_abi_version() == 1
    assert gdb.lib().gdb_status_string(-4) == b"GDB_ERR_TIMEOUT"
