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

    assert gdb.lib().gdb_abi_version() == gdb.ABI_VERSION
    assert gdb.lib().gdb_status_string(-4) == b"GDB_ERR_TIMEOUT"


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes structures have the C structs' sizes and field offsets
    (compiled here with gcc against include/gdb.h)."""
    import shutil
    import subprocess

    from gpu_discovery_barrier_gb300 import gdb

    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    structs = {"gdb_options": gdb.Options, "gdb_run_stats": gdb.RunStats,
               "gdb_mst_result": gdb.MstResult, "gdb_device_info": gdb.DeviceInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gdb.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


@pytest.mark.parametrize("field,value", [("pull_bitmap_kb", 65), ("pull_bitmap_kb", -2),
                                         ("sssp_split", 2), ("xf_release", 5)])
def test_out_of_range_options_are_rejected_before_any_cuda_call(field, value):
    """gdb_ctx_create checks the options first: no device is touched."""
    from gpu_discovery_barrier_gb300 import gdb

    o = gdb.default_options(**{field: value})
    h = ctypes.c_void_p()
    assert gdb.lib().gdb_ctx_create(ctypes.byref(o), ctypes.byref(h)) == -1
    assert not h.value
