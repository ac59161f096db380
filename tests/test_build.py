"""Host-side build logic (no GPU): the library builds run in parallel threads
(build.build_all), so everything they share must tolerate that."""
import concurrent.futures as cf
import shutil

import pytest

from gpu_discovery_barrier_gb300 import build


@pytest.mark.skipif(shutil.which("gcc") is None or shutil.which("g++") is None,
                    reason="needs the host C and C++ compilers")
def test_openmp_probes_in_parallel():
    """Concurrent OpenMP probes each use a directory of their own: every one
    gives the same answer, and none leaves a file in the library folder."""
    before = set(build.LIBDIR.iterdir()) if build.LIBDIR.exists() else set()
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        got = list(ex.map(build._openmp_flag, ["gcc", "g++"] * 4))
    assert all(g == got[0] for g in got), got
    after = set(build.LIBDIR.iterdir()) if build.LIBDIR.exists() else set()
    assert after == before, sorted(str(p) for p in after - before)
