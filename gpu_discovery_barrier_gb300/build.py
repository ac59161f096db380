"""Native build of every library in the repository.

Compiles, in parallel and in-tree:

* ``lib/libgdb.so``      -- the CUDA C-ABI library (sm_103a kernels + host
  runtime), declared in ``include/gdb.h``;
* ``lib/libgdbgen.so``   -- the deterministic graph generators;
* ``oracle/_build/liboracle.so`` -- the CPU oracle (test infrastructure);
* ``oracle/_ref/libgdbref.so``   -- the reference's own OpenCL C kernels
  through the C++ shim, only when the reference checkout is present (the
  development container), never on the GPU host.

Host code is portable C/C++ (no architecture flags), so the same sources
build on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"
# the reference checkout: GDB_REFERENCE_DIR, else a "reference" directory
# beside the repository (where the development container keeps it); the
# GPU host has neither and skips that build
REF_CHECKOUT = Path(os.environ.get("GDB_REFERENCE_DIR") or ROOT.parent / "reference")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = [
    "gdb_runtime.cu",
    "gdb_discovery.cu",
    "gdb_bfs.cu",
    "gdb_sssp.cu",
    "gdb_arcsplit.cu",
    "gdb_mis_color.cu",
    "gdb_bc.cu",
    "gdb_mst.cu",
    "gdb_batch.cu",
    "gdb_mlp.cu",
    "gdb_server.cu",
    "gdb_io.cu",
    "gdb_dmr.cu",
]
# per-file flags: the mesh refinement's double arithmetic must round as the
# reference's does, operation for operation (no contraction into FMAs)
CUDA_EXTRA = {"gdb_dmr.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _run(cmd: list[str], cwd: Path | None = None) -> None:
    res = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _openmp_flag(cc: str) -> list[str]:
    """-fopenmp when the host compiler has libgomp, else nothing.  Each call
    probes in a directory of its own: build_all runs the library builds in
    parallel threads, and two probes sharing a file race on it."""
    with tempfile.TemporaryDirectory(prefix="gdb_omp_") as d:
        probe = Path(d) / "probe.c"
        probe.write_text("#include <omp.h>\nint main(void){return omp_get_max_threads()<1;}\n")
        res = subprocess.run([cc, "-fopenmp", str(probe), "-o", str(Path(d) / "probe.bin")],
                             stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return ["-fopenmp"] if res.returncode == 0 else []


def build_graphgen() -> Path:
    out = LIBDIR / "libgdbgen.so"
    src = CSRC / "graphgen.cpp"
    if _stale(out, [src]):
        LIBDIR.mkdir(parents=True, exist_ok=True)
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", *_openmp_flag("g++"),
              str(src), "-o", str(out)])
    return out


def build_oracle() -> Path:
    out = ORACLE / "_build" / "liboracle.so"
    srcs = [ORACLE / "oracle.c", ORACLE / "oracle_dmr.c", ORACLE / "oracle_gen.c",
            ORACLE / "oracle.h"]
    if _stale(out, srcs):
        out.parent.mkdir(parents=True, exist_ok=True)
        # no floating-point contraction: the same doubles on x86 and Arm hosts
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
              *_openmp_flag("gcc"), *(str(s) for s in srcs if s.suffix == ".c"),
              "-lm", "-o", str(out)])
    return out


def build_reference() -> Path | None:
    """The reference's kernels through the shim; None when no checkout."""
    if not (REF_CHECKOUT / "code" / "discovery_protocol").is_dir():
        return None
    _run(["make", "-s", "-j8", f"REF={REF_CHECKOUT}"], cwd=ORACLE / "refshim")
    return ORACLE / "_ref" / "libgdbref.so"


def build_cuda(jobs: int | None = None) -> Path:
    nvcc = _nvcc()
    out = LIBDIR / "libgdb.so"
    objdir = PKG / "_build"
    objdir.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")) \
        + list(INCLUDE.glob("*.cuh"))
    flags = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
             "-I", str(INCLUDE), "-I", str(CSRC), "--expt-relaxed-constexpr"]
    if os.environ.get("GDB_PTXAS_VERBOSE"):
        flags += ["-Xptxas", "-v"]

    def compile_one(name: str) -> Path:
        src = CSRC / name
        obj = objdir / (name + ".o")
        if _stale(obj, [src, *headers]):
            _run([nvcc, *flags, *CUDA_EXTRA.get(name, []), "-c", str(src), "-o", str(obj)])
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, CUDA_SOURCES))
    if _stale(out, objs):
        _run([nvcc, "-shared", ARCH, "-o", str(out), *map(str, objs), "-lcudart"])
    return out


def build_all(with_reference: bool = True) -> dict[str, Path | None]:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f_cuda = ex.submit(build_cuda)
        f_gen = ex.submit(build_graphgen)
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference) if with_reference else None
        res = {"libgdb": f_cuda.result(), "libgdbgen": f_gen.result(),
               "liboracle": f_orc.result()}
        res["libgdbref"] = f_ref.result() if f_ref else None
    return res


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    fn = {"all": build_all, "cuda": build_cuda, "gen": build_graphgen,
          "oracle": build_oracle, "ref": build_reference}[what]
    print(fn())
