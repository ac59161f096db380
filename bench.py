#!/usr/bin/env python
"""Benchmark: the plain persistent suite on an R-MAT scale-22 graph.

One step = the full suite over one seeded R-MAT graph (scale 22, edge factor
16, a,b,c = 0.57,0.19,0.19, symmetrised, deduplicated): BFS and worklist
SSSP (weights U[1,255]) from 16 seeded sources, MIS and greedy colouring
with seeded priorities, BC from the same 16 sources, Boruvka MST with
unique weights.  The metric is edges/s: the arcs out of reached vertices
for every BFS / SSSP / BC source plus all arcs for MIS, colouring and MST,
divided by the device time of the step.

* value: graphs resident in HBM, outputs in device buffers, CUDA events on
  the library's stream around K steps (inputs > L2, so no flush is needed);
* e2e: the same step through the host-buffer C-ABI calls a user makes
  (graph upload from pinned host memory and result read-back included);
* roofline: algorithmic bytes / measured launch time of the kernel with the
  largest time share, against MEASURED_PEAKS.json's HBM bandwidth;
* cpu_baseline: the CPU oracle on a bounded sample of the same workload.

``--impl reference`` times the CPU implementation of the path on the host's
cores instead: the oracle port, spread over all host threads, because the
reference's own apps need an OpenCL runtime that neither machine has (its
kernels compile through oracle/refshim only where its sources are, to pin
the oracle).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NSRC = 16


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gdb", "reference"], default="gdb")
    p.add_argument("--scale", type=int, default=22)
    p.add_argument("--edge-factor", type=float, default=16)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-parity", action="store_true",
                   help="skip the full-size output check against the CPU oracle")
    p.add_argument("--apps", default="bfs,sssp,mis,color,bc,mst")
    p.add_argument("--batch-graphs", type=int, default=512)
    p.add_argument("--schedule", choices=["plain", "adaptive", "learned"], default="learned",
                   help="BFS/SSSP schedule of the suite (learned = the trained selector)")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--pull-bitmap-kb", type=int, default=0,
                   help="BFS pull levels' frontier bitmap stage (gdb_options.pull_bitmap_kb: "
                        "0 automatic, -1 none, 1..64 KB)")
    p.add_argument("--requests", type=int, default=4000, help="serve: requests submitted")
    p.add_argument("--rate", type=float, default=2000.0, help="serve: Poisson arrival rate (req/s)")
    p.add_argument("--slots", type=int, default=64, help="serve: concurrent slots")
    p.add_argument("--graph", default=None,
                   help="rmat workload: run the suite on this .gr / DIMACS / METIS file instead "
                        "(undirected; its weights for SSSP when it has them)")
    p.add_argument("--workload", choices=["rmat", "grid4096", "batch", "serve", "relaunch", "barrier"],
                   default="rmat",
                   help="rmat: the R-MAT suite (default); grid4096: the barrier-bound "
                        "4096x4096 grid, BFS and SSSP from the corner per barrier kind")
    return p.parse_args()


# ---------------------------------------------------------------- workload


def make_workload(scale: int, ef: float, path: str | None = None):
    from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

    if path:
        g = gdb.read_graph(path, directed=False)
        # generated weights are one per undirected edge; a file's own
        # weights are taken as given (not declared symmetric)
        symmetric = g.w is None
        w = g.w if g.w is not None else gg.uniform_weights(g, 1, 255, seed=1)
        g = gg.CSR(g.row_ptr, g.col, None, g.name)
    else:
        g = gg.rmat_scale(scale, ef, seed=1)
        w = gg.uniform_weights(g, 1, 255, seed=1)
        symmetric = True  # undirected R-MAT, one weight per edge
    return {
        "g": g,
        "w": w,
        "symmetric": symmetric,
        "uw": gg.unique_weights(g, seed=3),
        "prio": gg.priorities(g.V, seed=4),
        "src": gg.sources(g, NSRC, seed=2),
    }


def make_workload_cpu(scale: int, ef: float):
    """The same seeded workload from the oracle's own generator (no library
    of the product is loaded by the CPU implementation's arm)."""
    import oracle as O

    g = O.gen_rmat(1 << scale, ef, seed=1)
    return {
        "g": g,
        "w": O.gen_uniform_weights(g, 1, 255, seed=1),
        "symmetric": True,
        "uw": O.gen_unique_weights(g, seed=3),
        "prio": O.gen_priorities(g.V, seed=4),
        "src": O.gen_sources(g, NSRC, seed=2),
    }


def reach(g, dist):
    """(reached vertices, arcs out of them) from a BFS level vector."""
    m = dist != 1_000_000_000
    deg = g.degrees()
    return int(m.sum()), int(deg[m].sum())


# -------------------------------------------------------------- roofline

def alg_bytes(app: str, g, reached, rounds: int) -> float:
    """Algorithmic bytes of one launch (uint32 = 4 B), schedule-independent:
    BFS 8E_r + 12V_r + 4V; SSSP 12E_r + 12V_r + 4V; BC 20E_r + 24V_r + 12V
    per source; MST (12E + 16V) per round; colouring 24E + 16V (one count
    pass and one countdown pass over the arcs); MIS (12E + 8V) per round,
    bounded from above by the full graph."""
    V, E = g.V, g.E
    if app == "bfs":
        return sum(8 * er + 12 * vr + 4 * V for vr, er in reached)
    if app == "sssp":
        return sum(12 * er + 12 * vr + 4 * V for vr, er in reached)
    if app == "bc":
        return sum(20 * er + 24 * vr + 12 * V for vr, er in reached)
    if app == "mst":
        return rounds * (12 * E + 16 * V)
    if app == "color":
        # count pass (col + neighbour priority per arc) and one countdown
        # pass (col, neighbour degree and priority, counter) per arc
        return 8 * E + 8 * V + 16 * E + 8 * V
    return rounds * (12 * E + 8 * V)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- clocks


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"gdb_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        busy = [x for x in sm if smax and x > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------- GPU suite


def set_schedule(ctx, name: str) -> None:
    """plain / adaptive / learned (loads the committed selector weights)."""
    from gpu_discovery_barrier_gb300 import gdb, selector

    if name == "learned":
        p = selector.load()
        if p is None:
            raise SystemExit("learned schedule: selector_weights.json missing")
        ctx.selector_set(p)
    ctx.set_options(schedule={"plain": gdb.SCHED_PLAIN, "adaptive": gdb.SCHED_ADAPTIVE,
                              "learned": gdb.SCHED_LEARNED}[name])


class GpuSuite:
    def __init__(self, wl, apps, device, schedule="plain", bitmap_kb=0):
        import torch

        from gpu_discovery_barrier_gb300 import gdb

        self.torch = torch
        self.gdb = gdb
        self.wl = wl
        self.apps = apps
        self.device = device
        g = wl["g"]
        self.ctx = gdb.Ctx(device=device, pull_bitmap_kb=bitmap_kb)
        set_schedule(self.ctx, schedule)
        self.G = self.ctx.graph(g.row_ptr, g.col, wl["w"], symmetric=wl["symmetric"])
        self.Gu = self.ctx.graph(g.row_ptr, g.col, wl["uw"])
        dev = torch.device("cuda", device)
        V = g.V
        self.d_dist = torch.empty(V, dtype=torch.int32, device=dev)
        self.d_dists = torch.empty((len(wl["src"]), V), dtype=torch.int32, device=dev)
        self.d_out = torch.empty(V, dtype=torch.int32, device=dev)
        self.d_bc = torch.empty(V, dtype=torch.float32, device=dev)
        self.d_prio = torch.from_numpy(wl["prio"]).to(dev)
        self.d_src = torch.from_numpy(wl["src"].astype(np.int32)).to(dev)
        self.d_mst = torch.zeros(4, dtype=torch.int64, device=dev)
        self.stream = torch.cuda.ExternalStream(self.ctx.stream(), device=dev)

    def step_device(self, record: dict):
        """One suite pass on resident inputs; per-app kernel time and launches."""
        c, src = self.ctx, self.wl["src"]

        def note(app):
            st = c.last_stats()
            r = record.setdefault(app, {"ms": 0.0, "launches": 0, "calls": 0, "supersteps": 0})
            r["ms"] += st["kernel_ms"]
            r["launches"] += st["launches"]
            r["calls"] += 1
            r["supersteps"] += st["supersteps"]

        # the 16 sources' independent runs, spread over concurrent lanes
        if "bfs" in self.apps:
            c.bfs_sources_device(self.G, self.d_src.data_ptr(), len(src), self.d_dists.data_ptr())
            note("bfs")
        if "sssp" in self.apps:
            c.sssp_sources_device(self.G, self.d_src.data_ptr(), len(src), self.d_dists.data_ptr())
            note("sssp")
        if "mis" in self.apps:
            c.mis_device(self.G, self.d_prio.data_ptr(), self.d_out.data_ptr())
            note("mis")
        if "color" in self.apps:
            c.color_device(self.G, self.d_prio.data_ptr(), self.d_out.data_ptr())
            note("color")
        if "bc" in self.apps:
            c.bc_device(self.G, self.d_src.data_ptr(), len(src), self.d_bc.data_ptr())
            note("bc")
        if "mst" in self.apps:
            c.mst_device(self.Gu, self.d_mst.data_ptr(), None)
            note("mst")

    def e2e_buffers(self):
        """Page-locked host arrays (inputs and results) and two sets of
        device buffers the end-to-end steps copy them to and from (one
        step's inputs land in one set while the other set's step runs);
        allocated once, reused every step, as a serving loop would."""
        torch, wl = self.torch, self.wl
        g = wl["g"]
        dev = torch.device("cuda", self.device)
        ins = {"row": g.row_ptr, "col": g.col, "w": wl["w"], "uw": wl["uw"], "prio": wl["prio"],
               "src": wl["src"].astype(np.uint32)}
        outs = {"bfs": np.zeros((NSRC, g.V), np.uint32), "sssp": np.zeros((NSRC, g.V), np.uint32),
                "mis": np.zeros(g.V, np.int32), "color": np.zeros(g.V, np.int32),
                "bc": np.zeros(g.V, np.float32)}
        h, d, d2 = {}, {}, {}
        for k, a in {**ins, **outs}.items():
            h[k] = pinned_tensor(torch, a)
            d[k] = torch.empty_like(h[k], device=dev)
            d2[k] = torch.empty_like(h[k], device=dev) if k in ins else d[k]
        h["mst"] = torch.zeros(4, dtype=torch.int64, pin_memory=True)
        d["mst"] = d2["mst"] = torch.zeros(4, dtype=torch.int64, device=dev)
        return h, (d, d2)

    def upload(self, h, d, cs):
        """Issue one step's input copies (page-locked host -> device) on the
        copy stream `cs`; returns the events the apps wait for: row, column
        and sources first, then the weights, the priorities, the MST
        weights."""
        torch = self.torch
        ev = {k: torch.cuda.Event() for k in ("rc", "w", "p", "uw")}
        with torch.cuda.stream(cs):
            for k in ("row", "col", "src"):
                d[k].copy_(h[k], non_blocking=True)
            ev["rc"].record(cs)
            d["w"].copy_(h["w"], non_blocking=True)
            ev["w"].record(cs)
            d["prio"].copy_(h["prio"], non_blocking=True)
            ev["p"].record(cs)
            d["uw"].copy_(h["uw"], non_blocking=True)
            ev["uw"].record(cs)
        return ev

    def step_e2e(self, h, d, cs, ev=None, d_next=None, us=None, h_next=None):
        """The suite from page-locked host inputs to page-locked host
        results through the library's device-pointer entry points.  The
        step's inputs are on their way (`ev`, from upload(); issued here on
        `cs` when None); every app's result comes back on the copy stream
        `cs` while the next app runs.  With `d_next` (the other buffer set),
        the next step's inputs (`h_next`, default `h`) go up on the upload
        stream `us` under this step's kernels, in the other direction of the
        link.  Returns (bytes read back, the next step's upload events or
        None)."""
        torch, gdb = self.torch, self.gdb
        c, g = self.ctx, self.wl["g"]
        if ev is None:
            ev = self.upload(h, d, cs)
        ev_next = self.upload(h if h_next is None else h_next, d_next, us) if d_next is not None else None
        outs = 0

        def back(k):
            nonlocal outs
            with torch.cuda.stream(cs):
                h[k].copy_(d[k], non_blocking=True)
            outs += h[k].numel() * h[k].element_size()

        ev["rc"].synchronize()
        V, E = g.V, g.E
        G = gdb.Graph(c, (d["row"].data_ptr(), V + 1), (d["col"].data_ptr(), E),
                      (d["w"].data_ptr(), E), device=True, symmetric=self.wl["symmetric"])
        src = d["src"].data_ptr()
        if "bfs" in self.apps:
            c.bfs_sources_device(G, src, NSRC, d["bfs"].data_ptr())
            back("bfs")
        ev["w"].synchronize()
        if "sssp" in self.apps:
            c.sssp_sources_device(G, src, NSRC, d["sssp"].data_ptr())
            back("sssp")
        ev["p"].synchronize()
        if "mis" in self.apps:
            c.mis_device(G, d["prio"].data_ptr(), d["mis"].data_ptr())
            back("mis")
        if "color" in self.apps:
            c.color_device(G, d["prio"].data_ptr(), d["color"].data_ptr())
            back("color")
        if "bc" in self.apps:
            c.bc_device(G, src, NSRC, d["bc"].data_ptr())
            back("bc")
        Gu = None
        if "mst" in self.apps:
            ev["uw"].synchronize()
            Gu = gdb.Graph(c, (d["row"].data_ptr(), V + 1), (d["col"].data_ptr(), E),
                           (d["uw"].data_ptr(), E), device=True)
            c.mst_device(Gu, d["mst"].data_ptr(), None)
            torch.cuda.current_stream().synchronize()
            back("mst")
        cs.synchronize()
        G.close()
        if Gu is not None:
            Gu.close()
        return outs, ev_next


def pinned_tensor(torch, a: np.ndarray):
    """A page-locked host tensor holding a copy of `a` (32-bit integers as
    int32, floats as float32)."""
    t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                    pin_memory=True)
    t.numpy().view(a.dtype)[...] = a
    return t


_PINNED_KEEP: list = []


def pinned_copy(torch, a: np.ndarray) -> np.ndarray:
    """Copy into page-locked host memory (kept alive for the process)."""
    t = torch.empty(a.shape, dtype={np.dtype(np.uint32): torch.int32, np.dtype(np.int32): torch.int32,
                                    np.dtype(np.float32): torch.float32}[a.dtype], pin_memory=True)
    _PINNED_KEEP.append(t)
    out = t.numpy().view(a.dtype)
    out[...] = a
    return out


# ----------------------------------------------------------- CPU sample


def cpu_sample(wl, threads: int, full: bool):
    """Bounded sample of the suite on the CPU oracle.  `full`: every app,
    all 16 sources, spread over `threads` host threads (ctypes releases the
    GIL); otherwise one source of BFS/SSSP/BC plus MIS on one thread."""
    import oracle as O

    g, src = wl["g"], wl["src"]
    gw = g.with_weights(wl["w"])
    gu = g.with_weights(wl["uw"])
    srcs = [int(s) for s in src] if full else [int(src[0])]
    tasks = []
    for s in srcs:
        tasks.append(("bfs", lambda s=s: O.bfs(g, s)))
        tasks.append(("sssp", lambda s=s: O.sssp_worklist(gw, s)))
        tasks.append(("bc", lambda s=s: O.bc_f64(g, [s])))
    tasks.append(("mis", lambda: O.mis(g, wl["prio"])))
    if full:
        tasks.append(("color", lambda: O.color_fast(g, wl["prio"])))
        tasks.append(("mst", lambda: O.mst(gu)))
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda t: t[1](), tasks))
    return time.perf_counter() - t0, [t[0] for t in tasks], srcs


def units_of(names, srcs, er_by_src, E):
    u = 0
    per = {"bfs": [], "sssp": [], "bc": []}
    for n in names:
        if n in per:
            per[n].append(1)
    for n in ("bfs", "sssp", "bc"):
        u += sum(er_by_src[s] for s in srcs) if per[n] else 0
    u += E * sum(1 for n in names if n in ("mis", "color", "mst"))
    return u


# ------------------------------------------------------------------ main


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("GDB_BENCH_BACKEND") != "gloo" else "gloo")
    return rank, world, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def my_members(n: int, rank: int, world: int, seed: int):
    """This rank's members of the n-graph mixed batch: all of them on one
    GPU; on several, a placement of whole graphs balanced by arcs."""
    if world == 1:
        return None
    from gpu_discovery_barrier_gb300 import graphgen as gg, placement

    spec = gg.mixed_batch_spec(n, 1000, 1_000_000, seed=seed)
    return placement.place([m["arcs"] for m in spec], world)[rank]


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def suite_metric(schedule: str) -> str:
    return (f"edges/sec (persistent suite, {schedule} BFS/SSSP schedule: BFS+SSSP+BC x16 sources, "
            "MIS, colour, MST)")


def suite_config(args, g, world) -> dict:
    """The workload as both arms report it (identical dicts)."""
    return {"workload": (f"file {args.graph} suite" if args.graph
                         else f"rmat scale {args.scale} ef {args.edge_factor:g} suite"),
            "V": g.V, "E": g.E, "sources": NSRC, "apps": args.apps.split(","),
            "schedule": args.schedule, "global_batch": world,
            "parallelism": f"replicas x{world}", "l2": "inputs > L2 (no flush)"}


def base_line(args, world, metric_value, ms_per_step, cfg):
    return {
        "metric": suite_metric(args.schedule),
        "value": metric_value,
        "unit": "edges/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (seeded R-MAT generator; the reference's datasets are external)",
        "config": cfg,
    }


def mst_edges(g, arc_flags) -> np.ndarray:
    """Sorted unique undirected edges (min << 32 | max) of the flagged arcs."""
    sel = np.nonzero(np.asarray(arc_flags)[: g.E])[0]
    src = np.searchsorted(g.row_ptr.astype(np.int64), sel, side="right") - 1
    a, b = src.astype(np.uint64), g.col[sel].astype(np.uint64)
    return np.unique((np.minimum(a, b) << np.uint64(32)) | np.maximum(a, b))


def suite_parity(suite, wl, threads: int) -> dict:
    """Every app of the suite on the full workload, read back through the
    host-buffer API, against the CPU oracle (spread over `threads` host
    threads): BFS levels and SSSP distances for the 16 sources, the MIS set,
    the colours and the MST weight, edge count, components and edge set bit
    for bit; BC within 1e-4 relative of the FP64 Brandes oracle (the same
    tolerance as the tests), non-finite where the oracle is."""
    import oracle as O

    c, g, src = suite.ctx, wl["g"], [int(x) for x in wl["src"]]
    gw, gu = g.with_weights(wl["w"]), g.with_weights(wl["uw"])
    apps = suite.apps
    got = {}
    if "bfs" in apps:
        got["bfs"] = c.bfs_sources(suite.G, src)
    if "sssp" in apps:
        got["sssp"] = c.sssp_sources(suite.G, src)
    if "mis" in apps:
        got["mis"] = c.mis(suite.G, wl["prio"])
    if "color" in apps:
        got["color"] = c.color(suite.G, wl["prio"])
    if "bc" in apps:
        got["bc"] = c.bc(suite.G, src)
    if "mst" in apps:
        got["mst"] = c.mst(suite.Gu, with_arcs=True)
    t0 = time.perf_counter()
    tasks = {}
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for i, s in enumerate(src):
            if "bfs" in apps:
                tasks[("bfs", i)] = ex.submit(O.bfs, g, s)
            if "sssp" in apps:
                tasks[("sssp", i)] = ex.submit(O.sssp_worklist, gw, s)
            if "bc" in apps:
                tasks[("bc", i)] = ex.submit(O.bc_f64, g, [s])
        if "mis" in apps:
            tasks[("mis", 0)] = ex.submit(lambda: O.mis(g, wl["prio"])[0])
        if "color" in apps:
            tasks[("color", 0)] = ex.submit(lambda: O.color_fast(g, wl["prio"])[0])
        if "mst" in apps:
            tasks[("mst", 0)] = ex.submit(O.mst, gu)
        want = {k: f.result() for k, f in tasks.items()}
    res: dict = {}
    for app in ("bfs", "sssp"):
        if app in got:
            res[app] = all(np.array_equal(got[app][i], want[(app, i)]) for i in range(len(src)))
    for app in ("mis", "color"):
        if app in got:
            res[app] = bool(np.array_equal(got[app], want[(app, 0)]))
    detail = {}
    if "bc" in got:
        ref = np.sum([want[("bc", i)] for i in range(len(src))], axis=0)
        fin = np.isfinite(ref)
        b = got["bc"].astype(np.float64)
        scale = np.maximum(np.abs(ref[fin]), 1e-6 * max(1.0, float(np.abs(ref[fin]).max())))
        err = np.abs(b[fin] - ref[fin]) / scale
        res["bc"] = bool(np.all(np.abs(b[fin] - ref[fin]) <= 1e-4 * scale + 1e-6)
                         and not np.any(np.isfinite(b[~fin])))
        detail["bc_max_rel_err"] = float(err.max()) if err.size else 0.0
    if "mst" in got:
        m, r = got["mst"], want[("mst", 0)]
        res["mst"] = bool((m["weight64"], m["weight32"], m["edges"], m["components"])
                          == (r["weight64"], r["weight32"], r["edges"], r["components"])
                          and np.array_equal(mst_edges(g, m["arc_in_mst"]),
                                             mst_edges(g, r["arc_in_mst"])))
    detail["oracle_s"] = round(time.perf_counter() - t0, 1)
    detail["oracle_threads"] = threads
    res["detail"] = detail
    return res


def run_reference(args, rank, world):
    import oracle as O

    if rank != 0:
        return
    if args.graph:
        print(json.dumps({"impl": "reference", "unavailable": "the CPU implementation's arm runs "
                          "the generated R-MAT workload only (no graph-file reader on that side)"}))
        return
    wl = make_workload_cpu(args.scale, args.edge_factor)
    g = wl["g"]
    er = {int(s): reach(g, O.par_bfs(g, int(s)))[1] for s in wl["src"]}
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(wl, threads, full=False)
    times, units = [], 0
    for _ in range(args.steps):
        dt, names, srcs = cpu_sample(wl, threads, full=True)
        times.append(dt)
        units += units_of(names, srcs, er, g.E)
    total = sum(times)
    value = units / total
    line = base_line(args, 1, value, 1e3 * total / args.steps, suite_config(args, g, 1))
    line["impl"] = "reference"
    line["cpu_baseline"] = {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                            "sample": "full suite per step (16 sources of BFS/SSSP/BC, MIS, "
                                      "colour, MST) on the CPU oracle over all host threads; "
                                      "warm-up steps use the one-source sample"}
    line["e2e"] = {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)


def run_gdb(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    apps = args.apps.split(",")
    wl = make_workload(args.scale, args.edge_factor, args.graph)
    g = wl["g"]
    suite = GpuSuite(wl, apps, local, args.schedule, args.pull_bitmap_kb)
    er_by_src, reached, one_ms = {}, [], []
    for s in wl["src"]:
        vr, erv = reach(g, suite.ctx.bfs(suite.G, int(s)))
        one_ms.append(suite.ctx.last_stats()["kernel_ms"])  # one traversal alone on the GPU
        er_by_src[int(s)] = erv
        reached.append((vr, erv))
    sum_er = sum(er_by_src.values())
    units_per_step = 0
    for a in apps:
        units_per_step += sum_er if a in ("bfs", "sssp", "bc") else g.E

    for _ in range(args.warmup):
        suite.step_device({})
    rec: dict = {}
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(suite.stream):
            start.record(suite.stream)
            for _ in range(args.steps):
                suite.step_device(rec)
            end.record(suite.stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = start.elapsed_time(end)
    ms = reduce_max(ms, world)
    value = world * units_per_step * args.steps / (ms / 1e3)
    clocks = clk.summary()

    # the whole suite under the plain schedule, timed the same way, for
    # comparison (only BFS and SSSP depend on the schedule)
    plain = None
    if args.schedule != "plain" and any(a in apps for a in ("bfs", "sssp")):
        set_schedule(suite.ctx, "plain")
        suite.step_device({})
        prec: dict = {}
        torch.cuda.synchronize()
        with torch.cuda.stream(suite.stream):
            start.record(suite.stream)
            for _ in range(args.steps):
                suite.step_device(prec)
            end.record(suite.stream)
        torch.cuda.synchronize()
        pms = reduce_max(start.elapsed_time(end), world)
        plain = {"value": world * units_per_step * args.steps / (pms / 1e3),
                 "ms_per_step": pms / args.steps,
                 "per_app_ms": {a: prec[a]["ms"] / args.steps for a in prec}}
        set_schedule(suite.ctx, args.schedule)

    # roofline of every kernel, reported for the one with the largest time share
    peak, peak_kind = peaks()

    def app_roofline(app):
        # per call: BFS and SSSP take the 16 sources in one call (their
        # launches overlap on concurrent lanes), BC too
        r = rec[app]
        launch_ms = r["ms"] / r["calls"]
        rounds = max(1, r["supersteps"] // max(1, r["calls"]))
        if app in ("bfs", "sssp", "bc"):
            nbytes = alg_bytes(app, g, reached, 0)
        else:
            nbytes = alg_bytes(app, g, [], rounds)
        return nbytes, launch_ms, nbytes / (launch_ms / 1e3) / 1e9

    per_app_roof = {a: round(app_roofline(a)[2] / peak, 4) for a in rec}
    dom = max(rec, key=lambda a: rec[a]["ms"])
    nbytes, launch_ms, achieved = app_roofline(dom)
    # measured DRAM traffic per call (ncu, profiles/traffic.json) where it
    # was captured: the HBM fraction those bytes give at the measured time
    measured = {}
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists() and not args.graph and args.scale == 22 and args.edge_factor == 16:  # the captured workload
        tj = json.loads(tf.read_text())
        for a in rec:
            if isinstance(tj.get(a), (int, float)):
                # captured per single-source launch; a BFS / SSSP call runs NSRC of them
                measured[a] = tj[a] * (NSRC if a in ("bfs", "sssp") else 1)
    traffic = measured.get(dom)
    per_app_traffic_frac = {a: round(measured[a] / (app_roofline(a)[1] / 1e3) / 1e9 / peak, 4)
                            for a in measured}
    roof = {"bound": "hbm", "kernel": f"k_{dom}_xf", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "alg_bytes_per_launch": nbytes, "launch_ms": launch_ms, "traffic": traffic,
            "launch": ("one call: the 16 sources' launches on concurrent lanes"
                       if dom in ("bfs", "sssp") else "one launch")}

    # end to end: host inputs to host results every step (copies overlapped
    # with the kernels of earlier apps, see GpuSuite.step_e2e)
    e2e = None
    if not args.no_e2e:
        h, dbufs = suite.e2e_buffers()
        h2d = sum(h[k].numel() * h[k].element_size() for k in ("row", "col", "w", "uw", "prio", "src"))
        cs, us = torch.cuda.Stream(), torch.cuda.Stream()
        suite.step_e2e(h, dbufs[0], cs)
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d2h, ev = 0, None
        # exactly one upload and one read-back per timed step: step 1 sends
        # its own inputs, each step sends the next one's under its kernels,
        # the last step sends none
        for k in range(args.steps):
            d2h, ev = suite.step_e2e(h, dbufs[k % 2], cs, ev,
                                     dbufs[(k + 1) % 2] if k + 1 < args.steps else None, us)
        torch.cuda.synchronize()
        dt = reduce_max(time.perf_counter() - t0, world)
        e2e = {"value": world * units_per_step * args.steps / dt, "unit": "edges/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "path": "device-pointer entry points; each step's inputs up on a copy stream "
                       "under the previous step's kernels (the first step's at its start), each "
                       "app's result down while the next app runs"}
        # the last step's results, read back through the host copies, equal
        # the device-resident run's (a check of the end-to-end path)
        # (the device-resident step leaves SSSP's distances and the colours
        # in its buffers)
        e2e["results_match_device_run"] = bool(
            ("sssp" not in apps or np.array_equal(h["sssp"].numpy(), suite.d_dists.cpu().numpy()))
            and ("color" not in apps or np.array_equal(h["color"].numpy(), suite.d_out.cpu().numpy())))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        dt, names, srcs = cpu_sample(wl, 1, full=False)
        cpu = {"value": units_of(names, srcs, er_by_src, g.E) / dt, "unit": "edges/s", "cores": 1,
               "kind": "port", "sample": "BFS, worklist SSSP and BC from one source plus MIS on the "
                                         f"same graph, serial CPU oracle ({dt:.1f} s)"}

    # full-size parity of every app's output against the CPU oracle
    parity = None
    if not args.no_parity:
        parity = suite_parity(suite, wl, os.cpu_count() or 1)

    if rank == 0:
        line = base_line(args, world, value, ms / args.steps, suite_config(args, g, world))
        line["setup"] = {"block": suite.ctx.opt.block_size, "barrier": "xf",
                         "lock": "lock-free poll", "schedule": args.schedule}
        line["clocks"] = clocks
        line["e2e"] = e2e
        line["roofline"] = roof
        line["per_app_hbm_frac"] = per_app_roof
        line["per_app_hbm_frac_measured_traffic"] = per_app_traffic_frac
        line["cpu_baseline"] = cpu
        line["gpu_launches"] = sum(r["launches"] for r in rec.values())
        line["per_app_ms"] = {a: rec[a]["ms"] / args.steps for a in rec}
        line["schedule"] = args.schedule
        line["plain_schedule"] = plain
        line["per_app_supersteps"] = {a: rec[a]["supersteps"] // args.steps for a in rec}
        # the reach runs: one source per call, the traversal alone on the GPU
        line["bfs_one_source_ms"] = {"median": float(np.median(one_ms)), "min": float(np.min(one_ms)),
                                     "pull_bitmap_kb": args.pull_bitmap_kb}
        line["parity"] = parity
        print(json.dumps(line), flush=True)
        if parity is not None and not all(v is True for k, v in parity.items() if k != "detail"):
            print(f"PARITY FAILURE: {parity}", file=sys.stderr, flush=True)
            sys.exit(3)


def run_grid(args, rank, world, local):
    """Barrier-bound case: 4096x4096 grid (V = 16,777,216, 67,092,480 arcs,
    weights U[1,1000]), BFS and SSSP from the corner, thousands of
    supersteps; the same traversals on every barrier kind, plus the barrier
    latency of each kind at the CTA count the traversal kernels use."""
    import torch

    from gpu_discovery_barrier_gb300 import gdb, graphgen as gg

    torch.cuda.set_device(local)
    g = gg.grid(4096, 4096)
    w = gg.uniform_weights(g, 1, 1000, seed=1)
    dev = torch.device("cuda", local)
    d_out = torch.empty(g.V, dtype=torch.int32, device=dev)
    kinds = {"xf": (gdb.BARRIER_XF, gdb.SCHED_PLAIN),
             "xf_adaptive": (gdb.BARRIER_XF, gdb.SCHED_ADAPTIVE),
             "xf_learned": (gdb.BARRIER_XF, gdb.SCHED_LEARNED),
             "grid_sync": (gdb.BARRIER_GRID_SYNC, gdb.SCHED_PLAIN),
             "relaunch": (gdb.BARRIER_RELAUNCH, gdb.SCHED_PLAIN),
             "relaunch_graph": (gdb.BARRIER_RELAUNCH_GRAPH, gdb.SCHED_PLAIN)}
    res = {}
    from gpu_discovery_barrier_gb300 import selector

    with gdb.Ctx() as c:
        p = selector.load()
        if p is not None:
            c.selector_set(p)
        else:
            kinds.pop("xf_learned")
        G = c.graph(g.row_ptr, g.col, w, symmetric=True)  # grid, one weight per edge
        for name, (kind, sched) in kinds.items():
            c.set_options(barrier=kind, schedule=sched)
            r = {}
            for app in ("bfs", "sssp"):
                if app == "sssp" and kind == gdb.BARRIER_RELAUNCH:
                    continue
                fn = c.bfs_device if app == "bfs" else c.sssp_device
                for _ in range(args.warmup):
                    fn(G, 0, d_out.data_ptr())
                ms, steps = [], 0
                for _ in range(args.steps):
                    fn(G, 0, d_out.data_ptr())
                    st = c.last_stats()
                    ms.append(st["kernel_ms"])
                    steps = st["supersteps"]
                t = statistics.median(ms)
                r[app] = {"ms": t, "supersteps": steps, "edges_per_s": g.E / (t / 1e3),
                          "us_per_superstep": 1e3 * t / max(steps, 1),
                          "arcs_inspected": st["edges_processed"]}
                if app == "sssp":
                    r[app]["delta"] = st["sssp_delta"]
                    r[app]["phases"] = st["phases"]
            ns, groups = c.barrier_bench(kind, 512, 2000)
            r["barrier_ns"] = ns
            r["barrier_ctas"] = groups
            res[name] = r
        c.set_options(barrier=gdb.BARRIER_XF, schedule=gdb.SCHED_PLAIN)
    # the headline: the XF barrier under its fastest schedule on this graph
    # (plain, adaptive or learned, named in config); every barrier kind and
    # schedule is in the line
    xf_names = [k for k in ("xf", "xf_adaptive", "xf_learned") if k in res]
    head = min(xf_names, key=lambda k: res[k]["bfs"]["ms"] + res[k]["sssp"]["ms"])
    xf = res[head]
    value = 2 * g.E / ((xf["bfs"]["ms"] + xf["sssp"]["ms"]) / 1e3)
    cfg = {"workload": "grid 4096x4096, BFS + SSSP from vertex 0", "V": g.V, "E": g.E,
           "weights": "U[1,1000] seed 1", "global_batch": 1, "parallelism": "replicas x1",
           "l2": "inputs > L2 (no flush)", "schedule": head}
    line = base_line(args, world, value, xf["bfs"]["ms"] + xf["sssp"]["ms"], cfg)
    line["metric"] = "edges/sec (BFS + SSSP on the 4096x4096 grid, XF barrier)"
    line["plain_value"] = 2 * g.E / ((res["xf"]["bfs"]["ms"] + res["xf"]["sssp"]["ms"]) / 1e3)
    line["barrier_kinds"] = res
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_relaunch(args, rank, world, local):
    """Persistent against relaunched supersteps, per app, on the R-MAT
    suite graph: each app under the XF barrier (one persistent launch),
    under GDB_BARRIER_RELAUNCH (one launch per superstep with the stop flag
    read back, the reference's multi-kernel pattern) and under
    GDB_BARRIER_RELAUNCH_GRAPH (the same launches from a CUDA-graph WHILE
    node).  Outputs of the three forms are compared bit for bit (BC within
    1e-4)."""
    import torch

    from gpu_discovery_barrier_gb300 import gdb

    torch.cuda.set_device(local)
    wl = make_workload(args.scale, args.edge_factor, args.graph)
    g, src = wl["g"], [int(x) for x in wl["src"]]
    kinds = {"xf": gdb.BARRIER_XF, "relaunch": gdb.BARRIER_RELAUNCH,
             "relaunch_graph": gdb.BARRIER_RELAUNCH_GRAPH}
    apps = {
        "bfs": lambda c, G, Gu: c.bfs(G, src[0]),
        "sssp": lambda c, G, Gu: c.sssp(G, src[0]),
        "sssp_jacobi": lambda c, G, Gu: c.sssp_jacobi(G, src[0]),
        "mis": lambda c, G, Gu: c.mis(G, wl["prio"]),
        "color": lambda c, G, Gu: c.color(G, wl["prio"]),
        "bc": lambda c, G, Gu: c.bc(G, src),
    }
    res, outs = {}, {}
    for kname, kind in kinds.items():
        with gdb.Ctx(barrier=kind) as c:
            G = c.graph(g.row_ptr, g.col, wl["w"], symmetric=wl["symmetric"])
            for app, fn in apps.items():
                for _ in range(args.warmup):
                    out = fn(c, G, None)
                ms, st = [], None
                for _ in range(args.steps):
                    out = fn(c, G, None)
                    st = c.last_stats()
                    ms.append(st["kernel_ms"])
                t = statistics.median(ms)
                res.setdefault(app, {})[kname] = {"ms": t, "launches": st["launches"],
                                                  "supersteps": st["supersteps"]}
                outs.setdefault(app, {})[kname] = out
    same = {}
    for app, o in outs.items():
        a = o["xf"]
        if app == "bc":
            fin = np.isfinite(a)
            scale = np.maximum(np.abs(a[fin]), 1e-6 * max(1.0, float(np.abs(a[fin]).max())))
            same[app] = all(bool(np.all(np.abs(o[k][fin].astype(np.float64) - a[fin]) <= 1e-4 * scale
                                        + 1e-6)) for k in o)
        else:
            same[app] = all(np.array_equal(o[k], a) for k in o)
    for app, r in res.items():
        r["relaunch_over_xf"] = r["relaunch"]["ms"] / r["xf"]["ms"]
        r["graph_over_xf"] = r["relaunch_graph"]["ms"] / r["xf"]["ms"]
    total = {k: sum(res[a][k]["ms"] for a in res) for k in kinds}
    # work units as in the suite: arcs out of the reached vertices for the
    # traversals (BC: its 16 sources), every arc for Jacobi, MIS, colour
    with gdb.Ctx() as c:
        G = c.graph(g.row_ptr, g.col)
        er = [reach(g, c.bfs(G, s))[1] for s in src]
    units = 2 * er[0] + sum(er) + 3 * g.E
    value = units / (total["xf"] / 1e3)
    if rank == 0:
        cfg = suite_config(args, g, world)
        cfg["workload"] += " (persistent vs relaunched supersteps, per app)"
        line = base_line(args, world, value, total["xf"], cfg)
        line["metric"] = "edges/sec (per-app persistent XF vs relaunch vs graph relaunch)"
        line["per_app"] = res
        line["total_ms"] = total
        line["identical_across_forms"] = same
        line["gpu_launches"] = sum(res[a]["xf"]["launches"] for a in res)
        print(json.dumps(line), flush=True)


def run_barrier(args, rank, world, local):
    """The barrier alone: nanoseconds per barrier of every kind at 1, 2, 3
    and 4 CTAs of 512 threads per SM (gdb_barrier_bench: empty supersteps;
    the persistent kinds run 20,000 barriers in one launch, the relaunch
    kinds one launch per superstep), the median of `steps` runs after
    `warmup` unrecorded ones.  The headline is the XF barrier at 4 CTAs per
    SM, the reference's full co-residency."""
    import torch

    from gpu_discovery_barrier_gb300 import gdb

    torch.cuda.set_device(local)
    kinds = {"xf": gdb.BARRIER_XF, "xf_fixed": gdb.BARRIER_XF_FIXED,
             "grid_sync": gdb.BARRIER_GRID_SYNC, "relaunch": gdb.BARRIER_RELAUNCH,
             "relaunch_graph": gdb.BARRIER_RELAUNCH_GRAPH}
    res = {}
    with gdb.Ctx() as c:
        sms = c.device_info()["sm_count"]
        for per in (1, 2, 3, 4):
            c.set_options(max_ctas=per * sms)
            row = {}
            for name, kind in kinds.items():
                iters = 2000 if name.startswith("relaunch") else 20000
                for _ in range(args.warmup):
                    c.barrier_bench(kind, 512, iters)
                runs = [c.barrier_bench(kind, 512, iters) for _ in range(args.steps)]
                row[name] = {"ns": statistics.median(r[0] for r in runs), "ctas": runs[0][1]}
            row["xf_over_grid_sync"] = row["xf"]["ns"] / row["grid_sync"]["ns"]
            res[str(per * sms)] = row
    if rank == 0:
        full = res[str(4 * sms)]
        line = {
            "metric": "ns per barrier (XF barrier, 4 CTAs of 512 threads per SM)",
            "value": full["xf"]["ns"], "unit": "ns", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": full["xf"]["ns"] * 20000 / 1e6,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "none (empty supersteps)",
            "config": {"workload": "barrier alone, 1-4 CTAs of 512 threads per SM", "block": 512,
                       "sms": sms, "parallelism": f"replicas x{world}",
                       "l2": "no data (barrier words only)"},
            "per_ctas": res,
            "gpu_launches": args.steps,
        }
        print(json.dumps(line), flush=True)


def run_batch(args, rank, world, local):
    """Mixed batch: n graphs (V log-uniform in [1e3, 1e6], half R-MAT with
    edge factor 8..32, half grids with aspect ratio log-uniform in [1, 64]),
    one BFS and one SSSP from a seeded source each.  The batched form (one
    union graph, two persistent launches replayed from a captured CUDA
    graph, autotuned shape and thresholds) against the plain path run graph
    by graph (2n persistent launches); results compared bit-exact."""
    import torch

    from gpu_discovery_barrier_gb300 import autotune, gdb, graphgen as gg

    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    # the same batch on every rank count: whole graphs placed over the GPUs
    mine = my_members(args.batch_graphs, rank, world, seed=1)
    members = gg.mixed_batch(args.batch_graphs, 1000, 1_000_000, seed=1, members=mine)
    gen_s = time.perf_counter() - t0
    srcs = [m.meta["source"] for m in members]
    V = sum(m.V for m in members)
    E = sum(m.E for m in members)
    with gdb.Ctx() as c:
        stream = torch.cuda.ExternalStream(c.stream())
        dev = torch.device("cuda", local)
        # ---- plain path, graph by graph (device-resident, one pass)
        Gs = [c.graph(m.row_ptr, m.col, m.w) for m in members]
        d_b = torch.empty(max(m.V for m in members), dtype=torch.int32, device=dev)
        d_s = torch.empty_like(d_b)
        plain_out = []
        for i in range(min(4, len(members))):                  # warm-up
            c.bfs_device(Gs[i], srcs[i], d_b.data_ptr())
            c.sssp_device(Gs[i], srcs[i], d_s.data_ptr())
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        plain_kernel_ms = 0.0
        ev0.record(stream)
        for i, m in enumerate(members):
            c.bfs_device(Gs[i], srcs[i], d_b.data_ptr())
            plain_kernel_ms += c.last_stats()["kernel_ms"]
            c.sssp_device(Gs[i], srcs[i], d_s.data_ptr())
            plain_kernel_ms += c.last_stats()["kernel_ms"]
        ev1.record(stream)
        torch.cuda.synchronize()
        plain_ms = ev0.elapsed_time(ev1)
        # plain results for the comparison (untimed)
        for i, m in enumerate(members):
            plain_out.append((c.bfs(Gs[i], srcs[i]), c.sssp(Gs[i], srcs[i])))
        del Gs
        # ---- batched form
        U = c.graph_batch(members)
        off = U.vertex_offset
        usrc = [int(off[i]) + s for i, s in enumerate(srcs)]
        tune = None
        from gpu_discovery_barrier_gb300 import selector
        sel = selector.load()
        if sel is not None:
            c.selector_set(sel)
        if not args.no_tune:
            tune = autotune.tune_batch(c, U, usrc, apps=3, reps=2)
        with c.batch(U, usrc) as B:
            for _ in range(args.warmup):
                B.run()
            barrier(world)
            torch.cuda.synchronize()
            with ClockSampler(local) as clk:
                ev0.record(stream)
                for _ in range(args.steps):
                    B.launch()
                    B.wait()
                ev1.record(stream)
                torch.cuda.synchronize()
            ms = reduce_max(ev0.elapsed_time(ev1), world)
            clocks = clk.summary()
            res = B.results()
            arcs_bfs, steps_bfs = B.app_stats(gdb.BATCH_BFS)
            arcs_sssp, steps_sssp = B.app_stats(gdb.BATCH_SSSP)
            identical = all(
                np.array_equal(res["bfs"][off[i]:off[i + 1]], plain_out[i][0])
                and np.array_equal(res["sssp"][off[i]:off[i + 1]], plain_out[i][1])
                for i in range(len(members)))
            # work units: arcs of the reached vertices, per query
            deg = np.concatenate([np.diff(m.row_ptr.astype(np.int64)) for m in members])
            reached = res["bfs"] != gdb.LONESTAR_INF
            er = int(deg[reached].sum())
            vr = int(reached.sum())
            units = 2 * er
            # whole job: every rank's units over the slowest rank's time
            units_all = reduce_sum(units, world)
            value = units_all * args.steps / (ms / 1e3)
            plain_value = units_all / (reduce_max(plain_ms, world) / 1e3)
            identical = reduce_sum(0.0 if identical else 1.0, world) == 0.0
            # end to end through the host-buffer API: sources in, both
            # result arrays out, every step
            e2e = None
            if not args.no_e2e:
                B.set_sources(usrc)
                B.run()
                B.results()
                barrier(world)
                t1 = time.perf_counter()
                for _ in range(args.steps):
                    B.set_sources(usrc)
                    B.run()
                    B.results()
                dt = reduce_max(time.perf_counter() - t1, world)
                e2e = {"value": units_all * args.steps / dt, "unit": "edges/s",
                       "h2d_bytes_per_step": int(reduce_sum(4 * len(usrc), world)),
                       "d2h_bytes_per_step": int(reduce_sum(8 * V, world))}
    # algorithmic bytes of one replay: BFS + SSSP over the reached part
    nbytes = (8 * er + 12 * vr + 4 * V) + (12 * er + 12 * vr + 4 * V)
    peak, peak_kind = peaks()
    achieved = nbytes / (ms / args.steps / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_bfs_xf + k_sssp_xf (one replay)", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "alg_bytes_per_launch": nbytes, "launch_ms": ms / args.steps, "traffic": None}
    cfg = {"workload": f"mixed batch: {len(members)} graphs (V log-uniform 1e3..1e6, half R-MAT "
                       "ef 8..32, half grids aspect 1..64), BFS + SSSP per graph",
           "V": int(reduce_sum(V, world)), "E": int(reduce_sum(E, world)),
           "graphs": args.batch_graphs, "global_batch": 1,
           "parallelism": (f"graph placement over {world} GPUs (balanced by arcs)" if world > 1
                           else "one GPU"), "l2": "inputs > L2 (no flush)",
           "tuned": tune["options"] if tune else None, "generation_s": round(gen_s, 1)}
    if rank == 0:
        line = base_line(args, world, value, ms / args.steps, cfg)
        line["metric"] = "edges/sec (batched BFS + SSSP over the mixed batch)"
        line["scaling"] = "strong"  # the same 512 graphs at every GPU count
        line["clocks"] = clocks
        line["e2e"] = e2e
        line["roofline"] = roof
        line["cpu_baseline"] = None
        line["gpu_launches"] = 2 * args.steps
        line["plain"] = {"value": plain_value, "ms": plain_ms, "kernel_ms_sum": plain_kernel_ms,
                         "launches": 2 * len(members)}
        line["speedup_vs_plain"] = value / plain_value
        line["bit_identical"] = bool(identical)
        line["supersteps"] = {"bfs": steps_bfs, "sssp": steps_sssp}
        line["arcs_inspected"] = {"bfs": arcs_bfs, "sssp": arcs_sssp}
        print(json.dumps(line), flush=True)


def run_serve(args, rank, world, local):
    """Request loop: 64 resident graphs drawn like the mixed batch (V
    log-uniform in [1e3, 1e6], half R-MAT, half grids), BFS / SSSP /
    single-source BC requests arriving as a seeded Poisson stream; reports
    throughput and p50/p99 latency, and checks a sample of results against
    the same requests run alone."""
    import torch

    from gpu_discovery_barrier_gb300 import gdb, graphgen as gg, placement, selector

    torch.cuda.set_device(local)
    # the same 64 graphs and request stream at every GPU count: each GPU
    # keeps the graphs placed on it and serves the requests for them
    ngraphs = 64
    spec = gg.mixed_batch_spec(ngraphs, 1000, 1_000_000, seed=3)
    mine = my_members(ngraphs, rank, world, seed=3) or list(range(ngraphs))
    members = gg.mixed_batch(ngraphs, 1000, 1_000_000, seed=3, members=mine)
    local_of = {gi: j for j, gi in enumerate(mine)}
    rng = np.random.default_rng(17)
    n = args.requests
    gaps = rng.exponential(1.0 / args.rate, n)
    graph_of = rng.integers(0, ngraphs, n)
    app_of = rng.integers(1, 4, n)
    src_of = [int(rng.integers(spec[i]["V"])) for i in graph_of]
    with gdb.Ctx() as c:
        set_schedule(c, args.schedule)
        Gs = [c.graph(m.row_ptr, m.col, m.w) for m in members]
        deg = [np.diff(m.row_ptr.astype(np.int64)) for m in members]
        with c.server(slots=args.slots, pool_bytes=8 << 30) as srv:
            ids = [srv.add_graph(G) for G in Gs]
            # warm-up: one request per app on the smallest graph
            small = int(np.argmin([m.V for m in members]))
            for app in (1, 2, 3):
                srv.submit(ids[small], app, 0)
            srv.drain(120.0)
            srv.poll(16)
            barrier(world)
            with ClockSampler(local) as clk:
                t0 = time.perf_counter()
                due = t0
                sub = {}
                for k in range(n):
                    due += gaps[k]
                    if graph_of[k] not in local_of:
                        continue  # another GPU's graph
                    while True:
                        now = time.perf_counter()
                        if now >= due:
                            break
                        if due - now > 2e-4:
                            time.sleep(due - now - 1e-4)
                    rid, out = srv.submit(ids[local_of[graph_of[k]]], int(app_of[k]), src_of[k])
                    sub[rid] = (k, out)
                srv.drain(0)
                wall = time.perf_counter() - t0
            clocks = clk.summary()
            done = srv.poll(n + 16)
    lat = np.array([d["total_ms"] for d in done])
    run = np.array([d["run_ms"] for d in done])
    qms = np.array([d["queue_ms"] for d in done])
    ok = all(d["status"] == 0 for d in done)
    # work: arcs of the source's component (the reached arcs; BC counts its
    # forward and backward pass)
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import connected_components

    comp_arcs = []
    for m, dg in zip(members, deg):
        A = csr_matrix((np.ones(m.E, np.int8), m.col, m.row_ptr), shape=(m.V, m.V))
        _, lab = connected_components(A, directed=False)
        comp_arcs.append((lab, np.bincount(lab, weights=dg)))
    units = 0
    for d in done:
        lab, arcs = comp_arcs[d["graph"]]
        units += int(arcs[lab[d["src"]]]) * (2 if d["app"] == 3 else 1)
    # sample check: alone == in the mix
    identical = True
    with gdb.Ctx() as c2:
        set_schedule(c2, args.schedule)
        for d in done[:: max(1, len(done) // 24)]:
            k, out = sub[d["id"]]
            m = members[local_of[graph_of[k]]]
            G = c2.graph(m.row_ptr, m.col, m.w)
            app, src = d["app"], d["src"]
            if app == 1:
                identical &= bool(np.array_equal(out, c2.bfs(G, src)))
            elif app == 2:
                identical &= bool(np.array_equal(out, c2.sssp(G, src)))
            else:
                want = c2.bc(G, [src]).astype(np.float64)
                fin = np.isfinite(want)
                identical &= bool(np.array_equal(fin, np.isfinite(out)))
                if fin.any():
                    w = want[fin]
                    scale = np.maximum(np.abs(w), 1e-6 * max(1.0, float(np.abs(w).max())))
                    identical &= bool(np.all(np.abs(out[fin] - w) <= 1e-4 * scale + 1e-6))
            G.close()
    # whole job: every rank's requests, the slowest rank's wall time, the
    # latency percentiles over all requests
    per_rank = placement.gather_results({rank: {
        "lat": lat.tolist(), "run": run.tolist(), "queue": qms.tolist(), "ok": ok,
        "identical": identical, "units": units,
        "d2h": int(sum(members[local_of[graph_of[sub[d['id']][0]]]].V for d in done)) * 4}}, world)
    wall = reduce_max(wall, world)
    cfg = {"workload": f"serving: {ngraphs} resident graphs (mixed-batch distribution), "
                       f"BFS/SSSP/BC-single-source, Poisson {args.rate:g} req/s",
           "requests": n, "slots": args.slots, "global_batch": 1,
           "parallelism": (f"graph placement over {world} GPUs (balanced by arcs)" if world > 1
                           else "one GPU"),
           "l2": "inputs > L2 (no flush)", "schedule": args.schedule}
    if rank == 0:
        parts = list(per_rank.values())
        lat = np.concatenate([np.array(p["lat"]) for p in parts])
        run = np.concatenate([np.array(p["run"]) for p in parts])
        qms = np.concatenate([np.array(p["queue"]) for p in parts])
        units = sum(p["units"] for p in parts)
        value = units / wall
        line = base_line(args, world, value, 1e3 * wall / max(args.steps, 1), cfg)
        line["metric"] = "edges/sec (request loop, continuous batching)"
        line["scaling"] = "strong"  # the same request stream at every GPU count
        line["steps"] = 1
        line["clocks"] = clocks
        line["e2e"] = {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 4 * n,
                       "d2h_bytes_per_step": sum(p["d2h"] for p in parts)}
        line["roofline"] = None
        line["cpu_baseline"] = None
        line["gpu_launches"] = int(lat.size)
        line["serving"] = {
            "offered_rps": args.rate, "achieved_rps": lat.size / wall, "wall_s": wall,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "run_p50_ms": float(np.percentile(run, 50)),
            "run_p99_ms": float(np.percentile(run, 99)), "queue_p99_ms": float(np.percentile(qms, 99)),
            "all_ok": all(p["ok"] for p in parts),
            "alone_equals_mix_sample": all(p["identical"] for p in parts)}
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "grid4096":
        run_grid(args, rank, world, local)
    elif args.workload == "batch":
        run_batch(args, rank, world, local)
    elif args.workload == "serve":
        run_serve(args, rank, world, local)
    elif args.workload == "relaunch":
        run_relaunch(args, rank, world, local)
    elif args.workload == "barrier":
        run_barrier(args, rank, world, local)
    else:
        run_gdb(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
