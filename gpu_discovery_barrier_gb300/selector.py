"""The learned schedule selector: trace generation, training, regret.

The network (12 features, two hidden layers of 32, 6 outputs, FP32; layout
in csrc/gdb_selector.cuh) predicts log2 costs of the options of two
decisions:

* BFS, per level, taken by the master CTA inside the barrier before the
  level: push (top-down from the queue) or pull (bottom-up against the
  previous level).  Levels are the same under any schedule, so one all-push
  and one all-pull run of a graph time both options at every level (the
  level's duration from barrier to barrier), and the trace-optimal schedule
  is the per-level minimum.
* SSSP, per run: label-correcting worklist, near-far at the automatic
  bucket width, near-far at 4x that width, or the worklist under graph
  relaunch.  Each option is timed on every training graph.
* SSSP, per settle superstep of the light/heavy split, taken inside the
  kernel at the start of the superstep: push (the bucket's vertices relax
  their heavy arcs) or pull (every vertex beyond the split takes the
  minimum over its heavy in-arcs), the same push / pull outputs as a BFS
  level with decision kind 3.  Both directions give the same distances, so
  the run's supersteps are the same under any choice: an all-push and an
  all-pull run time both options at every settle, as for BFS levels.

Training runs on the GPU through the library's own CUDA kernels
(gdb_mlp_train: forward, backward and Adam); the gradient of those kernels
is checked against an FP64 CPU restatement in the tests.  Regret is the
extra time of the selector's choices over the trace-optimal ones, and gain
the time saved against the plain schedule (all push; worklist SSSP).
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import gdb, graphgen as gg

WEIGHTS = Path(__file__).resolve().parent / "selector_weights.json"
F, OUT = gdb.MLP_FEATURES, gdb.MLP_OUTPUTS
PUSH, PULL, SSSP_PLAIN, SSSP_NF, SSSP_NF4, SSSP_RELAUNCH = range(6)


def init_params(seed: int, shift: np.ndarray, scale: np.ndarray) -> np.ndarray:
    """He-initialised blob with a fixed feature normalisation."""
    rng = np.random.default_rng(seed)
    parts = [shift, scale, rng.normal(0, math.sqrt(2 / F), (F, 32)), np.zeros(32),
             rng.normal(0, math.sqrt(2 / 32), (32, 32)), np.zeros(32),
             rng.normal(0, math.sqrt(1 / 32), (32, OUT)), np.zeros(OUT)]
    p = np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in parts]).astype(np.float32)
    assert p.size == gdb.MLP_PARAMS
    return p


def load(path: Path = WEIGHTS) -> np.ndarray | None:
    try:
        d = json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return None
    p = np.asarray(d["params"], dtype=np.float32)
    return p if p.size == gdb.MLP_PARAMS else None


def save(params: np.ndarray, meta: dict, path: Path = WEIGHTS) -> None:
    Path(path).write_text(json.dumps({"params": [float(v) for v in params], "meta": meta}))


# ------------------------------------------------------------------ traces


@dataclass
class BfsTrace:
    name: str
    x: np.ndarray        # [L, 12] features of each level (from the push run)
    us_push: np.ndarray  # [L]
    us_pull: np.ndarray  # [L]


def bfs_trace(ctx: gdb.Ctx, G: gdb.Graph, src: int, name: str = "", reps: int = 2) -> BfsTrace:
    """Per-level durations of the all-push and all-pull schedules (the
    median over `reps` runs of each)."""
    runs = {}
    for mode in (0, 1):
        us = []
        for _ in range(reps):
            _, x, _, t = ctx.bfs_trace(G, src, mode)
            us.append(t)
            if mode == 0:
                feats = x
        runs[mode] = np.median(np.stack(us), axis=0)
    L = min(len(runs[0]), len(runs[1]), len(feats))
    return BfsTrace(name, feats[:L], runs[0][:L], runs[1][:L])


@dataclass
class SsspSample:
    name: str
    x: np.ndarray      # [12]
    ms: np.ndarray     # [4]: worklist, near-far, near-far x4, relaunch


def sssp_sample(ctx: gdb.Ctx, G: gdb.Graph, src: int, name: str = "", reps: int = 2) -> SsspSample:
    base = {f: getattr(ctx.opt, f) for f in ("barrier", "schedule", "sssp_delta")}
    x = ctx.sssp_features(G, 1)
    ctx.set_options(barrier=gdb.BARRIER_XF, schedule=gdb.SCHED_ADAPTIVE, sssp_delta=0)
    ctx.sssp(G, src)
    delta = ctx.last_stats()["sssp_delta"]
    configs = [dict(barrier=gdb.BARRIER_XF, schedule=gdb.SCHED_PLAIN, sssp_delta=0),
               dict(barrier=gdb.BARRIER_XF, schedule=gdb.SCHED_PLAIN, sssp_delta=delta),
               dict(barrier=gdb.BARRIER_XF, schedule=gdb.SCHED_PLAIN, sssp_delta=4 * delta),
               dict(barrier=gdb.BARRIER_RELAUNCH_GRAPH, schedule=gdb.SCHED_PLAIN, sssp_delta=0)]
    ms = []
    for cfg in configs:
        ctx.set_options(**cfg)
        t = []
        for _ in range(reps):
            ctx.sssp(G, src)
            t.append(ctx.last_stats()["kernel_ms"])
        ms.append(float(np.median(t)))
    ctx.set_options(**base)
    return SsspSample(name, x, np.asarray(ms))


@dataclass
class SettleTrace:
    name: str
    x: np.ndarray        # [S, 12] features of each settle superstep (kind 3)
    us_push: np.ndarray  # [S]
    us_pull: np.ndarray  # [S]


def settle_trace(ctx: gdb.Ctx, G: gdb.Graph, src: int, name: str = "", reps: int = 2) -> SettleTrace:
    """Per-settle durations of the all-push and all-pull settle directions
    under the near-far schedule with the light/heavy split at the automatic
    width (the median over `reps` runs of each)."""
    base = {f: getattr(ctx.opt, f) for f in ("schedule", "sssp_delta", "sssp_split")}
    ctx.set_options(schedule=gdb.SCHED_ADAPTIVE, sssp_delta=0, sssp_split=0)
    runs, feats = {}, np.zeros((0, F), np.float32)
    for mode in (0, 1):
        us = []
        for _ in range(reps):
            _, x, _, t = ctx.sssp_trace(G, src, mode)
            us.append(t)
            if mode == 0:
                feats = x
        n = min(len(u) for u in us)
        runs[mode] = np.median(np.stack([u[:n] for u in us]), axis=0)
    ctx.set_options(**base)
    S = min(len(runs[0]), len(runs[1]), len(feats))
    return SettleTrace(name, feats[:S], runs[0][:S], runs[1][:S])


def settle_rule(x: np.ndarray) -> np.ndarray:
    """The fixed settle direction (1 = pull) from the features: pull when
    the unsettled vertices' heavy arcs plus one look at every vertex are
    fewer than the bucket's heavy arcs."""
    mf = np.exp2(x[:, 1]) - 1
    mu = np.exp2(x[:, 2]) - 1
    V = np.exp2(x[:, 3]) - 1
    return (mu + V < mf).astype(np.int64)


def training_graphs(small: bool = False):
    """Synthetic graphs spanning the workloads' shapes: R-MAT of several
    scales and edge factors, square and elongated grids, mixed-batch
    members.  Each entry: (name, CSR with weights, sources)."""
    out = []
    scales = [10, 12, 14] if small else [12, 14, 16, 18, 20, 22]
    for sc in scales:
        for ef in ((8, 32) if small else (8, 16, 32)):
            g = gg.rmat_scale(sc, ef, seed=100 + sc * 7 + ef)
            g = g.with_weights(gg.uniform_weights(g, 1, 255, seed=sc + ef))
            out.append((f"rmat{sc}_ef{ef}", g, [int(s) for s in gg.sources(g, 2, seed=sc)]))
    grids = [(64, 64), (16, 512)] if small else [(256, 256), (1024, 1024), (64, 8192), (2048, 2048),
                                                 (4096, 4096)]
    for r, c in grids:
        g = gg.grid(r, c)
        g = g.with_weights(gg.uniform_weights(g, 1, 1000, seed=r + c))
        out.append((f"grid{r}x{c}", g, [0]))
    for i, m in enumerate(gg.mixed_batch(4 if small else 12, 1000, 200_000, seed=77)):
        out.append((f"mixed{i}_{m.meta['kind']}", m, [m.meta["source"]]))
    return out


def collect(ctx: gdb.Ctx, graphs, reps: int = 2, ctas=(0,)):
    """Traces of every graph and source at every launch shape in `ctas`
    (options.max_ctas values; 0 = all co-resident CTAs): the warps of the
    launch are a feature, so the network sees how the options scale."""
    bfs, sssp = [], []
    base = ctx.opt.max_ctas
    for name, g, srcs in graphs:
        G = ctx.graph(g.row_ptr, g.col, g.w)
        for k in ctas:
            ctx.set_options(max_ctas=k)
            for s in srcs:
                bfs.append(bfs_trace(ctx, G, s, f"{name}@{k}", reps))
                sssp.append(sssp_sample(ctx, G, s, f"{name}@{k}", reps))
        G.close()
    ctx.set_options(max_ctas=base)
    return bfs, sssp


def collect_settle(ctx: gdb.Ctx, graphs, reps: int = 2, ctas=(0,)):
    """Settle traces of every graph and source at every launch shape; runs
    without settle supersteps (no split) give no rows."""
    out = []
    base = ctx.opt.max_ctas
    for name, g, srcs in graphs:
        G = ctx.graph(g.row_ptr, g.col, g.w)
        for k in ctas:
            ctx.set_options(max_ctas=k)
            for s in srcs:
                tr = settle_trace(ctx, G, s, f"{name}@{k}", reps)
                if len(tr.x):
                    out.append(tr)
        G.close()
    ctx.set_options(max_ctas=base)
    return out


# --------------------------------------------------------------- training


def dataset(bfs: list[BfsTrace], sssp: list[SsspSample], settle: list[SettleTrace] = ()):
    """Rows (x, target, mask).  A BFS level yields one row per mode, its
    previous-mode feature set both ways (the implementation keeps the queue
    in both modes, so switching costs nothing); a settle superstep one row
    with its push and pull targets; targets are log2 us."""
    X, T, M = [], [], []
    for tr in settle:
        for i in range(len(tr.x)):
            t = np.zeros(OUT)
            m = np.zeros(OUT)
            t[PUSH], t[PULL] = math.log2(max(tr.us_push[i], 0.05)), math.log2(max(tr.us_pull[i], 0.05))
            m[PUSH] = m[PULL] = 1.0
            X.append(tr.x[i])
            T.append(t)
            M.append(m)
    for tr in bfs:
        for l in range(len(tr.x)):
            for prev in (0.0, 1.0):
                x = tr.x[l].copy()
                x[9] = prev
                t = np.zeros(OUT)
                m = np.zeros(OUT)
                t[PUSH], t[PULL] = math.log2(max(tr.us_push[l], 0.05)), math.log2(max(tr.us_pull[l], 0.05))
                m[PUSH] = m[PULL] = 1.0
                X.append(x)
                T.append(t)
                M.append(m)
    for s in sssp:
        t = np.zeros(OUT)
        m = np.zeros(OUT)
        for k in range(4):
            t[SSSP_PLAIN + k] = math.log2(max(s.ms[k] * 1e3, 0.05))
            m[SSSP_PLAIN + k] = 1.0
        X.append(s.x)
        T.append(t)
        M.append(m)
    return (np.asarray(X, dtype=np.float32), np.asarray(T, dtype=np.float32),
            np.asarray(M, dtype=np.float32))


def train(ctx: gdb.Ctx, X, T, M, epochs: int = 4000, lr: float = 3e-3, wd: float = 1e-4,
          seed: int = 1):
    shift = X.mean(0)
    scale = 1.0 / np.maximum(X.std(0), 1e-3)
    p0 = init_params(seed, shift, scale)
    loss0, _ = ctx.mlp_loss_grad(p0, X, T, M)
    p, loss = ctx.mlp_train(p0, X, T, M, epochs, lr, wd)
    final, _ = ctx.mlp_loss_grad(p, X, T, M)
    return p, {"loss_init": loss0, "loss_final": final, "epochs": epochs, "rows": int(len(X))}


# ------------------------------------------------------------------ regret


def bfs_choices(ctx: gdb.Ctx, p: np.ndarray, tr: BfsTrace) -> np.ndarray:
    """The selector's mode per level of a trace (previous mode threaded)."""
    modes = np.zeros(len(tr.x), dtype=np.int64)
    prev = 0
    for l in range(len(tr.x)):
        x = tr.x[l].copy()
        x[9] = prev
        y = ctx.mlp_forward(p, x)[0]
        modes[l] = 1 if y[PULL] < y[PUSH] else 0
        prev = modes[l]
    return modes


def settle_choices(ctx: gdb.Ctx, p: np.ndarray, tr: SettleTrace) -> np.ndarray:
    """The selector's direction (1 = pull) per settle superstep of a trace."""
    if not len(tr.x):
        return np.zeros(0, np.int64)
    y = ctx.mlp_forward(p, tr.x)
    return (y[:, PULL] < y[:, PUSH]).astype(np.int64)


def settle_regret(ctx: gdb.Ctx, p: np.ndarray, settle: list[SettleTrace]) -> dict:
    """Settle supersteps: the selector's choices against the per-superstep
    optimum, the fixed rule and all-push."""
    opt = sel = rule = push = 0.0
    for tr in settle:
        ch = settle_choices(ctx, p, tr)
        r = settle_rule(tr.x)
        opt += float(np.minimum(tr.us_push, tr.us_pull).sum())
        sel += float(np.where(ch == 1, tr.us_pull, tr.us_push).sum())
        rule += float(np.where(r == 1, tr.us_pull, tr.us_push).sum())
        push += float(tr.us_push.sum())
    return {"optimal_us": opt, "selector_us": sel, "rule_us": rule, "push_us": push,
            "regret": sel / opt - 1 if opt else 0.0, "gain_vs_rule": rule / sel if sel else 0.0,
            "supersteps": int(sum(len(t.x) for t in settle))}


def regret(ctx: gdb.Ctx, p: np.ndarray, bfs: list[BfsTrace], sssp: list[SsspSample]) -> dict:
    b_opt = b_sel = b_plain = 0.0
    for tr in bfs:
        ch = bfs_choices(ctx, p, tr)
        b_opt += float(np.minimum(tr.us_push, tr.us_pull).sum())
        b_sel += float(np.where(ch == 1, tr.us_pull, tr.us_push).sum())
        b_plain += float(tr.us_push.sum())
    s_opt = s_sel = s_plain = 0.0
    for s in sssp:
        y = ctx.mlp_forward(p, s.x)[0]
        k = int(np.argmin(y[SSSP_PLAIN:SSSP_PLAIN + 4]))
        s_opt += float(s.ms.min())
        s_sel += float(s.ms[k])
        s_plain += float(s.ms[0])
    return {"bfs": {"optimal_us": b_opt, "selector_us": b_sel, "plain_us": b_plain,
                    "regret": b_sel / b_opt - 1 if b_opt else 0.0,
                    "gain_vs_plain": b_plain / b_sel if b_sel else 0.0},
            "sssp": {"optimal_ms": s_opt, "selector_ms": s_sel, "plain_ms": s_plain,
                     "regret": s_sel / s_opt - 1 if s_opt else 0.0,
                     "gain_vs_plain": s_plain / s_sel if s_sel else 0.0}}


def main(argv=None) -> None:
    import argparse

    ap = argparse.ArgumentParser(description="train the schedule selector on GPU traces")
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--small", action="store_true")
    ap.add_argument("--epochs", type=int, default=4000)
    ap.add_argument("--ctas", default="152,304,0", help="launch shapes (max_ctas) to trace")
    args = ap.parse_args(argv)
    ctas = tuple(int(k) for k in args.ctas.split(","))
    graphs = training_graphs(args.small)
    held = [graphs[i] for i in range(len(graphs)) if i % 5 == 4]
    fit = [graphs[i] for i in range(len(graphs)) if i % 5 != 4]
    with gdb.Ctx() as ctx:
        bfs_fit, sssp_fit = collect(ctx, fit, ctas=ctas)
        bfs_held, sssp_held = collect(ctx, held, ctas=ctas)
        settle_fit = collect_settle(ctx, fit, ctas=ctas)
        settle_held = collect_settle(ctx, held, ctas=ctas)
        X, T, M = dataset(bfs_fit, sssp_fit, settle_fit)
        p, info = train(ctx, X, T, M, epochs=args.epochs)
        info["regret_fit"] = regret(ctx, p, bfs_fit, sssp_fit)
        info["regret_held_out"] = regret(ctx, p, bfs_held, sssp_held)
        info["regret_fit"]["settle"] = settle_regret(ctx, p, settle_fit)
        info["regret_held_out"]["settle"] = settle_regret(ctx, p, settle_held)
        info["fit_graphs"] = [n for n, _, _ in fit]
        info["held_out_graphs"] = [n for n, _, _ in held]
        info["launch_shapes"] = list(ctas)
    save(p, info, Path(args.out))
    print(json.dumps(info, indent=1))


if __name__ == "__main__":
    main()
