"""Autotuner for the batched form.

Chooses the launch shape (threads per CTA, CTAs per SM), the schedule
(plain push, or direction-optimising with its two frontier thresholds) and
whether SSSP splits its arcs into light and heavy classes, for a captured
batch, by timing replays with a coordinate search: the shape first under
the plain schedule, then the schedule and thresholds at the best shape,
then the split.  Every candidate's results are compared with the first
candidate's on the device: a configuration only changes speed, never an
answer, and the tuner raises if one does.

Results are cached in a JSON file (``$GDB_TUNE_CACHE``, default
``~/.cache/gdb_tune.json``) keyed by GPU, SM count and the batch's size, so
a restarted server starts tuned.  The reference tuned work-group sizes by
hand-kept tables per app and device (pannotia/scripts/wg_size_data.py,
lonestar/scripts/wg_size_data.py); this replaces those tables.
"""
from __future__ import annotations

import json
import os
import statistics
from pathlib import Path

from . import gdb

SHAPES = [(512, 3), (512, 2), (512, 1), (256, 6), (256, 4)]
SCHEDULES = [(gdb.SCHED_PLAIN, 0, 0), (gdb.SCHED_ADAPTIVE, 14, 24), (gdb.SCHED_ADAPTIVE, 8, 24),
             (gdb.SCHED_ADAPTIVE, 24, 24), (gdb.SCHED_ADAPTIVE, 14, 64)]
LEARNED = (gdb.SCHED_LEARNED, 0, 0)  # tried when the context holds a selector


def cache_path() -> Path:
    return Path(os.environ.get("GDB_TUNE_CACHE", Path.home() / ".cache" / "gdb_tune.json"))


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass


def key(ctx: gdb.Ctx, g: gdb.Graph, nsrc: int, apps: int) -> str:
    info = ctx.device_info()
    return f"sm{info['sm_count']}_cc{info['cc_major']}{info['cc_minor']}|V{g.V}|E{g.E}|q{nsrc}|apps{apps}"


def _options(shape, sched, sms: int, split: int = 0) -> dict:
    (block, per_sm), (schedule, alpha, beta) = shape, sched
    return {"block_size": block, "max_ctas": per_sm * sms, "schedule": schedule,
            "pull_alpha": alpha, "push_beta": beta, "sssp_split": split}


def _time(ctx: gdb.Ctx, g: gdb.Graph, sources, apps: int, opts: dict, reps: int, ref):
    """Median replay time of one configuration and its device results."""
    import torch

    ctx.set_options(**opts)
    with ctx.batch(g, sources, apps) as b:
        b.run()
        ms = statistics.median(b.run() for _ in range(reps))
        outs = []
        for app in (gdb.BATCH_BFS, gdb.BATCH_SSSP):
            if apps & app:
                outs.append(_device_u32(torch, b.device_result(app), g.V))
        if ref is not None:
            for a, r in zip(outs, ref):
                if not torch.equal(a, r):
                    raise RuntimeError(f"autotune: configuration {opts} changed the results")
            outs = None
    return ms, outs


def _device_u32(torch, ptr: int, n: int):
    """Copy of n uint32 (viewed as int32) from a library-owned device array."""
    return torch.as_tensor(gdb.DeviceArray(ptr, n, "<i4"), device="cuda").clone()


def tune_batch(ctx: gdb.Ctx, g: gdb.Graph, sources, apps: int = 3, reps: int = 3,
               use_cache: bool = True) -> dict:
    """Tune, set the best options on ctx and return
    {"options": ..., "ms": ..., "trials": [...], "cached": bool}."""
    k = key(ctx, g, len(sources), apps)
    cache = _load() if use_cache else {}
    if k in cache:
        ctx.set_options(**cache[k]["options"])
        return dict(cache[k], cached=True)
    sms = ctx.device_info()["sm_count"]
    base = {f: getattr(ctx.opt, f) for f in ("block_size", "max_ctas", "schedule", "pull_alpha",
                                             "push_beta", "sssp_split")}
    trials = []
    ref = None
    best = None
    for shape in SHAPES:
        opts = _options(shape, SCHEDULES[0], sms)
        try:
            ms, outs = _time(ctx, g, sources, apps, opts, reps, ref)
        except gdb.GdbError as e:
            trials.append({"options": opts, "error": str(e)})
            continue
        if ref is None:
            ref = outs
        trials.append({"options": opts, "ms": ms})
        if best is None or ms < best[1]:
            best = (shape, ms)
    if best is None:
        ctx.set_options(**base)
        raise RuntimeError("autotune: no configuration ran")
    shape = best[0]
    best_opts, best_ms = _options(shape, SCHEDULES[0], sms), best[1]
    scheds = SCHEDULES[1:] + ([LEARNED] if getattr(ctx, "has_selector", False) else [])
    best_sched = SCHEDULES[0]
    for sched in scheds:
        opts = _options(shape, sched, sms)
        ms, _ = _time(ctx, g, sources, apps, opts, reps, ref)
        trials.append({"options": opts, "ms": ms})
        if ms < best_ms:
            best_opts, best_ms, best_sched = opts, ms, sched
    # the SSSP light/heavy arc split (automatic by default): a batch whose
    # members include high-diameter graphs can do better without it
    if apps & gdb.BATCH_SSSP and best_sched[0] != gdb.SCHED_PLAIN:
        opts = _options(shape, best_sched, sms, split=-1)
        ms, _ = _time(ctx, g, sources, apps, opts, reps, ref)
        trials.append({"options": opts, "ms": ms})
        if ms < best_ms:
            best_opts, best_ms = opts, ms
    ctx.set_options(**best_opts)
    out = {"options": best_opts, "ms": best_ms, "trials": trials}
    if use_cache:
        cache = _load()
        cache[k] = out
        _store(cache)
    return dict(out, cached=False)
