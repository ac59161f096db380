"""Loading of the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

from gpu_discovery_barrier_gb300 import graphgen as gg

GOLDEN = Path(__file__).resolve().parent / "golden"


def _sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def names() -> list[str]:
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load(name: str):
    """(graph, weights, unique weights, priorities, fixture dict, meta)."""
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    fx = {k: z[k] for k in z.files if k != "meta"}
    if "row_ptr" in fx:
        g = gg.CSR(fx["row_ptr"], fx["col"], None, name)
        w, uw, prio = fx["w"], fx["uw"], fx["prio"]
    else:
        gen = meta["generator"]
        assert gen["kind"] == "grid"
        g = gg.grid(gen["rows"], gen["cols"])
        w = gg.uniform_weights(g, 1, 100, seed=1)
        uw = gg.unique_weights(g, seed=9)
        prio = gg.priorities(g.V, seed=4)
    # the generator must reproduce the reference's inputs exactly
    assert _sha(g.row_ptr, g.col, w, uw, prio) == meta["input_sha256"], name
    return g, w, uw, prio, fx, meta
