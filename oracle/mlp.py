"""FP64 CPU oracle of the schedule selector's network -- TEST INFRASTRUCTURE.

Only tests/ use this module, as the checker of the CUDA forward/backward
kernels (gdb_mlp_forward, gdb_mlp_loss_grad).  It restates the network and
its loss in numpy float64:

    xn = (x - shift) * scale
    h1 = relu(xn @ W1 + b1)       W1: [12, 32]
    h2 = relu(h1 @ W2 + b2)       W2: [32, 32]
    y  = h2 @ W3 + b3             W3: [32, 6]
    L  = sum(m * (y - t)^2) / sum(m)

with the parameter blob laid out as shift[12], scale[12], W1, b1, W2, b2,
W3, b3 (row-major, input-major weights); the gradient of the shift/scale
entries is defined as 0 (they are fitted once and kept fixed).
"""
from __future__ import annotations

import numpy as np

F, H1, H2, OUT = 12, 32, 32, 6
SIZES = [("shift", (F,)), ("scale", (F,)), ("W1", (F, H1)), ("b1", (H1,)), ("W2", (H1, H2)),
         ("b2", (H2,)), ("W3", (H2, OUT)), ("b3", (OUT,))]
PARAMS = sum(int(np.prod(s)) for _, s in SIZES)  # 1694


def unpack(p: np.ndarray) -> dict:
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def forward(p: np.ndarray, x: np.ndarray) -> np.ndarray:
    q = unpack(p)
    xn = (np.asarray(x, dtype=np.float64) - q["shift"]) * q["scale"]
    h1 = np.maximum(xn @ q["W1"] + q["b1"], 0.0)
    h2 = np.maximum(h1 @ q["W2"] + q["b2"], 0.0)
    return h2 @ q["W3"] + q["b3"]


def loss_grad(p: np.ndarray, x: np.ndarray, t: np.ndarray, m: np.ndarray) -> tuple[float, np.ndarray]:
    q = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    inv = 1.0 / m.sum() if m.sum() > 0 else 0.0
    xn = (x - q["shift"]) * q["scale"]
    a1 = xn @ q["W1"] + q["b1"]
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ q["W2"] + q["b2"]
    h2 = np.maximum(a2, 0.0)
    y = h2 @ q["W3"] + q["b3"]
    e = y - t
    loss = float((m * e * e).sum() * inv)
    dy = 2.0 * m * e * inv
    dh2 = (dy @ q["W3"].T) * (a2 > 0)
    dh1 = (dh2 @ q["W2"].T) * (a1 > 0)
    g = {"shift": np.zeros(F), "scale": np.zeros(F),
         "W1": xn.T @ dh1, "b1": dh1.sum(0), "W2": h1.T @ dh2, "b2": dh2.sum(0),
         "W3": h2.T @ dy, "b3": dy.sum(0)}
    return loss, pack(g)


def init(seed: int, shift=None, scale=None) -> np.ndarray:
    """He-initialised parameters (float32 blob) with the given normalisation."""
    rng = np.random.default_rng(seed)
    d = {"shift": np.zeros(F) if shift is None else shift,
         "scale": np.ones(F) if scale is None else scale,
         "W1": rng.normal(0, np.sqrt(2 / F), (F, H1)), "b1": np.zeros(H1),
         "W2": rng.normal(0, np.sqrt(2 / H1), (H1, H2)), "b2": np.zeros(H2),
         "W3": rng.normal(0, np.sqrt(1 / H2), (H2, OUT)), "b3": np.zeros(OUT)}
    return pack(d).astype(np.float32)
