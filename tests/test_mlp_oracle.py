"""The FP64 oracle of the selector network, pinned by finite differences
(CPU only): it is the checker of the CUDA forward/backward kernels."""
import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = mlp.init(3, shift=rng.normal(0, 1, 12), scale=rng.uniform(0.5, 2, 12)).astype(np.float64)
    x = rng.normal(0, 1, (40, 12))
    t = rng.normal(0, 1, (40, 6))
    m = (rng.random((40, 6)) < 0.5).astype(np.float64)
    loss, g = mlp.loss_grad(p, x, t, m)
    assert np.all(g[:24] == 0)
    eps = 1e-6
    idx = list(range(24, mlp.PARAMS, 37)) + [mlp.PARAMS - 1]
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = mlp.loss_grad(q, x, t, m)
        q[i] -= 2 * eps
        lm, _ = mlp.loss_grad(q, x, t, m)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_oracle_layout_and_forward():
    p = mlp.init(1)
    assert p.size == mlp.PARAMS == 1694
    d = mlp.unpack(p)
    assert d["W1"].shape == (12, 32) and d["W3"].shape == (32, 6)
    x = np.zeros((3, 12))
    y = mlp.forward(p, x)
    assert y.shape == (3, 6)
    np.testing.assert_allclose(mlp.pack(d), p.astype(np.float64))
