"""Pins the numpy restatement of the warm-start network (oracle/mlp.py) by central
finite differences, so that it can check the GPU gradients."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import mlp  # noqa: E402


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = rng.normal(0, 0.2, mlp.N_PARAMS)
    X = rng.normal(0, 1, (40, mlp.F))
    y = rng.normal(0, 1, 40)
    loss, g = mlp.loss_grad(p, X, y)
    idx = np.concatenate([rng.choice(np.arange(o, o + n), 6, replace=False)
                          for o, n in ((mlp.OFF_W1, 128 * mlp.F), (mlp.OFF_B1, 128), (mlp.OFF_W2, 16384),
                                       (mlp.OFF_B2, 128), (mlp.OFF_W3, 16384), (mlp.OFF_B3, 128),
                                       (mlp.OFF_W4, 128))] + [[mlp.OFF_B4]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp.loss_grad(pp, X, y)[0] - mlp.loss_grad(pm, X, y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    assert loss > 0


def test_parameter_layout_size():
    assert mlp.N_PARAMS == 35585 == 128 * 18 + 128 + 2 * (128 * 128 + 128) + 128 + 1
