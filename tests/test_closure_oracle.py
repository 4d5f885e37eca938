"""CPU checks of the oracle's closure network: the analytic gradient against
central finite differences, and Adam on a quadratic."""
from __future__ import annotations

import numpy as np


def random_net(orc, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, orc.MLP_PARAMS)
    norm = np.concatenate([rng.normal(0, 0.5, 7), rng.uniform(0.5, 2.0, 7)])
    X = rng.normal(0, 1, (64, 7))
    y = rng.uniform(0, 3, 64)
    return p, norm, X, y


def test_mlp_gradient_matches_finite_differences(orc):
    p, norm, X, y = random_net(orc)
    loss, g = orc.mlp_loss_grad(p, norm, X, y)
    rng = np.random.default_rng(1)
    idx = rng.choice(orc.MLP_PARAMS, 60, replace=False)
    h = 1e-6
    for k in idx:
        e = np.zeros_like(p)
        e[k] = h
        fd = (orc.mlp_loss_grad(p + e, norm, X, y)[0] - orc.mlp_loss_grad(p - e, norm, X, y)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])), k


def test_mlp_adam_descends(orc):
    p, norm, X, y = random_net(orc, seed=3)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    l0 = orc.mlp_loss_grad(p, norm, X, y)[0]
    for t in range(1, 301):
        _, g = orc.mlp_loss_grad(p, norm, X, y)
        p, m, v = orc.mlp_adam(p, g, m, v, t, 1e-2)
    assert orc.mlp_loss_grad(p, norm, X, y)[0] < 0.2 * l0
