"""The MLP oracle itself: with BF16 rounding switched off its backward pass
matches central finite differences of its forward pass (float64), so the
oracle the GPU gradients are checked against is a correct gradient."""
from __future__ import annotations

import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = np.zeros(M.P_COUNT)
    p[M.P_W1:M.P_W2] = (rng.normal(0, 0.5, (M.H, M.IN_PAD)) * (np.arange(M.IN_PAD) < M.IN)).reshape(-1)
    p[M.P_W2:M.P_W3] = rng.normal(0, 0.2, M.H * M.H)
    w3 = np.zeros((M.OUT_PAD, M.H))
    w3[:M.OUT] = rng.normal(0, 0.2, (M.OUT, M.H))
    p[M.P_W3:M.P_B1] = w3.reshape(-1)
    p[M.P_B1:M.P_B3] = rng.normal(0, 0.1, 2 * M.H)
    p[M.P_B3:M.P_B3 + M.OUT] = rng.normal(0, 0.1, M.OUT)
    samples = rng.normal(0, 1, (37, 14))
    mean = np.zeros(14)
    inv_std = np.ones(14)
    M.ROUND = False
    try:
        g, _ = M.gradient(p, samples, mean, inv_std)
        for idx in list(rng.choice(np.flatnonzero(g != 0), 40, replace=False)):
            h = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[idx] += h
            pm[idx] -= h
            fd = (M.gradient(pp, samples, mean, inv_std)[1] - M.gradient(pm, samples, mean, inv_std)[1]) / (2 * h)
            assert abs(fd - g[idx]) <= 1e-5 * max(1.0, abs(fd)), (idx, fd, g[idx])
    finally:
        M.ROUND = True


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.0e-3], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0          # halfway, even mantissa kept
    assert r[2] == 1.015625     # halfway, rounds to even (up)
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) / 3.0e-3 < 2 ** -8
