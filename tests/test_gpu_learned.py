"""Learned warm start on the GPU: the BF16 tensor-core MLP kernels against the
CPU oracle (oracle/mlp_oracle.py), sample recording by the plain solver,
training on the GPU, and what the trained network gains over the plain warm
start of new contacts (zero impulse)."""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import scenes
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def random_samples(rng, n):
    s = rng.normal(0.0, 1.0, (n, 14)).astype(np.float32)
    s[:, 12:] *= 0.3
    return s


def test_gradient_matches_oracle(gpu_lib):
    from forge2d_gb300.world import WarmStartModel
    rng = np.random.default_rng(1)
    m = WarmStartModel(seed=5)
    mean = rng.normal(0, 0.2, 14).astype(np.float32)
    inv_std = rng.uniform(0.5, 2.0, 14).astype(np.float32)
    m.set_normalization(mean, inv_std)
    p = m.params()
    p[M.P_B1:M.P_B3] = rng.normal(0, 0.1, 2 * M.H).astype(np.float32)
    m.set_params(p)
    for n in (16, 777, 4096):           # one tile, a ragged batch, a full batch
        s = random_samples(rng, n)
        g, loss = m.gradient(s)
        gr, lr = M.gradient(m.params(), s, mean, inv_std)
        assert abs(loss - lr) <= 1e-3 * max(1.0, lr)
        for name, a, b in (("W1", M.P_W1, M.P_W2), ("W2", M.P_W2, M.P_W3), ("W3", M.P_W3, M.P_B1),
                           ("b1", M.P_B1, M.P_B2), ("b2", M.P_B2, M.P_B3), ("b3", M.P_B3, M.P_COUNT)):
            err = np.linalg.norm(g[a:b] - gr[a:b]) / max(np.linalg.norm(gr[a:b]), 1e-12)
            assert err < 1e-2, (n, name, err)
    m.close()


def test_prediction_matches_oracle(gpu_lib):
    from forge2d_gb300.world import WarmStartModel
    rng = np.random.default_rng(2)
    m = WarmStartModel(seed=9)
    mean = rng.normal(0, 0.2, 14).astype(np.float32)
    inv_std = rng.uniform(0.5, 2.0, 14).astype(np.float32)
    m.set_normalization(mean, inv_std)
    f = rng.normal(0, 1, (1000, 12)).astype(np.float32)
    got = m.predict(f)
    ref = M.predict(m.params(), f, mean, inv_std)
    assert np.abs(got - ref).max() <= 1e-3 * max(1.0, np.abs(ref).max())
    m.close()


def record(seed, frames, count=3000):
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(enableSleep=0, enableContinuous=1))
    scenes.pile(g, count=count, seed=seed, width=40.0, height=100.0)
    g.set_sample_recording(400_000)
    for _ in range(frames):
        assert g.step(1.0 / 60.0, 4) == 0
    s = g.samples()
    g.close()
    return s


def test_training_gains_over_zero_warm_start(gpu_lib):
    """Trained on samples of one pile, the network's initial impulses for
    the new points of another pile are much closer to the impulses the
    solver converges to than the plain warm start (zero) is."""
    from forge2d_gb300.world import WarmStartModel
    train = record(seed=11, frames=150)
    held = record(seed=12, frames=150)
    assert len(train) > 10_000 and len(held) > 10_000
    assert np.isfinite(train).all()
    m = WarmStartModel(seed=3)
    m.fit_normalization(train)
    loss0 = m.gradient(train)[1]
    loss = m.train(train, epochs=8, batch=2048, lr=2e-3)
    assert loss < 0.5 * loss0
    pred = m.predict(held[:, :12])
    t = held[:, 12:14]
    mse_zero = float((t ** 2).mean())
    mse_model = float(((pred - t) ** 2).mean())
    assert mse_model < 0.8 * mse_zero, (mse_model, mse_zero)
    m.close()
