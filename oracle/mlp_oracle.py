"""CPU oracle of the learned warm-start MLP. TEST INFRASTRUCTURE ONLY.

Restates, in float64 NumPy, the network forward_gpu/backward of
forge2d_gb300/csrc/mlp.cu with the same rounding points: features and
targets are normalised in float32, the matrix-product inputs (features,
weights, hidden activations, back-propagated pre-activation gradients) are
rounded to BF16 (round to nearest even), accumulation and biases stay in
high precision, ReLU derivatives use the sign of the pre-activation. The GPU
accumulates in FP32 in another order, so results agree to FP32 rounding, not
bit for bit.

Parameter vector layout (FP32 master): W1 [64][16] (columns 12..15 zero),
W2 [64][64], W3 [8][64] (rows 2..7 zero), b1 [64], b2 [64], b3 [8].
"""
from __future__ import annotations

import numpy as np

IN, IN_PAD, H, OUT, OUT_PAD = 12, 16, 64, 2, 8
P_W1 = 0
P_W2 = P_W1 + H * IN_PAD
P_W3 = P_W2 + H * H
P_B1 = P_W3 + OUT_PAD * H
P_B2 = P_B1 + H
P_B3 = P_B2 + H
P_COUNT = P_B3 + OUT_PAD


ROUND = True  # False: no BF16 rounding (exact network, for finite differences)


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float64."""
    if not ROUND:
        return np.asarray(x, np.float64)
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float32 if ROUND else np.float64)
    w1 = p[P_W1:P_W2].reshape(H, IN_PAD)
    w2 = p[P_W2:P_W3].reshape(H, H)
    w3 = p[P_W3:P_B1].reshape(OUT_PAD, H)
    return w1, w2, w3, p[P_B1:P_B2], p[P_B2:P_B3], p[P_B3:P_COUNT]


def normalise(samples, mean, inv_std):
    s = np.asarray(samples, np.float32)
    x = np.zeros((len(s), IN_PAD), np.float32)
    x[:, :IN] = (s[:, :IN] - mean[:IN]) * inv_std[:IN]
    t = (s[:, IN:IN + OUT] - mean[IN:IN + OUT]) * inv_std[IN:IN + OUT]
    return x, t.astype(np.float64)


def forward(params, x):
    w1, w2, w3, b1, b2, b3 = unpack(params)
    xb = bf16(x)
    z1 = xb @ bf16(w1).T + b1
    h1 = bf16(np.maximum(z1, 0.0))
    z2 = h1 @ bf16(w2).T + b2
    h2 = bf16(np.maximum(z2, 0.0))
    y = h2 @ bf16(w3).T + b3
    return xb, z1, h1, z2, h2, y


def gradient(params, samples, mean, inv_std):
    """(grad vector, loss) of 0.5 * mean ||y - t||^2 over the samples."""
    x, t = normalise(samples, np.asarray(mean, np.float32), np.asarray(inv_std, np.float32))
    w1, w2, w3, _, _, _ = unpack(params)
    xb, z1, h1, z2, h2, y = forward(params, x)
    n = len(x)
    e = y[:, :OUT] - t
    loss = 0.5 * float((e * e).sum()) / n
    dy = e / n
    g = np.zeros(P_COUNT)
    g[P_W3:P_W3 + OUT * H] = (dy.T @ h2).reshape(-1)
    g[P_B3:P_B3 + OUT] = dy.sum(0)
    dh2 = dy @ bf16(w3)[:OUT]
    dz2 = dh2 * (z2 > 0)
    g[P_B2:P_B3] = dz2.sum(0)
    dz2b = bf16(dz2)
    g[P_W2:P_W3] = (dz2b.T @ h1).reshape(-1)
    dh1 = dz2b @ bf16(w2)
    dz1 = dh1 * (z1 > 0)
    g[P_B1:P_B2] = dz1.sum(0)
    dz1b = bf16(dz1)
    gw1 = dz1b.T @ xb
    gw1[:, IN:] = 0.0
    g[P_W1:P_W2] = gw1.reshape(-1)
    return g, loss


def predict(params, feats, mean, inv_std):
    """Denormalised (normal, tangent) impulse predictions of raw features."""
    f = np.asarray(feats, np.float32)
    x = np.zeros((len(f), IN_PAD), np.float32)
    x[:, :IN] = (f[:, :IN] - mean[:IN]) * inv_std[:IN]
    y = forward(params, x)[-1][:, :OUT]
    return y / np.asarray(inv_std[IN:IN + OUT], np.float64) + np.asarray(mean[IN:IN + OUT], np.float64)
