"""CPU oracle of the learned engine's MLP kernels (test infrastructure only:
imported by tests and never by the engine).

The reference has no learned predictor; this restates the engine's own
arithmetic so that the GPU forward, loss and gradients can be checked
value for value:

- parameters and inputs are rounded to BF16 (round to nearest even);
- hidden unit u: a = b1[u], then a = fma(W1[u][k], x[k], a) for k = 0..63;
  hb = bf16(relu(a)); part = w2[u] * hb (exact in FP32);
- output: a butterfly sum over each warp of 32 units (xor 16, 8, 4, 2, 1),
  then (w0 + w1) + (w2 + w3), then + b2, then + x[RESID] (the network
  predicts the change from the last tick's active-synapse fraction);
- loss = mean (y - t)^2 accumulated as fma(d * d, 1/B, loss); dy = (2 d)(1/B);
  per block of 16 samples, in sample order: gw2 = fma(dy, hb, gw2),
  gb2 += dy, dh = dy * w2 if a > 0 else 0, gb1 += dh, g1[k] = fma(dh, x[k], g1[k]);
  block partials are summed in block order.

FMA is emulated as one float64 operation rounded to float32 (the product of
two float32 values is exact in float64); `grad_float64` is the plain float64
gradient used to pin the backward pass by finite differences.
"""
from __future__ import annotations

import numpy as np

FEATURES, HIDDEN = 64, 128
OFF_B1 = HIDDEN * FEATURES
OFF_W2 = OFF_B1 + HIDDEN
OFF_B2 = OFF_W2 + HIDDEN
PARAMS = OFF_B2 + 1
GRAD_PER = 16
RESID = 8
f32 = np.float32


def bf16(x) -> np.ndarray:
    """Round float32 values to BF16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def fma(a, b, c) -> np.ndarray:
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def unpack(params: np.ndarray):
    p = bf16(params)
    return (p[:OFF_B1].reshape(HIDDEN, FEATURES), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2], p[OFF_B2])


def forward(params: np.ndarray, x: np.ndarray):
    """Returns (y[B], a[B][128], hb[B][128]) exactly as the kernels compute them."""
    W1, b1, w2, b2 = unpack(params)
    xb = bf16(x)
    a = np.broadcast_to(b1, (xb.shape[0], HIDDEN)).astype(np.float32).copy()
    for k in range(FEATURES):
        a = fma(W1[:, k][None, :], xb[:, k][:, None], a)
    hb = bf16(np.maximum(a, f32(0)))
    part = (w2[None, :].astype(np.float32) * hb).astype(np.float32)
    v = part.reshape(-1, 4, 32).copy()
    lanes = np.arange(32)
    for o in (16, 8, 4, 2, 1):
        v = (v + v[:, :, lanes ^ o]).astype(np.float32)
    r = v[:, :, 0]
    y = ((r[:, 0] + r[:, 1]).astype(np.float32) + (r[:, 2] + r[:, 3]).astype(np.float32)).astype(np.float32)
    y = (y + f32(b2)).astype(np.float32)
    y = (y + xb[:, RESID]).astype(np.float32)
    return y, a, hb


def loss_grad(params: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Mean squared error and its gradient with the kernels' order of operations."""
    W1, b1, w2, b2 = unpack(params)
    xb = bf16(x)
    y, a, hb = forward(params, x)
    B = x.shape[0]
    ic = f32(1.0) / f32(B)
    nb = (B + GRAD_PER - 1) // GRAD_PER
    partial = np.zeros((nb, PARAMS + 1), np.float32)
    for blk in range(nb):
        g1 = np.zeros((HIDDEN, FEATURES), np.float32)
        gb1 = np.zeros(HIDDEN, np.float32)
        gw2 = np.zeros(HIDDEN, np.float32)
        gb2 = f32(0)
        loss = f32(0)
        for s in range(blk * GRAD_PER, min(B, (blk + 1) * GRAD_PER)):
            d = f32(y[s] - f32(t[s]))
            dy = f32(f32(f32(2.0) * d) * ic)
            loss = fma(f32(d * d), ic, loss)
            gw2 = fma(dy, hb[s], gw2)
            gb2 = f32(gb2 + dy)
            dh = np.where(a[s] > 0, (dy * w2).astype(np.float32), f32(0)).astype(np.float32)
            gb1 = (gb1 + dh).astype(np.float32)
            g1 = fma(dh[:, None], xb[s][None, :], g1)
        partial[blk, :OFF_B1] = g1.reshape(-1)
        partial[blk, OFF_B1:OFF_W2] = gb1
        partial[blk, OFF_W2:OFF_B2] = gw2
        partial[blk, OFF_B2] = gb2
        partial[blk, PARAMS] = loss
    tot = np.zeros(PARAMS + 1, np.float32)
    for blk in range(nb):
        tot = (tot + partial[blk]).astype(np.float32)
    return float(tot[PARAMS]), tot[:PARAMS]


def loss_float64(params: np.ndarray, x: np.ndarray, t: np.ndarray) -> float:
    """The same loss without any rounding (float64), for finite differences."""
    p = np.asarray(params, np.float64)
    W1 = p[:OFF_B1].reshape(HIDDEN, FEATURES)
    a = np.asarray(x, np.float64) @ W1.T + p[OFF_B1:OFF_W2]
    y = np.maximum(a, 0) @ p[OFF_W2:OFF_B2] + p[OFF_B2] + np.asarray(x, np.float64)[:, RESID]
    return float(np.mean((y - np.asarray(t, np.float64)) ** 2))


def grad_float64(params: np.ndarray, x: np.ndarray, t: np.ndarray) -> np.ndarray:
    """Analytic float64 gradient of loss_float64."""
    p = np.asarray(params, np.float64)
    W1 = p[:OFF_B1].reshape(HIDDEN, FEATURES)
    xd = np.asarray(x, np.float64)
    a = xd @ W1.T + p[OFF_B1:OFF_W2]
    h = np.maximum(a, 0)
    y = h @ p[OFF_W2:OFF_B2] + p[OFF_B2] + xd[:, RESID]
    dy = 2.0 * (y - np.asarray(t, np.float64)) / x.shape[0]
    dh = (dy[:, None] * p[OFF_W2:OFF_B2][None, :]) * (a > 0)
    g = np.zeros(PARAMS)
    g[:OFF_B1] = (dh.T @ xd).reshape(-1)
    g[OFF_B1:OFF_W2] = dh.sum(0)
    g[OFF_W2:OFF_B2] = h.T @ dy
    g[OFF_B2] = dy.sum()
    return g


def init_params(seed: int = 0) -> np.ndarray:
    """Fan-in scaled uniform weights, zero biases (for tests)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(PARAMS, np.float32)
    p[:OFF_B1] = rng.uniform(-0.306, 0.306, OFF_B1)
    p[OFF_B1:OFF_W2] = rng.uniform(-0.05, 0.05, HIDDEN)
    p[OFF_W2:OFF_B2] = rng.uniform(-0.2165, 0.2165, HIDDEN)
    p[OFF_B2] = 0.01
    return p
