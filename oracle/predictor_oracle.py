"""CPU oracle of the learned engine's MLP kernels (test infrastructure only:
imported by tests and never by the engine).

The reference has no learned predictor; this restates the engine's own
arithmetic so that the GPU forward, loss and gradients can be checked:

- parameters and inputs are rounded to BF16 (round to nearest even);
- hidden pre-activations a = b1 + W1 x: the kernels accumulate the exact
  products of BF16 values in FP32 on the tensor cores (mma m16n8k16), whose
  internal order is not specified; here they are summed in float64 and
  rounded once to float32, so a can differ from the GPU's in its last bits
  (and, rarely, the BF16 rounding of the activation with it);
- hb = bf16(relu(a)); the output layer in the kernels' fixed FP32 order: the
  units in 4 groups of 32 (32p .. 32p + 31); in a group, lane q (0..3) sums
  w2[u] * hb[u] over the tiles nt = 0..3 for u = 32p + 8nt + 2q, then +1;
  lanes (q0 + q1) + (q2 + q3); groups (G0 + G1) + (G2 + G3); + b2;
  + x[RESID] (the network predicts the change from the last tick's
  active-synapse fraction);
- per block of 16 samples: dy = (2 d) / B; loss term d^2 / B; gw2[u] and
  gb1[u] from the two rows of each lane (g, g + 8) reduced over g = 0..7 in a
  butterfly (xor 1, 2, 4 of g); dh = dy w2 where a > 0, rounded to BF16 for
  the W1 gradient (dh^T x on the tensor cores: float64 here, then float32);
  gb2 and the loss summed over the 16 rows in order; block partials summed in
  block order.

`loss_float64` / `grad_float64` are the plain float64 loss and gradient,
used to pin the backward pass by finite differences.
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


def _hidden(params: np.ndarray, x: np.ndarray):
    W1, b1, w2, b2 = unpack(params)
    xb = bf16(x)
    a = (b1[None, :].astype(np.float64) + xb.astype(np.float64) @ W1.T.astype(np.float64)).astype(np.float32)
    hb = bf16(np.maximum(a, f32(0)))
    return W1, b1, w2, b2, xb, a, hb


def _output(w2, b2, xb, hb):
    part = (w2[None, :].astype(np.float32) * hb).astype(np.float32)   # exact: BF16 x BF16
    groups = []
    for grp in range(4):
        lanes = []
        for q in range(4):
            acc = np.zeros(hb.shape[0], np.float32)
            for nt in range(4):
                u0 = 32 * grp + 8 * nt + 2 * q
                acc = (acc + part[:, u0]).astype(np.float32)
                acc = (acc + part[:, u0 + 1]).astype(np.float32)
            lanes.append(acc)
        groups.append(((lanes[0] + lanes[1]).astype(np.float32) + (lanes[2] + lanes[3]).astype(np.float32))
                      .astype(np.float32))
    y = ((groups[0] + groups[1]).astype(np.float32) + (groups[2] + groups[3]).astype(np.float32)).astype(np.float32)
    y = (y + f32(b2)).astype(np.float32)
    return (y + xb[:, RESID]).astype(np.float32)


def forward(params: np.ndarray, x: np.ndarray):
    """Returns (y[B], a[B][128], hb[B][128]) as the kernels compute them (a up to its last bits)."""
    W1, b1, w2, b2, xb, a, hb = _hidden(params, x)
    return _output(w2, b2, xb, hb), a, hb


def _butterfly8(v):
    """Sum over axis 0 (8 entries, g = 0..7) as xor 1, 2, 4 shuffles add them."""
    v = v.astype(np.float32)
    for o in (1, 2, 4):
        v = (v + v[np.arange(8) ^ o]).astype(np.float32)
    return v[0]


def loss_grad(params: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Mean squared error and its gradient with the kernels' order of operations."""
    W1, b1, w2, b2, xb, a, hb = _hidden(params, x)
    y = _output(w2, b2, xb, hb)
    B = x.shape[0]
    ic = f32(1.0) / f32(B)
    nb = (B + GRAD_PER - 1) // GRAD_PER
    tot = np.zeros(PARAMS + 1, np.float32)
    for blk in range(nb):
        rows = np.arange(blk * GRAD_PER, (blk + 1) * GRAD_PER)
        valid = rows < B
        r = np.where(valid, rows, 0)
        d = np.where(valid, (y[r] - np.asarray(t, np.float32)[r]).astype(np.float32), f32(0)).astype(np.float32)
        dy = ((f32(2.0) * d).astype(np.float32) * ic).astype(np.float32)
        lt = ((d * d).astype(np.float32) * ic).astype(np.float32)
        ab = np.where(valid[:, None], a[r], f32(0)).astype(np.float32)
        hbb = np.where(valid[:, None], hb[r], f32(0)).astype(np.float32)
        xbb = np.where(valid[:, None], xb[r], f32(0)).astype(np.float32)
        dh = np.where(ab > 0, (dy[:, None] * w2[None, :]).astype(np.float32), f32(0)).astype(np.float32)
        # rows g and g + 8 of each lane, then the butterfly over g
        v_w2 = ((dy[:8, None] * hbb[:8]).astype(np.float32) + (dy[8:, None] * hbb[8:]).astype(np.float32))
        v_b1 = (dh[:8] + dh[8:]).astype(np.float32)
        part = np.zeros(PARAMS + 1, np.float32)
        part[:OFF_B1] = (bf16(dh).astype(np.float64).T @ xbb.astype(np.float64)).astype(np.float32).reshape(-1)
        part[OFF_B1:OFF_W2] = _butterfly8(v_b1)
        part[OFF_W2:OFF_B2] = _butterfly8(v_w2)
        gb2 = f32(0)
        loss = f32(0)
        for k in range(GRAD_PER):
            gb2 = f32(gb2 + dy[k])
            loss = f32(loss + lt[k])
        part[OFF_B2] = gb2
        part[PARAMS] = loss
        tot = (tot + part).astype(np.float32)
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
