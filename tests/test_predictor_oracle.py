"""The MLP oracle (CPU): BF16 rounding known answers and the backward pass
pinned by finite differences of its float64 loss."""
import numpy as np
import pytest

from oracle import predictor_oracle as M


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7, -2.5, 3.0e-3, 65504.0,
                  1.0 + 2 ** -8 + 2 ** -20], np.float32)
    want = np.array([1.0, 1.0, 1.015625, 1.0078125, -2.5, 0.0030059814453125, 65536.0, 1.0078125], np.float32)
    assert np.array_equal(M.bf16(x), want)


def test_float64_gradient_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(5))
    p = M.init_params(3).astype(np.float64)
    x = rng.uniform(0, 1, (24, M.FEATURES))
    t = rng.uniform(0, 1, 24)
    g = M.grad_float64(p, x, t)
    eps = 1e-6
    for i in [0, 77, 4095, M.OFF_B1 - 1, M.OFF_B1 + 5, M.OFF_W2, M.OFF_W2 + 127, M.OFF_B2]:
        q = p.copy()
        q[i] += eps
        lp = M.loss_float64(q, x, t)
        q[i] -= 2 * eps
        lm = M.loss_float64(q, x, t)
        assert abs((lp - lm) / (2 * eps) - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_kernel_order_gradient_close_to_float64():
    """The BF16/FP32 restatement stays within BF16 rounding of the exact gradient."""
    rng = np.random.Generator(np.random.PCG64(6))
    p = M.init_params(4)
    x = rng.uniform(0, 1, (48, M.FEATURES)).astype(np.float32)
    t = rng.uniform(0, 1, 48).astype(np.float32)
    loss, g = M.loss_grad(p, x, t)
    pb, xb = M.bf16(p).astype(np.float64), M.bf16(x).astype(np.float64)
    g64 = M.grad_float64(pb, xb, t)
    assert loss == pytest.approx(M.loss_float64(pb, xb, t), rel=2e-2)
    assert np.abs(g - g64).max() <= 2e-2 * np.abs(g64).max()


def test_forward_shapes_and_relu():
    p = M.init_params(0)
    x = np.zeros((3, M.FEATURES), np.float32)
    y, a, hb = M.forward(p, x)
    assert y.shape == (3,) and a.shape == (3, M.HIDDEN)
    assert np.all(hb >= 0) and np.all((hb > 0) == (a > 0))
