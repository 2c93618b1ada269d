"""The radiance cache's CPU reference (oracle/cache_ref.py) on its own: the emulated-BF16
gradient agrees with float32 autograd to BF16 precision, the hand-written backward equals
autograd exactly when no rounding is applied, and the encoding has its stated values."""
import numpy as np
import torch

from nbounce_gb300 import _lib as L
from oracle import cache_ref as R


def _weights(seed):
    rng = np.random.default_rng(seed)
    w = rng.uniform(-0.3, 0.3, R.N_PARAMS).astype(np.float32)
    w[R.LIVE_END:] = 0.0
    return w


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 64)).astype(np.float32)
    x[:, 62] = 1.0
    y = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    return x, y


def test_emulated_gradient_close_to_fp32_autograd():
    w = _weights(1)
    x, y = _batch(512, 2)
    ge, le = R.gradient_emulated(w, x, y)
    g32, l32 = R.gradient_fp32(w, x, y)
    assert abs(le - l32) < 2e-2 * l32
    assert np.linalg.norm(ge - g32) < 5e-2 * np.linalg.norm(g32)


def test_manual_backward_equals_autograd_without_rounding(monkeypatch):
    monkeypatch.setattr(R, "bf", lambda t: t)
    w = _weights(3)
    x, y = _batch(256, 4)
    ge, le = R.gradient_emulated(w, x, y)
    g32, l32 = R.gradient_fp32(w, x, y)
    assert abs(le - l32) < 1e-6 * l32
    assert np.linalg.norm(ge - g32) < 1e-5 * np.linalg.norm(g32)


def test_adam_first_step_is_signed_lr():
    w = np.zeros(R.N_PARAMS)
    g = np.where(np.arange(R.N_PARAMS) % 2 == 0, 1e-3, -2e-3)
    w1, _, _ = R.adam_step(w, np.zeros_like(w), np.zeros_like(w), g, 1, 1e-2, 0.9, 0.99, 1e-12)
    live = np.arange(R.N_PARAMS) < R.LIVE_END
    assert np.allclose(w1[live], -1e-2 * np.sign(g[live]), rtol=1e-6)


def test_encoding_values():
    v = np.zeros(2, L.CACHE_VERTEX_DTYPE)
    v["pos"] = [[0, 0, 0], [5, -10, 10]]
    v["wo"] = [[0, 0, 1], [1, 0, 0]]
    v["n"] = [[0, 0, -1], [0, 1, 0]]
    v["roughness"] = [0.125, 1.0]
    v["metallic"] = [0.0, 1.0]
    v["color"] = [[0.5, 0.25, 1.0], [0.2, 0.4, 0.6]]
    f = R.encode(v, [-10, -10, -10], [10, 10, 10])
    # centre of the box: p = 0.5 -> tri(0.5) = -1, then tri(1), tri(2), ... = 1
    assert f[0, 0] == -1.0 and np.all(f[0, 1:12] == 1.0)
    # theta(wo = +z) = 0 -> first bin 0.5, theta(n = -z) = 1 -> last bin 0.5
    assert np.allclose(f[0, 36:40], [0.5, 0, 0, 0]) and np.allclose(f[0, 44:48], [0, 0, 0, 0.5])
    assert np.allclose(f[0, 52:56], [1, 0, 0, 0])  # roughness 0.125 is the centre of bin 0
    assert np.allclose(f[0, 56:59], [0.5, 0.25, 1.0]) and np.allclose(f[0, 59:62], 0.04)
    assert np.allclose(f[1, 56:59], 0) and np.allclose(f[1, 59:62], [0.2, 0.4, 0.6])
    assert np.all(f[:, 62] == 1.0) and np.all(f[:, 63] == 0.0)
    assert np.all(np.abs(f[:, :36]) <= 1.0)


def test_forward_shapes():
    w = _weights(5)
    x, _ = _batch(33, 6)
    p, hs, W = R.forward(w, x)
    assert p.shape == (33, 3) and len(hs) == 6 and W[5].shape == (16, 64)
    assert isinstance(p, torch.Tensor)
