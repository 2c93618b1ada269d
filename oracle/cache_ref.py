"""CPU reference of the radiance cache (TEST INFRASTRUCTURE ONLY: tests/ use it to check the
library's cache kernels; the product never imports it).

Restates with torch on the CPU what the cache kernels compute:
  encode(v, lo, hi)        the 64 network inputs of cache vertices
  forward(w, x)            outputs (n, 3) and the activations
  gradient_emulated(w,x,y) mean gradient of the relative L2 loss with BF16 rounding at the
                           points where the kernels round (inputs, weights, activations,
                           output gradients), products accumulated in float32: agrees with the
                           GPU up to float32 summation order
  gradient_fp32(w,x,y)     plain float32 autograd of the same loss (the gradient the kernels
                           approximate)
  adam_step(...)           one Adam update
Loss: sum over rows and channels of (p - y)^2 / (p^2 + 0.01), the denominator held constant,
divided by 3 n (Mueller et al. 2021, relative L2).
"""
import numpy as np
import torch

LAYERS = [(64, 64)] * 5 + [(16, 64)]
N_PARAMS = sum(o * i for o, i in LAYERS)
LIVE_END = 5 * 4096 + 3 * 64


def split(w):
    out, off = [], 0
    for o, i in LAYERS:
        out.append(w[off:off + o * i].reshape(o, i))
        off += o * i
    return out


def bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def forward(w, x, bf16=True):
    W = [torch.as_tensor(np.asarray(l, np.float32)) for l in split(np.asarray(w, np.float32))]
    h = torch.as_tensor(np.asarray(x, np.float32))
    if bf16:
        W = [bf(m) for m in W]
        h = bf(h)
    hs = [h]
    for l in range(5):
        h = torch.relu(h @ W[l].T)
        if bf16:
            h = bf(h)
        hs.append(h)
    return (h @ W[5].T)[:, :3], hs, W


def gradient_emulated(w, x, y):
    p, hs, W = forward(w, x, True)
    y = torch.as_tensor(np.asarray(y, np.float32))
    n = p.shape[0]
    d = p - y
    den = p * p + 0.01
    loss = float((d * d / den).sum() / (3 * n))
    dz = torch.zeros(n, 16)
    dz[:, :3] = bf(2.0 * d / den)
    grads = [None] * 6
    grads[5] = dz.T @ hs[5]
    for l in range(4, -1, -1):
        dh = dz @ W[l + 1]
        dz = bf(dh * (hs[l + 1] > 0))
        grads[l] = dz.T @ hs[l]
    g = torch.cat([t.reshape(-1) for t in grads]) / (3 * n)
    g[LIVE_END:] = 0.0
    return g.numpy(), loss


def gradient_fp32(w, x, y):
    wt = torch.tensor(np.asarray(w, np.float32), requires_grad=True)
    xt = torch.as_tensor(np.asarray(x, np.float32))
    yt = torch.as_tensor(np.asarray(y, np.float32))
    off, h = 0, xt
    mats = []
    for o, i in LAYERS:
        mats.append(wt[off:off + o * i].reshape(o, i))
        off += o * i
    for l in range(5):
        h = torch.relu(h @ mats[l].T)
    p = (h @ mats[5].T)[:, :3]
    loss = ((p - yt) ** 2 / (p.detach() ** 2 + 0.01)).sum() / (3 * xt.shape[0])
    loss.backward()
    g = wt.grad.clone()
    g[LIVE_END:] = 0.0
    return g.numpy(), float(loss.detach())


def adam_step(w, m, v, g, t, lr, beta1, beta2, eps):
    w, m, v, g = (np.asarray(a, np.float64) for a in (w, m, v, g))
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    w = w - lr * mh / (np.sqrt(vh) + eps)
    w[LIVE_END:] = 0.0
    return w, m, v


def _one_blob4(s):
    i = np.arange(4, dtype=np.float32) + np.float32(0.5)
    return np.maximum(np.float32(0.0), np.float32(1.0) - np.abs(s[:, None] * np.float32(4.0) - i[None, :]))


def encode(v, lo, hi):
    """v: structured array with fields pos, roughness, wo, metallic, n, color (CACHE_VERTEX_DTYPE)."""
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    inv = np.where(hi > lo, np.float32(1.0) / np.where(hi > lo, hi - lo, 1), np.float32(1.0)).astype(np.float32)
    n = v.shape[0]
    f = np.zeros((n, 64), np.float32)
    p = np.clip((v["pos"].astype(np.float32) - lo) * inv, 0, 1).astype(np.float32)
    for a in range(3):
        for k in range(12):
            x = p[:, a] * np.float32(2.0 ** k)
            f[:, 12 * a + k] = np.abs(np.float32(4.0) * (x - np.floor(x)) - np.float32(2.0)) - np.float32(1.0)

    def sph(d):
        theta = np.arccos(np.clip(d[:, 2], -1, 1)) / np.pi
        phi = np.arctan2(d[:, 1], d[:, 0]) / (2 * np.pi) + 0.5
        return theta.astype(np.float32), phi.astype(np.float32)

    to, po = sph(v["wo"].astype(np.float64))
    tn, pn = sph(v["n"].astype(np.float64))
    f[:, 36:40] = _one_blob4(to)
    f[:, 40:44] = _one_blob4(po)
    f[:, 44:48] = _one_blob4(tn)
    f[:, 48:52] = _one_blob4(pn)
    f[:, 52:56] = _one_blob4(v["roughness"].astype(np.float32))
    m = v["metallic"].astype(np.float32)[:, None]
    c = v["color"].astype(np.float32)
    f[:, 56:59] = (1 - m) * c
    f[:, 59:62] = np.float32(0.04) * (1 - m) + c * m
    f[:, 62] = 1.0
    return f
