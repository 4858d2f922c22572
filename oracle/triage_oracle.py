"""CPU oracle of the triage network (forward, loss and backward).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA training and inference kernels.
Only tests/ may import it; the product never does.

The network has no counterpart in the reference, so this is a restatement of the
mathematics the CUDA path implements, with the same BF16 rounding points:
  a1 = bf16(relu(conv(x, bf16 W1) + b1))
  a2 = bf16(relu(conv(a1, bf16 W2) + b2))
  z  = conv(a2, bf16 W3)[..., :2] + b3[:2]                         (FP32 logits)
  L  = mean over the 2N outputs of w * (softplus(z) - y z),  w = pos_weight if y else 1
  dz = bf16(w (sigmoid(z) - y) / 2N)
  dW3 = sum_v a2[v + tap] dz[v], dY2 = bf16(convT(dz, W3) * (a2 > 0)), and so on down.
conv is a 3x3x3 cross-correlation with zero padding, W indexed [tap][cin][cout] with
tap = dx + 3 dy + 9 dz (offsets -1..1).  Arrays are (Z, Y, X, 16) float32 in memory order.
"""
from __future__ import annotations

import numpy as np

TAPS = [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(27)]  # (dx, dy, dz)
NW = 27 * 16 * 16
NPARAMS = 3 * NW + 48


def bf16(a):
    """Round float32 to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def from_row_planar(raw: np.ndarray, dims) -> np.ndarray:
    """uint16 row-planar [Z][Y][2][X][8] -> float32 (Z, Y, X, 16)."""
    X, Y, Z = dims
    r = np.asarray(raw, dtype=np.uint16).reshape(Z, Y, 2, X, 8)
    f = (r.astype(np.uint32) << 16).view(np.float32)
    return np.concatenate([f[:, :, 0], f[:, :, 1]], axis=-1)


def to_row_planar(a: np.ndarray) -> np.ndarray:
    """float32 (Z, Y, X, 16) (already BF16 values) -> uint16 row-planar."""
    b = bf16(a)
    u = (b.view(np.uint32) >> 16).astype(np.uint16)
    return np.stack([u[..., :8], u[..., 8:]], axis=2).reshape(-1)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    W = [p[i * NW:(i + 1) * NW].reshape(27, 16, 16) for i in range(3)]
    b = [p[3 * NW + 16 * i:3 * NW + 16 * (i + 1)] for i in range(3)]
    return W, b


def _shift(x, dx, dy, dz):
    """y[z, y, x] = x[z + dz, y + dy, x + dx], zero outside."""
    Z, Y, X, C = x.shape
    out = np.zeros_like(x)
    zs, ys, xs = slice(max(0, -dz), min(Z, Z - dz)), slice(max(0, -dy), min(Y, Y - dy)), slice(max(0, -dx), min(X, X - dx))
    zt, yt, xt = slice(max(0, dz), min(Z, Z + dz)), slice(max(0, dy), min(Y, Y + dy)), slice(max(0, dx), min(X, X + dx))
    out[zs, ys, xs] = x[zt, yt, xt]
    return out


def conv(x, W):
    """out[v, co] = sum_tap sum_ci x[v + off(tap), ci] W[tap, ci, co] (float64 accumulation)."""
    x = x.astype(np.float64)
    out = np.zeros(x.shape[:3] + (W.shape[2],), dtype=np.float64)
    for t, (dx, dy, dz) in enumerate(TAPS):
        out += _shift(x, dx, dy, dz) @ W[t].astype(np.float64)
    return out


def conv_t(d, W):
    """Input gradient of conv: out[u, ci] = sum_tap sum_co d[u - off(tap), co] W[tap, ci, co]."""
    d = d.astype(np.float64)
    out = np.zeros(d.shape[:3] + (W.shape[1],), dtype=np.float64)
    for t, (dx, dy, dz) in enumerate(TAPS):
        out += _shift(d, -dx, -dy, -dz) @ W[t].T.astype(np.float64)
    return out


def wgrad(x, d):
    """dW[tap, ci, co] = sum_v x[v + off(tap), ci] d[v, co]."""
    x = x.astype(np.float64)
    d2 = d.astype(np.float64).reshape(-1, d.shape[-1])
    g = np.zeros((27, x.shape[-1], d.shape[-1]), dtype=np.float64)
    for t, (dx, dy, dz) in enumerate(TAPS):
        g[t] = _shift(x, dx, dy, dz).reshape(-1, x.shape[-1]).T @ d2
    return g


def forward(feat, params, rounding=True):
    """feat: (Z, Y, X, 16) float32.  Returns a1, a2 (Z, Y, X, 16) and logits (2, Z, Y, X)."""
    W, b = unpack(params)
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    a1 = r(np.maximum(conv(feat, r(W[0])) + b[0], 0).astype(np.float32 if rounding else np.float64))
    a2 = r(np.maximum(conv(a1, r(W[1])) + b[1], 0).astype(np.float32 if rounding else np.float64))
    z = conv(a2, r(W[2]))[..., :2] + b[2][:2]
    return a1, a2, np.moveaxis(z, -1, 0).astype(np.float32 if rounding else np.float64)


def loss_and_grads(feat, params, targets, pos_weight, rounding=True):
    """Loss and gradient of every parameter (NPARAMS float64)."""
    W, b = unpack(params)
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    a1, a2, z = forward(feat, params, rounding)
    y = np.asarray(targets, dtype=np.float64).reshape(z.shape)
    z64 = z.astype(np.float64)
    w = np.where(y > 0, pos_weight, 1.0)
    n2 = z.size
    sp = np.maximum(z64, 0) + np.log1p(np.exp(-np.abs(z64)))
    loss = float((w * (sp - y * z64)).sum() / n2)
    dz = w * (1 / (1 + np.exp(-z64)) - y) / n2
    d3 = np.zeros(feat.shape[:3] + (16,), dtype=np.float64)
    d3[..., :2] = np.moveaxis(dz, 0, -1)
    d3 = r(d3.astype(np.float32) if rounding else d3)
    gW3, gb3 = wgrad(a2, d3), d3.reshape(-1, 16).sum(0)
    d2 = r((conv_t(d3, r(W[2])) * (a2 > 0)).astype(np.float32 if rounding else np.float64))
    gW2, gb2 = wgrad(a1, d2), d2.reshape(-1, 16).sum(0)
    d1 = r((conv_t(d2, r(W[1])) * (a1 > 0)).astype(np.float32 if rounding else np.float64))
    gW1, gb1 = wgrad(feat, d1), d1.reshape(-1, 16).sum(0)
    g = np.concatenate([gW1.ravel(), gW2.ravel(), gW3.ravel(), gb1, gb2, gb3])
    return loss, g
