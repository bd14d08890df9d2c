"""CPU reference (float64) of the learned-proposal MLP's training step: the
forward pass with int8 fake-quantised weights and bfloat16 activations, the
mean-squared-error loss and its straight-through gradients (test helper; it
checks the GPU training kernels)."""
import numpy as np

F, H = 40, 64


def bf16(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def quantize_rows(w):
    m = np.abs(w).max(axis=-1, keepdims=True)
    s = np.where(m > 0, m / 127.0, 1e-8)
    return np.rint(np.clip(w / s, -127, 127)) * s


def forward_backward(w1, b1, w2, b2, x, y, round_h=True):
    w1, b1, w2, y = (np.asarray(a, dtype=np.float64) for a in (w1, b1, w2, y))
    q1 = quantize_rows(w1)
    q2 = quantize_rows(w2[None, :])[0]
    xs = np.asarray(x, dtype=np.float64) / 16.0
    pre = xs @ q1.T + b1
    h = bf16(np.maximum(pre, 0.0)) if round_h else np.maximum(pre, 0.0)
    out = h @ q2 + b2
    n = len(y)
    loss = np.mean((out - y) ** 2)
    dout = 2.0 * (out - y) / n
    gw2 = h.T @ dout
    gb2 = dout.sum()
    dpre = dout[:, None] * q2[None, :] * (pre > 0)
    gw1 = dpre.T @ xs
    gb1 = dpre.sum(axis=0)
    return loss, gw1, gb1, gw2, gb2
