"""FP64 numpy restatement of the proposal MLP's loss and gradient.

Test infrastructure only: it checks the library's CUDA forward/backward
kernels (ecmg_mlp_loss_grad) and never runs on the product path.  The network
has no reference counterpart; the layer sizes, the tanh form of GELU and the
parameter layout follow include/ecmg.h:

    h1 = gelu(x W1 + b1), h2 = gelu(h1 W2 + b2), z = h2 W3 + b3
    loss = mean over rows of -log softmax(z)[y]
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT = 96, 128, 160
_K0 = np.sqrt(2.0 / np.pi)
_K1 = 0.044715


def bf16_to_f64(bits: np.ndarray) -> np.ndarray:
    """bf16 bit patterns (uint16) -> float64"""
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def f32_to_bf16(x: np.ndarray) -> np.ndarray:
    """round-to-nearest-even float32 -> bf16 bit patterns (uint16)"""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def split(flat):
    flat = np.asarray(flat, np.float64)
    o = 0
    out = []
    for shp in [(N_IN, N_HID), (N_HID,), (N_HID, N_HID), (N_HID,), (N_HID, N_OUT), (N_OUT,)]:
        n = int(np.prod(shp))
        out.append(flat[o:o + n].reshape(shp))
        o += n
    return out


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_K0 * (x + _K1 * x ** 3)))


def gelu_grad(x):
    u = _K0 * (x + _K1 * x ** 3)
    th = np.tanh(u)
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * _K0 * (1.0 + 3.0 * _K1 * x * x)


def forward(flat, x):
    W1, b1, W2, b2, W3, b3 = split(flat)
    z1 = x @ W1 + b1
    a1 = gelu(z1)
    z2 = a1 @ W2 + b2
    a2 = gelu(z2)
    z3 = a2 @ W3 + b3
    return z1, a1, z2, a2, z3


def loss_grad(flat, x, y):
    """mean cross-entropy and its gradient (flat, float64)"""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.int64)
    W1, b1, W2, b2, W3, b3 = split(flat)
    z1, a1, z2, a2, z3 = forward(flat, x)
    B = x.shape[0]
    m = z3.max(axis=1, keepdims=True)
    e = np.exp(z3 - m)
    se = e.sum(axis=1, keepdims=True)
    logp = z3 - m - np.log(se)
    loss = -logp[np.arange(B), y].mean()
    dz3 = e / se
    dz3[np.arange(B), y] -= 1.0
    dz3 /= B
    gW3 = a2.T @ dz3
    gb3 = dz3.sum(0)
    d2 = (dz3 @ W3.T) * gelu_grad(z2)
    gW2 = a1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ W2.T) * gelu_grad(z1)
    gW1 = x.T @ d1
    gb1 = d1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


def predict(flat, x):
    return forward(flat, np.asarray(x, np.float64))[4].argmax(axis=1)
