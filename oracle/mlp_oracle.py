"""FP64 numpy restatement of the proposal MLP's loss and gradient.

Test infrastructure only: it checks the library's CUDA forward/backward
kernels (ecmg_mlp_loss_grad) and never runs on the product path; with
bf16_operands it rounds the matrix-product operands as the library's
tensor-core GEMMs do.  The network
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


def _bf16(a):
    """float64 -> float32 -> bf16 (round to nearest even) -> float64"""
    return bf16_to_f64(f32_to_bf16(np.asarray(a, np.float32)))


def loss_grad(flat, x, y, bf16_operands=False):
    """mean cross-entropy and its gradient (flat, float64).  With
    bf16_operands every matrix-product operand is rounded to BF16 as the
    library's tensor-core GEMMs take it (weights, activations between layers,
    the backward deltas); sums, biases and elementwise steps stay wide."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.int64)
    r = _bf16 if bf16_operands else (lambda a: a)
    W1, b1, W2, b2, W3, b3 = split(flat)
    z1 = r(x) @ r(W1) + b1
    a1 = gelu(z1)
    z2 = r(a1) @ r(W2) + b2
    a2 = gelu(z2)
    z3 = r(a2) @ r(W3) + b3
    B = x.shape[0]
    m = z3.max(axis=1, keepdims=True)
    e = np.exp(z3 - m)
    se = e.sum(axis=1, keepdims=True)
    logp = z3 - m - np.log(se)
    loss = -logp[np.arange(B), y].mean()
    dz3 = e / se
    dz3[np.arange(B), y] -= 1.0
    dz3 /= B
    gW3 = r(a2).T @ r(dz3)
    gb3 = dz3.sum(0)
    d2 = (r(dz3) @ r(W3).T) * gelu_grad(z2)
    gW2 = r(a1).T @ r(d2)
    gb2 = d2.sum(0)
    d1 = (r(d2) @ r(W2).T) * gelu_grad(z1)
    gW1 = r(x).T @ r(d1)
    gb1 = d1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


def predict(flat, x):
    return forward(flat, np.asarray(x, np.float64))[4].argmax(axis=1)
