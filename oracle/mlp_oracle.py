"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

Float64 restatement of the early-retirement network of the CUDA library (csrc/frg_mlp.cuh,
csrc/frg_mlp.cu): 32 -> 64 -> 64 -> 3, ReLU, weights rounded to BF16 for the forward pass,
class-weighted softmax cross entropy averaged over the batch, and its gradient by
back-propagation with respect to the rounded weights. The network has no counterpart in
the reference; this is the checker of the library's forward, backward and optimizer
kernels (tests/test_retire_gpu.py) and is itself checked against central finite
differences (tests/test_mlp_cpu.py).

Parameter layout (as in the library): W1[64][32] b1[64] W2[64][64] b2[64] W3[3][64] b3[3].
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 32, 64, 3
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NOUT, NH)), ("b3", (NOUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def bf16_round(p):
    """Round float32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(p, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (a >> 16) & 1
    r = ((a + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    out, off = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[off:off + n].reshape(shape)
        off += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def forward(p, X):
    w = unpack(p)
    z1 = X @ w["W1"].T + w["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(z2, 0.0)
    z3 = h2 @ w["W3"].T + w["b3"]
    return z1, h1, z2, h2, z3


def loss_grad(p, X, y, class_w):
    """Mean class-weighted cross entropy and its gradient (float64)."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.int64)
    B = len(y)
    w = unpack(p)
    z1, h1, z2, h2, z3 = forward(p, X)
    m = z3.max(axis=1, keepdims=True)
    e = np.exp(z3 - m)
    se = e.sum(axis=1, keepdims=True)
    wc = np.asarray(class_w, np.float64)[y] / B
    loss = float(-(wc * (z3[np.arange(B), y] - m[:, 0] - np.log(se[:, 0]))).sum())
    onehot = np.zeros_like(z3)
    onehot[np.arange(B), y] = 1.0
    dz3 = wc[:, None] * (e / se - onehot)
    g = {"W3": dz3.T @ h2, "b3": dz3.sum(axis=0)}
    dz2 = (dz3 @ w["W3"]) * (z2 > 0)
    g["W2"], g["b2"] = dz2.T @ h1, dz2.sum(axis=0)
    dz1 = (dz2 @ w["W2"]) * (z1 > 0)
    g["W1"], g["b1"] = dz1.T @ X, dz1.sum(axis=0)
    return loss, pack(g)


def probs(p, X):
    z3 = forward(p, np.asarray(X, np.float64))[-1]
    e = np.exp(z3 - z3.max(axis=1, keepdims=True))
    return e / e.sum(axis=1, keepdims=True)
