"""CPU oracle of the surrogate network (TEST INFRASTRUCTURE, never the product).

The reference has no learned component: this restates, in numpy, the exact
arithmetic of the BF16 training and inference kernels of
``stab_gb300/csrc/mlp.cu`` so that their forward pass, gradients and Adam
step can be checked against it, and it pins itself with float64 finite
differences (``tests/test_mlp_oracle.py``).

Network: 6 inputs -> 4 hidden layers of 256 with GELU (erf form) -> 162
outputs.  Layer l computes Z = bf16(H) @ bf16(W) + b with float32
accumulation; the hidden output H = GELU(Z) is kept in float32 and rounded
to bf16 where the next GEMM reads it.  Backward, with w_j the output weights
of the loss L = sum_ij w_j (Y_ij - T_ij)^2 / B:
    dY = 2 w (Y - T) / B                          (float32)
    dW = bf16(H_prev)^T @ bf16(dZ),  db = sum_rows dZ
    dH_prev = bf16(dZ) @ bf16(W)^T,  dZ_prev = dH_prev * GELU'(Z_prev)
Adam (float32): m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
    W -= lr * (m / (1-b1^t)) / (sqrt(v / (1-b2^t)) + eps).
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

SIZES = (6, 256, 256, 256, 256, 162)


def bf16(x) -> np.ndarray:
    """Round float32 to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (a + 0x7FFF + ((a >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def gelu(z, dtype=np.float32):
    z = np.asarray(z, dtype=np.float64)
    return (0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))).astype(dtype)


def gelu_grad(z, dtype=np.float32):
    z = np.asarray(z, dtype=np.float64)
    cdf = 0.5 * (1.0 + erf(z / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)
    return (cdf + z * pdf).astype(dtype)


def _mm(a, b, dtype=np.float32):
    # bf16 operands are exact in float32; accumulate in float64 then round
    # once (the kernels accumulate in float32: the difference is far below
    # one bf16 step)
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(dtype)


def _rounder(rounding, dtype):
    if rounding:
        return bf16
    return lambda t: np.asarray(t, dtype=dtype)


def forward(params, X, rounding=True, dtype=np.float32):
    """params: list of (W[K, N], b[N]).  Returns Y and the cache.  With
    rounding=False and dtype=float64 this is the exact network, used to pin
    the oracle's gradients by finite differences."""
    r = _rounder(rounding, dtype)
    H = np.asarray(X, dtype=dtype)
    cache = []
    for li, (W, b) in enumerate(params):
        Hin = r(H)
        Z = _mm(Hin, r(W), dtype) + np.asarray(b, dtype=dtype)
        last = li == len(params) - 1
        cache.append((Hin, Z))
        H = Z if last else gelu(Z, dtype)
    return H, cache


def loss_grad(Y, T, w, dtype=np.float32):
    B = Y.shape[0]
    d = (np.asarray(Y, np.float64) - np.asarray(T, np.float64))
    L = float(np.sum(w * d ** 2) / B)
    dY = (2.0 * np.asarray(w, np.float64) * d / B).astype(dtype)
    return L, dY


def backward(params, cache, dY, rounding=True, dtype=np.float32):
    r = _rounder(rounding, dtype)
    grads = [None] * len(params)
    dZ = dY
    for li in range(len(params) - 1, -1, -1):
        W, b = params[li]
        Hin, Z = cache[li]
        dZr = r(dZ)
        gW = _mm(Hin.T, dZr, dtype)
        gb = np.sum(dZ.astype(np.float64), axis=0).astype(dtype)
        grads[li] = (gW, gb)
        if li > 0:
            dH = _mm(dZr, r(W).T, dtype)
            _, Zp = cache[li - 1]
            dZ = (dH * gelu_grad(Zp, dtype)).astype(dtype)
    return grads


def adam(params, grads, state, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """In-place Adam step t (1-based) on float32 master weights."""
    out = []
    for (W, b), (gW, gb), st in zip(params, grads, state):
        new = []
        for p, g, key in ((W, gW, "W"), (b, gb, "b")):
            m, v = st[key]
            m[...] = (b1 * m + (1 - b1) * g).astype(np.float32)
            v[...] = (b2 * v + (1 - b2) * g * g).astype(np.float32)
            mh = m / np.float32(1 - b1 ** t)
            vh = v / np.float32(1 - b2 ** t)
            new.append((p - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32))
        out.append((new[0], new[1]))
    return out


def adam_state(params):
    return [{"W": (np.zeros_like(W), np.zeros_like(W)), "b": (np.zeros_like(b), np.zeros_like(b))}
            for W, b in params]
