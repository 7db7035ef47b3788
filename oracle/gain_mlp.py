"""CPU oracle of the learned form's gain network and of its training pairs.

Test infrastructure only: the GPU library never imports or calls this file.

The network (no counterpart in the reference): 65 -> 256 -> 256 -> 64,
GELU(x) = x * Phi(x) after the hidden layers, sigmoid output, loss = mean
squared error over the n x 64 gains.  Everything here is float64; the GPU
computes with BF16 weights and activations and FP32 accumulation, so the
comparison tolerances in the tests are those of BF16 rounding.

The training pairs restate the reference's step-2 Wiener rule
(src/core/nldct.cpp:2123-2135: w = y^2 / (y^2 + (beta2 sigma)^2) on the
orthonormal Haar transform of the member axis, nldct.cpp:1846-1860) for the
member-mean Haar row, with y from the basic estimate and the patch transform
Z = G.B of nldct.cpp:2061-2070 (productMatrix, src/core/matrix_funs.cpp).
"""
from __future__ import annotations

import math

import numpy as np

N_IN, N_HID, N_OUT = 65, 256, 64
SHAPES = [(N_IN, N_HID), (N_HID,), (N_HID, N_HID), (N_HID,), (N_HID, N_OUT), (N_OUT,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)

_erf = np.vectorize(math.erf, otypes=[np.float64])


def split(blob):
    blob = np.asarray(blob, np.float64).ravel()
    assert blob.size == N_PARAMS
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(blob[o:o + n].reshape(s))
        o += n
    return out


def join(parts):
    return np.concatenate([np.asarray(p, np.float64).ravel() for p in parts])


def bf16_round(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    cdf = 0.5 * (1.0 + _erf(x / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)
    return cdf + x * pdf


def forward(blob, X):
    W1, b1, W2, b2, W3, b3 = split(blob)
    P1 = X @ W1 + b1
    H1 = gelu(P1)
    P2 = H1 @ W2 + b2
    H2 = gelu(P2)
    P3 = H2 @ W3 + b3
    Y = 1.0 / (1.0 + np.exp(-P3))
    return Y, (X, P1, H1, P2, H2)


def loss_and_grad(blob, X, T):
    """Mean squared error over all outputs and its gradient (blob layout)."""
    W1, b1, W2, b2, W3, b3 = split(blob)
    Y, (X, P1, H1, P2, H2) = forward(blob, X)
    n = X.shape[0]
    E = Y - T
    loss = float(np.mean(E * E))
    dP3 = 2.0 * E / (n * N_OUT) * Y * (1.0 - Y)
    dW3 = H2.T @ dP3
    db3 = dP3.sum(0)
    dP2 = (dP3 @ W3.T) * gelu_grad(P2)
    dW2 = H1.T @ dP2
    db2 = dP2.sum(0)
    dP1 = (dP2 @ W2.T) * gelu_grad(P1)
    dW1 = X.T @ dP1
    db1 = dP1.sum(0)
    return loss, join([dW1, db1, dW2, db2, dW3, db3])


def features(Z, sigma):
    """Network inputs of one group: Z[m][k] = patch coefficients of member m."""
    var = np.mean(Z.astype(np.float64) ** 2, axis=0)
    f = np.log(np.maximum(var, 1e-6 * sigma * sigma) / (sigma * sigma))
    return np.concatenate([f, [sigma / 255.0]])


def haar(Z):
    """Orthonormal Haar transform along axis 0 (power-of-two length), in the
    reference's level order (nldct.cpp:1846-1860)."""
    z = np.array(Z, np.float64)
    n = z.shape[0]
    s, h = 2, 1
    while s <= n:
        for i in range(0, n, s):
            a, b = z[i].copy(), z[i + h].copy()
            z[i] = (a + b) / math.sqrt(2.0)
            z[i + h] = (a - b) / math.sqrt(2.0)
        s *= 2
        h *= 2
    return z


def target(Zb, sigma, beta):
    """Step-2 Wiener gains of the member-mean Haar row from the basic group's
    coefficients Zb[m][k]."""
    y = haar(Zb)[0]
    bs = beta * sigma
    return y * y / (y * y + bs * bs)
