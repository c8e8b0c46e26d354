"""CPU reference of the chemistry surrogate network (test infrastructure).

Only tests/ import this module, as the checker of libocfd's ocfd_mlp_* kernels.
It restates the network and its training step with the GPU's quantisation
points: BF16 weights, inputs and hidden activations, BF16 gradients entering the
tensor-core products, FP32 elsewhere; products are accumulated in FP64 here
(the GPU accumulates in FP32), so agreement is to FP32 rounding, with rare
one-ulp BF16 rounding flips of an activation.
"""
from __future__ import annotations

import math

import numpy as np

N_IN, N_OUT, H = 12, 10, 128
LN = (128, 128, 128, 128, 16)
LK = (16, 128, 128, 128, 128)
WOFF = (0, 2048, 18432, 34816, 51200)
WTOT = 53248
BOFF = (0, 128, 256, 384, 512)
BTOT = 528


def bf16(x):
    """round to the nearest BF16 (ties to even), as float32 values"""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


_erf = np.vectorize(math.erf, otypes=[np.float64])


def gelu(z):
    z = z.astype(np.float64)
    return (0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))).astype(np.float32)


def gelu_grad(z):
    z = z.astype(np.float64)
    return (0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)).astype(
        np.float32)


def layer(W, l):
    return W[WOFF[l]:WOFF[l] + LN[l] * LK[l]].reshape(LN[l], LK[l])


def forward(W, b, X):
    """W, b: FP32 master parameters; X: [M x 12] normalised inputs.  Returns
    (Y [M x 16], list of (input operand, Z) per layer)."""
    Wb = bf16(W)
    A = np.zeros((X.shape[0], 16), np.float32)
    A[:, :N_IN] = bf16(X)
    cache = []
    for l in range(5):
        Z = (A.astype(np.float64) @ layer(Wb, l).T.astype(np.float64)).astype(np.float32) + \
            b[BOFF[l]:BOFF[l] + LN[l]].astype(np.float32)
        cache.append((A, Z))
        if l < 4:
            A = bf16(gelu(Z))
    return Z, cache


def train_grads(W, b, X, T):
    """MSE loss over the 10 outputs and its gradients (as the GPU step computes them)."""
    M = X.shape[0]
    Y, cache = forward(W, b, X)
    d = Y[:, :N_OUT] - T
    loss = float((d.astype(np.float64) ** 2).mean())
    dZ = np.zeros_like(Y)
    dZ[:, :N_OUT] = np.float32(2.0 / (M * N_OUT)) * d
    Wb = bf16(W)
    gW = np.zeros(WTOT, np.float32)
    gb = np.zeros(BTOT, np.float32)
    for l in range(4, -1, -1):
        A, _ = cache[l]
        dZb = bf16(dZ)
        gW[WOFF[l]:WOFF[l] + LN[l] * LK[l]] = (dZb.astype(np.float64).T @ A.astype(np.float64)).astype(np.float32).ravel()
        gb[BOFF[l]:BOFF[l] + LN[l]] = dZ.astype(np.float64).sum(axis=0).astype(np.float32)
        if l > 0:
            dA = (dZb.astype(np.float64) @ layer(Wb, l).astype(np.float64)).astype(np.float32)
            dZ = dA * gelu_grad(cache[l - 1][1])
    return loss, gW, gb
