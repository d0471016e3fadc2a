"""FP64 CPU oracle of the learned warm-start network (TEST INFRASTRUCTURE ONLY).

Only ``tests/`` may import this module; the product library never does.  The
network has no counterpart in the reference (mpFlow starts every
reconstruction from the homogeneous distribution), so this oracle is "parity
unpinned": it restates the network's mathematics -- a GELU perceptron with a
mean-squared-error loss and its backpropagation -- in FP64 numpy, optionally
rounding to BF16 at exactly the points where the GPU kernels hold BF16
values, and is itself checked against central finite differences.

Network: Z1 = X W1^T + b1, H1 = gelu(Z1), Z2 = H1 W2^T + b2, H2 = gelu(Z2),
Y = H2 W3^T + b3; loss = sum_{b, j<valid} (Y - T)^2 / (B valid);
gelu(z) = z Phi(z) with the standard normal CDF Phi.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

SQRT1_2 = 1.0 / math.sqrt(2.0)
INV_SQRT_2PI = 1.0 / math.sqrt(2.0 * math.pi)


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even) via FP32, as FP64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z * SQRT1_2))


def gelu_deriv(z):
    return 0.5 * (1.0 + erf(z * SQRT1_2)) + z * INV_SQRT_2PI * np.exp(-0.5 * z * z)


def forward(params, x, emulate_bf16: bool = True):
    """params = (W1, b1, W2, b2, W3, b3); returns a dict of intermediates."""
    W1, b1, W2, b2, W3, b3 = [np.asarray(p, np.float64) for p in params]
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    X = r(x)
    Z1 = X @ r(W1).T + b1
    H1 = r(gelu(Z1))
    Z2 = H1 @ r(W2).T + b2
    H2 = r(gelu(Z2))
    Y = H2 @ r(W3).T + b3
    return {"X": X, "Z1": Z1, "H1": H1, "Z2": Z2, "H2": H2, "Y": Y}


def loss_and_gradients(params, x, target, valid: int, emulate_bf16: bool = True):
    """Loss and gradients (dW1, db1, dW2, db2, dW3, db3) of the mean squared
    error over the first `valid` outputs."""
    W1, b1, W2, b2, W3, b3 = [np.asarray(p, np.float64) for p in params]
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    c = forward(params, x, emulate_bf16)
    B, N = c["Y"].shape
    D = np.zeros_like(c["Y"])
    D[:, :valid] = c["Y"][:, :valid] - np.asarray(target, np.float64)[:, :valid]
    loss = float((D * D).sum() / (B * valid))
    dY = 2.0 * D / (B * valid)
    dYb = r(dY)
    db3 = dY.sum(axis=0)
    dW3 = dYb.T @ c["H2"]
    dZ2 = (dYb @ r(W3)) * gelu_deriv(c["Z2"])
    dZ2b = r(dZ2)
    db2 = dZ2.sum(axis=0)
    dW2 = dZ2b.T @ c["H1"]
    dZ1 = (dZ2b @ r(W2)) * gelu_deriv(c["Z1"])
    db1 = dZ1.sum(axis=0)
    dW1 = r(dZ1).T @ c["X"]
    return loss, (dW1, db1, dW2, db2, dW3, db3)


def loss_only(params, x, target, valid: int) -> float:
    Y = forward(params, x, emulate_bf16=False)["Y"]
    D = Y[:, :valid] - np.asarray(target, np.float64)[:, :valid]
    return float((D * D).sum() / (Y.shape[0] * valid))
