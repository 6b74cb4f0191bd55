"""CPU restatement of the learned warm start's per-node MLP (test infrastructure).

This checks the device network kernels: forward pass, mean
squared error loss and its gradient, in float64 numpy, with the weights
rounded to bfloat16 exactly as the device kernels read them (round to
nearest even of the float32 value) and the biases kept in float32.

The network is not part of EndoBeams.jl (the reference starts each Newton
loop from the HHT predictor, src/predictor.jl:1-27); its definition here is
the one the library's C ABI documents: 48 -> 128 -> 128 -> 6, SiLU
activations, parameter vector W1 [48 x 128] row-major, b1, W2, b2, W3, b3.
"""
from __future__ import annotations

import numpy as np

NIN, H, NOUT = 48, 128, 6
OFF_W1 = 0
OFF_B1 = OFF_W1 + NIN * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * NOUT
NPARAMS = OFF_B3 + NOUT


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    r = ((b + 0x7FFF + lsb) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(params: np.ndarray, bf16: bool = True):
    p = np.asarray(params, np.float32)
    w = bf16_round(p) if bf16 else p
    W1 = w[OFF_W1:OFF_B1].reshape(NIN, H).astype(np.float64)
    W2 = w[OFF_W2:OFF_B2].reshape(H, H).astype(np.float64)
    W3 = w[OFF_W3:OFF_B3].reshape(H, NOUT).astype(np.float64)
    b1 = p[OFF_B1:OFF_W2].astype(np.float64)
    b2 = p[OFF_B2:OFF_W3].astype(np.float64)
    b3 = p[OFF_B3:].astype(np.float64)
    return W1, b1, W2, b2, W3, b3


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(params, X, bf16=True, keep=False):
    W1, b1, W2, b2, W3, b3 = unpack(params, bf16)
    x = np.asarray(X, np.float32).astype(np.float64)
    z1 = x @ W1 + b1
    h1 = z1 * _sig(z1)
    z2 = h1 @ W2 + b2
    h2 = z2 * _sig(z2)
    y = h2 @ W3 + b3
    if keep:
        return y, (x, z1, h1, z2, h2)
    return y


def loss_grad(params, X, T, bf16=True):
    """Loss = mean over rows and outputs of (y - T)^2 (NaN targets contribute 0,
    the mean still divides by all rows); gradient with respect to the float32
    parameters (weights enter through their bfloat16 rounding)."""
    W1, b1, W2, b2, W3, b3 = unpack(params, bf16)
    y, (x, z1, h1, z2, h2) = forward(params, X, bf16, keep=True)
    T = np.asarray(T, np.float64)
    n = x.shape[0]
    d = np.where(np.isnan(T), 0.0, y - np.nan_to_num(T))
    loss = float((d * d).sum() / (n * NOUT))
    dy = d * (2.0 / (n * NOUT))
    g = np.zeros(NPARAMS)
    g[OFF_W3:OFF_B3] = (h2.T @ dy).ravel()
    g[OFF_B3:] = dy.sum(0)
    s2 = _sig(z2)
    dz2 = (dy @ W3.T) * (s2 + z2 * s2 * (1 - s2))
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    s1 = _sig(z1)
    dz1 = (dz2 @ W2.T) * (s1 + z1 * s1 * (1 - s1))
    g[OFF_W1:OFF_B1] = (x.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g


def init_params(seed: int = 0, out_gain: float = 0.1) -> np.ndarray:
    """He-style initialisation; the output layer scaled by out_gain."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    p[OFF_W1:OFF_B1] = rng.standard_normal(NIN * H) * np.sqrt(2.0 / NIN)
    p[OFF_W2:OFF_B2] = rng.standard_normal(H * H) * np.sqrt(2.0 / H)
    p[OFF_W3:OFF_B3] = rng.standard_normal(H * NOUT) * np.sqrt(1.0 / H) * out_gain
    return p
