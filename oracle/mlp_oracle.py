"""CPU oracle (test infrastructure) of the learned-initial-guess MLP:
forward pass, mean-squared-error loss and gradients in float64 numpy, with
the BF16 roundings the GPU path applies (GEMM operands and the stored SiLU
outputs and activation gradients), so that the tensor-core kernels can be
checked gradient by gradient.  Layout of the flat parameter vector as in
channel_flow_gb300.mlp (W1 [128 x 320], b1, W2 [128 x 128], b2,
W3T [128 x 16], b3)."""
from __future__ import annotations

import numpy as np

H, K1, N3, OUT = 128, 320, 16, 5


def bf16(x):
    """Round to BF16 (nearest even) and return as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _split(p, offs):
    out = {}
    for name, (o, s) in offs.items():
        out[name] = np.asarray(p[o:o + int(np.prod(s))], dtype=np.float64).reshape(s)
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward_backward(p, offs, X, T, M):
    """X [Mpad x 320] (BF16 values), T [Mpad x 16]; loss and gradients over
    the first M rows."""
    P = _split(p, offs)
    W1, W2, W3T = bf16(P["W1"]), bf16(P["W2"]), bf16(P["W3T"])
    X = np.asarray(X, np.float64)
    Z1 = X @ W1.T + P["b1"]
    H1 = bf16(silu(Z1))
    Z2 = H1 @ W2.T + P["b2"]
    H2 = bf16(silu(Z2))
    Y = H2 @ W3T + P["b3"]
    Mpad = X.shape[0]
    dYf = np.zeros((Mpad, N3))
    d = Y[:M, :OUT] - T[:M, :OUT]
    loss = float(np.sum(d * d))
    dYf[:M, :OUT] = 2.0 * d / (M * OUT)
    dY = bf16(dYf)
    dH2 = dY @ W3T.T
    s2 = 1.0 / (1.0 + np.exp(-Z2))
    dZ2 = bf16(dH2 * s2 * (1 + Z2 * (1 - s2)))
    dH1 = dZ2 @ W2
    s1 = 1.0 / (1.0 + np.exp(-Z1))
    dZ1 = bf16(dH1 * s1 * (1 + Z1 * (1 - s1)))
    g = {"W3T": H2.T @ dY, "b3": dY.sum(0), "W2": dZ2.T @ H1, "b2": dZ2.sum(0), "W1": dZ1.T @ X,
         "b1": dZ1.sum(0)}
    flat = np.zeros(len(p))
    for name, (o, s) in offs.items():
        flat[o:o + int(np.prod(s))] = g[name].ravel()
    return loss, Y, flat
