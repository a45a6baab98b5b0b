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


# ---------------------------------------------------------------------------
# data kernels: features, targets, the guess and the scalings, on fields in
# the reference layout [X_out+6][Y_out+4][Z_out+4] (interior i = 3..,
# j = 2.., k = 2..; rows x-major, z fastest)

def _interior(a, X, Y, Z, di=0, dj=0, dk=0):
    return a[3 + di:3 + di + X, 2 + dj:2 + dj + Y, 2 + dk:2 + dk + Z].reshape(-1)


def rms(levels, X, Y, Z):
    """RMS per variable of the first and second time differences
    (cf_mlp_rms); levels = [U^n, U^(n-1), U^(n-2)], five arrays each."""
    out = np.zeros(10)
    for v in range(5):
        a0, a1, a2 = (_interior(levels[l][v], X, Y, Z) for l in range(3))
        out[v] = np.sqrt(np.mean((a0 - a1) ** 2))
        out[5 + v] = np.sqrt(np.mean(((a0 - 2.0 * a1) + a2) ** 2))
    return out


def features(levels, scale10, X, Y, Z, rows=None):
    """Feature rows (BF16 values as float64) of cf_mlp_features: column
    135 l + 27 v + s = kind l (first / second difference) of variable v at
    stencil neighbour s, times the float32 reciprocal of its scale."""
    n = X * Y * Z
    rows = np.arange(n) if rows is None else np.asarray(rows)
    F = np.zeros((len(rows), K1))
    sc = np.asarray(scale10, np.float32)
    for l in range(2):
        for v in range(5):
            inv = np.float32(1.0) / sc[5 * l + v]
            for st in range(27):
                di, dj, dk = st // 9 - 1, (st // 3) % 3 - 1, st % 3 - 1
                a0 = _interior(levels[0][v], X, Y, Z, di, dj, dk)[rows]
                a1 = _interior(levels[1][v], X, Y, Z, di, dj, dk)[rows]
                if l == 0:
                    d = a0 - a1
                else:
                    d = (a0 - 2.0 * a1) + _interior(levels[2][v], X, Y, Z, di, dj, dk)[rows]
                F[:, 135 * l + 27 * v + st] = bf16(d.astype(np.float32) * inv)
    return F


def _coef(coef10):
    c = np.ones(10) if coef10 is None else np.asarray(coef10, np.float64)
    return c[:5], c[5:]


def targets(next_level, levels, scale10, oscale5, X, Y, Z, rows=None, coef10=None):
    """cf_mlp_targets: the error of the predictor U^n + a dU^n + b d2U
    (coef10 = a[0..4], b[5..9]; None: a = b = 1) over
    scale10[5+v] * oscale5[v]."""
    n = X * Y * Z
    rows = np.arange(n) if rows is None else np.asarray(rows)
    a, b = _coef(coef10)
    T = np.zeros((len(rows), N3))
    for v in range(5):
        u = [_interior(x[v], X, Y, Z)[rows] for x in (next_level, levels[0], levels[1], levels[2])]
        d1 = u[1] - u[2]
        d2 = (u[1] - 2.0 * u[2]) + u[3]
        e = ((u[0] - u[1]) - a[v] * d1) - b[v] * d2
        T[:, v] = e / (np.float64(np.float32(scale10[5 + v])) * np.float64(np.float32(oscale5[v])))
    return T


def apply(levels, scale10, oscale5, Y_out16, X, Y, Z, coef10=None):
    """cf_mlp_apply on the interior: U^n + a dU^n + b d2U + the scaled
    correction (Y_out16 None: the predictor alone); returns five interior
    arrays [X*Y*Z]."""
    a, b = _coef(coef10)
    out = []
    for v in range(5):
        un, u1, u2 = (_interior(levels[l][v], X, Y, Z) for l in range(3))
        c = 0.0
        if Y_out16 is not None:
            c = np.float64(np.float32(scale10[5 + v])) * np.float64(np.float32(oscale5[v])) * \
                np.asarray(Y_out16[:, v], np.float64)
        d1 = un - u1
        d2 = (un - 2.0 * u1) + u2
        out.append(((un + a[v] * d1) + b[v] * d2) + c)
    return out


def base_sums(levels4, X, Y, Z):
    """cf_mlp_base_sums: per variable the sums d1 d1, d1 d2, d2 d2, t d1,
    t d2, t t (levels4 = U^(n+1), U^n, U^(n-1), U^(n-2)); shape (5, 6)."""
    out = np.zeros((5, 6))
    for v in range(5):
        u = [_interior(x[v], X, Y, Z) for x in levels4]
        d1 = u[1] - u[2]
        d2 = (u[1] - 2.0 * u[2]) + u[3]
        t = u[0] - u[1]
        out[v] = [d1 @ d1, d1 @ d2, d2 @ d2, t @ d1, t @ d2, t @ t]
    return out
