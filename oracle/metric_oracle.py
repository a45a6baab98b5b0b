"""CPU oracle (test infrastructure) of the wavy-wall metric generator
(channel_flow_gb300/csrc/cf_metrics.cu): the mapping, its derivatives in the
analytic and conservative forms, the inverse and Y_point, restated in numpy
float64 on the same index positions.  With amplitude 0 and the analytic form
the mapping is the reference's flat channel (Jacobian.cpp:65-99,
Jacobian_u.cpp, Jacobian_v.cpp, Jacobian_w.cpp, Grid.cpp:49-108).
"""
from __future__ import annotations

import math

import numpy as np

# index offsets of the positions: xi = (i - CI) dXI, eta = (j - CJ) dET
CI = {"cell": 1.5, "u": 1.0, "v": 0.5, "w": 0.5}
CJ = {"cell": 1.5, "u": 0.5, "v": 1.0, "w": 0.5}


def _wall(A, kw, xi):
    return A * np.sin(kw * xi)


def _y0(high, g, eta):
    return 0.5 * high * (1.0 - np.tanh(g * (1.0 - 2.0 * eta)) / math.tanh(g))


def ymap(high, A, wavelength, g, xi, eta):
    kw = 2.0 * math.pi / wavelength
    yw = _wall(A, kw, xi)
    return yw + _y0(high, g, eta) * (1.0 - yw / high)


def metrics(shape, dXI, dET, high, A, wavelength, g, conservative, where):
    """[J, xidx, xidy, xidz, etdx, etdy, etdz, ztdx, ztdy, ztdz] on every
    index of an array of `shape`."""
    X, Y, Z = shape
    i = np.arange(X, dtype=np.float64)[:, None]
    j = np.arange(Y, dtype=np.float64)[None, :]
    xi = (i - CI[where]) * dXI
    eta = (j - CJ[where]) * dET
    kw = 2.0 * math.pi / wavelength
    if conservative:
        y_xi = (ymap(high, A, wavelength, g, xi + 0.5 * dXI, eta) - ymap(high, A, wavelength, g, xi - 0.5 * dXI, eta)) / dXI
        y_eta = (ymap(high, A, wavelength, g, xi, eta + 0.5 * dET) - ymap(high, A, wavelength, g, xi, eta - 0.5 * dET)) / dET
    else:
        s = 1.0 / np.cosh(g * (1.0 - 2.0 * eta))
        ydet0 = high * g * 1. / math.tanh(g) * s * s
        yw = _wall(A, kw, xi)
        y_xi = A * kw * np.cos(kw * xi) * (1.0 - _y0(high, g, eta) / high)
        y_eta = ydet0 * (1.0 - yw / high)
    y_xi, y_eta = np.broadcast_arrays(y_xi, y_eta)
    # forward matrix [[1, 0, 0], [y_xi, y_eta, 0], [0, 0, 1]] and its inverse
    Jq = 1.0 / y_eta
    zeros = np.zeros_like(Jq)
    ones = np.ones_like(Jq)
    m = [y_eta * Jq, zeros, zeros, -y_xi * Jq, Jq, zeros, zeros, zeros, y_eta * Jq]
    out = [Jq] + m
    return [np.ascontiguousarray(np.broadcast_to(a[:, :, None], shape)) for a in out]


def y_point(shape, dXI, dET, high, A, wavelength, g):
    X, Y, Z = shape
    ny = Y - 3
    i = np.arange(X, dtype=np.float64)
    xi = (i - 1.5) * dXI
    kw = 2.0 * math.pi / wavelength
    yw = _wall(A, kw, xi)
    yp = np.zeros((X, Y))
    for jj in range(Y):
        yp[:, jj] = ymap(high, A, wavelength, g, xi, (jj - 1.5) * dET)
    y2, yny = yp[:, 2].copy(), yp[:, ny].copy()
    y1 = 2.0 * yw - y2
    ynyy = yny + 2.0 * (y2 - yw)
    yp[:, 1] = y1
    yp[:, ny + 1] = ynyy
    yp[:, 0] = 2.0 * y1 - y2
    yp[:, ny + 2] = 2.0 * ynyy - yny
    return np.ascontiguousarray(np.broadcast_to(yp[:, :, None], shape))


def divergence_of_constant_flux(fu, fv, fw, dXI, dET, dZT, direction):
    """Finite-volume divergence, at the interior cells, of the constant
    unit flux in Cartesian direction `direction` (0: x, 1: y, 2: z) through
    the faces, with the face arrays in the reference indexing: the
    contravariant area of a face set is (metric of that face's coordinate,
    component `direction`) / J_face (cf. Dual_time_stepping.cpp:399-401)."""
    X, Y, Z = fu[0].shape
    ax = fu[1 + direction] / fu[0]           # xi_{x,y,z} / J_u
    ay = fv[4 + direction] / fv[0]           # eta_{x,y,z} / J_v
    az = fw[7 + direction] / fw[0]           # zeta_{x,y,z} / J_w
    i = slice(3, X - 3)
    j = slice(2, Y - 2)
    k = slice(2, Z - 2)
    im, jm, km = slice(2, X - 4), slice(1, Y - 3), slice(1, Z - 3)
    # cell (i, j, k): x faces [i][j-1][k-1] and [i-1][j-1][k-1], and so on
    dx = (ax[i, jm, km] - ax[im, jm, km]) / dXI
    dy = (ay[im, j, km] - ay[im, jm, km]) / dET
    dz = (az[im, jm, k] - az[im, jm, km]) / dZT
    return dx + dy + dz
