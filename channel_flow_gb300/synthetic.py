"""Seeded synthetic channel states, grids and metrics (host set-up, numpy).

The reference reads its state from ``initial.bin`` and builds its grid and
metrics in ``Grid.cpp`` / ``Jacobian*.cpp``; no dataset is involved.  This
module produces the same kinds of arrays for the benchmark channels and the
parity tests: a laminar parabolic profile plus seeded uniform noise, on the
reference's single-rank layout ``[X_out+6][Y_out+4][Z_out+4]`` (z fastest).

Set-up only: nothing here is on the timed path.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

# Physical constants of the reference (prm.h:7-11, Viscous_terms.h:3-5)
K_GAMMA = 1.4
R_GAS = 287.0
E_PRECOND = 0.0001
CV = 717.5
MU_L = 0.0000185
PR_L = 0.72
F_BODY = 599.29876710   # prm.h:14
HIGH = 0.005            # prm.h:19, channel height 2h
Q0_BULK = 20.464969232814912   # prm.h:15, Driven_force's target bulk flux
T_WALL = 298.0592       # Y_boundary_condition.cpp:87
RHO_REF = 1.1842        # main.cpp:382 normalisation density


@dataclass(frozen=True)
class Grid:
    """Grid and constants of one run.  Index conventions follow the
    reference at one rank: interior cells i = 3..gend (gend = X_out+2),
    j = 2..ny (ny = Y_out+1), k = 2..nz (nz = Z_out+1)."""
    X_out: int
    Y_out: int
    Z_out: int
    deltaXI: float
    deltaET: float
    deltaZT: float
    K: float = K_GAMMA
    R: float = R_GAS
    e: float = E_PRECOND
    Cv: float = CV
    mu_L: float = MU_L
    Pr_L: float = PR_L
    f: float = F_BODY
    high: float = HIGH
    Q0: float = Q0_BULK

    @property
    def shape(self):
        return (self.X_out + 6, self.Y_out + 4, self.Z_out + 4)

    @property
    def gend(self):
        return self.X_out + 2

    @property
    def ny(self):
        return self.Y_out + 1

    @property
    def nz(self):
        return self.Z_out + 1

    @property
    def cells(self):
        return self.X_out * self.Y_out * self.Z_out

    @property
    def interior(self):
        """Slices of the interior cells i=3..gend, j=2..ny, k=2..nz."""
        return (slice(3, self.gend + 1), slice(2, self.ny + 1), slice(2, self.nz + 1))

    def with_(self, **kw):
        return replace(self, **kw)


def reference_grid(X_out, Y_out, Z_out, high=HIGH) -> Grid:
    """The reference's own domain 4*pi*h x 2h x 2*pi*h (Resolution.h:13-15)."""
    h = 0.5 * high
    return Grid(X_out, Y_out, Z_out, 4 * math.pi * h / X_out, 1.0 / Y_out, 2 * math.pi * h / Z_out,
                high=high)


def channel_grid(X_out, Y_out, Z_out, lx_over_h=2 * math.pi, lz_over_h=math.pi, high=HIGH) -> Grid:
    """Benchmark channels: 2*pi*h x 2h x pi*h with h = high/2."""
    h = 0.5 * high
    return Grid(X_out, Y_out, Z_out, lx_over_h * h / X_out, 1.0 / Y_out, lz_over_h * h / Z_out,
                high=high)


def _stretch(g: Grid, gamma: float, joff: float, j):
    """Analytic tanh stretching of the flat-wall channel (Jacobian.cpp:73-88):
    returns (etdy, ydet) at wall-normal index j with offset joff (1.5 cells,
    0.5 x/z faces, 1.0 y faces)."""
    hh = 0.5 * g.high
    arg = gamma * (1 - 2 * (j - joff) * g.deltaET)
    temp = hh * (1 - 1.0 / math.tanh(gamma) * np.tanh(arg))
    temp1 = (1 - temp / hh) * math.tanh(gamma)
    etdy = math.tanh(gamma) / (2 * hh * gamma * (1 - temp1 * temp1))
    temp2 = 1 / np.cosh(arg)
    ydet = g.high * gamma * 1.0 / math.tanh(gamma) * temp2 * temp2
    return etdy, ydet


METRIC_NAMES = ("xidx", "xidy", "xidz", "etdx", "etdy", "etdz", "ztdx", "ztdy", "ztdz")


def flat_metrics(g: Grid, gamma: float, where: str, perturb: float = 0.0, seed: int = 0):
    """J and the nine metric arrays of cell centres ('cell') or x/y/z faces
    ('u','v','w') for flat walls, evaluated at every index of the array.
    ``perturb`` > 0 adds seeded relative noise to all ten arrays and fills
    the zero cross terms with noise of that relative size, to exercise the
    general curvilinear code paths in parity tests."""
    joff = {"cell": 1.5, "u": 0.5, "v": 1.0, "w": 0.5}[where]
    X, Y, Z = g.shape
    j = np.arange(Y, dtype=np.float64)
    etdy1, ydet1 = _stretch(g, gamma, joff, j)
    out = {}
    out["J"] = np.broadcast_to((1.0 / ydet1)[None, :, None], g.shape).copy()
    for n in METRIC_NAMES:
        out[n] = np.zeros(g.shape)
    out["xidx"][:] = 1.0
    out["etdy"][:] = etdy1[None, :, None]
    out["ztdz"][:] = 1.0
    if perturb > 0:
        rng = np.random.default_rng(seed)
        scale = {"xi": 1.0, "et": float(np.max(etdy1)), "zt": 1.0}
        for n in METRIC_NAMES:
            a = out[n]
            a *= 1 + perturb * rng.uniform(-1, 1, g.shape)
            a += perturb * scale[n[:2]] * rng.uniform(-1, 1, g.shape)
        out["J"] *= 1 + perturb * rng.uniform(-1, 1, g.shape)
    return out


def y_points(g: Grid, gamma: float = 2.8):
    """Cell-centre wall distance with the ghost rule of Grid.cpp:49-108:
    tanh stretching (gamma 2.8 there), Y[1] = -Y[2], Y[nyy] = Y[ny] + 2 Y[2],
    one-deep z copies."""
    X, Y, Z = g.shape
    hh = 0.5 * g.high
    yp = np.zeros(Y)
    for jj in range(2, g.ny + 1):
        yp[jj] = hh * (1 - 1.0 / math.tanh(gamma) * math.tanh(gamma * (1 - 2 * (jj - 1.5) * g.deltaET)))
    yp[1] = -yp[2]
    yp[g.ny + 1] = yp[g.ny] + 2 * yp[2]
    yp[0] = 2 * yp[1] - yp[2]
    yp[g.ny + 2] = 2 * yp[g.ny + 1] - yp[g.ny]
    return np.broadcast_to(yp[None, :, None], g.shape).copy()


def channel_state(g: Grid, J, seed: int = 0, mach: float = 0.5, noise: float = 0.05,
                  jitter: float = 0.01, rho_b: float = RHO_REF, gamma: float = 1.5,
                  wall_damped: bool = False, yy=None):
    """Seeded channel state U/J = (rho, rho u, rho v, rho w, E)/J on every
    cell of the array: laminar parabola u = 1.5 U_b (1 - eta^2) plus uniform
    +-noise*U_b on u, v, w, and +-jitter relative noise on rho and T (the
    unguarded limiter ratios need distinct neighbours, so exact ties are
    avoided).  U_b = mach * sqrt(K R T_wall).  ``wall_damped``: the
    velocity noise is scaled by the parabola's shape 1 - eta^2, so it
    vanishes at the no-slip walls (the noise keeps its +-noise*U_b
    amplitude on the centre line).  ``yy``: the stretched wall-normal
    position per j (0 .. 2) to use instead of evaluating the tanh map; with
    it the state is built from correctly rounded operations only, so it is
    the same on every platform."""
    rng = np.random.default_rng(seed)
    X, Y, Z = g.shape
    ub = mach * math.sqrt(g.K * g.R * T_WALL)
    j = np.arange(Y, dtype=np.float64)
    eta = np.clip(1 - 2 * (j - 1.5) * g.deltaET, -1.0, 1.0)          # +1 bottom wall .. -1 top
    # position in the stretched coordinate mapped back to [-1, 1]
    if yy is None:
        yy = 1 - 1.0 / math.tanh(gamma) * np.tanh(gamma * eta)        # 0 .. 2
    yy = np.asarray(yy, dtype=np.float64)
    prof = 1.5 * ub * (1 - (yy - 1) ** 2)
    amp = noise * ub * ((1 - (yy - 1) ** 2)[None, :, None] if wall_damped else 1.0)
    rho = rho_b * (1 + jitter * rng.uniform(-1, 1, g.shape))
    T = T_WALL * (1 + jitter * rng.uniform(-1, 1, g.shape))
    u = prof[None, :, None] + amp * rng.uniform(-1, 1, g.shape)
    v = amp * rng.uniform(-1, 1, g.shape)
    w = amp * rng.uniform(-1, 1, g.shape)
    p = rho * g.R * T
    E = p / (g.K - 1) + 0.5 * rho * (u * u + v * v + w * w)
    return [np.ascontiguousarray(x / J) for x in (rho, rho * u, rho * v, rho * w, E)]


def bulk_velocity(g: Grid, mach: float = 0.5):
    return mach * math.sqrt(g.K * g.R * T_WALL)


def channel_physics(g: Grid, mach: float, re_bulk: float, rho_b: float = RHO_REF) -> Grid:
    """The grid with the viscosity and body force of a channel at bulk Mach
    number ``mach`` and bulk Reynolds number ``re_bulk`` = rho_b U_b (2h) / mu
    (length: the full channel height 2h = ``high``), U_b = mach *
    sqrt(K R T_wall): mu = rho_b U_b 2h / Re_b; the body force f = 3 mu U_b /
    h^2 holds the laminar parabola in balance with the wall shear (the
    reference keeps f constant, prm.h:14); Q0 = rho_b U_b is Driven_force's
    target bulk flux.  The other constants (K, R, Cv, Pr_L, e) stay the
    reference's."""
    ub = bulk_velocity(g, mach)
    h = 0.5 * g.high
    mu = rho_b * ub * g.high / re_bulk
    return g.with_(mu_L=mu, f=3.0 * mu * ub / (h * h), Q0=rho_b * ub)


def time_step(g: Grid, mach: float, h_over_ub: float = 0.005) -> float:
    """Physical time step h_over_ub * h / U_b (the configurations' 0.005 h/U_b)."""
    return h_over_ub * 0.5 * g.high / bulk_velocity(g, mach)
