"""Seeded per-routine cases shared by the parity tests.

Each ``*_case`` function returns the list of field arrays in the reference
routine's argument order (main.h), filled with a seeded channel state,
perturbed curvilinear metrics and random (but identical) initial contents of
the output and scratch arrays, so that two implementations handed copies of
the same list can be compared array by array.
"""
from __future__ import annotations

import numpy as np

from channel_flow_gb300 import synthetic as syn

# test grids (X_out, Y_out, Z_out): the second one has Z_out > Y_out + 1 so
# that Flux_Z_limiter takes its 3rd-order branch for k >= ny
GRIDS = [(12, 10, 8), (8, 6, 12), (16, 12, 10)]


def grid(dims):
    return syn.reference_grid(*dims)


def _rand_like(g, rng, scale=1.0):
    return scale * rng.uniform(-1, 1, g.shape)


def metric_set(g, where, seed, perturb=0.02):
    m = syn.flat_metrics(g, 1.5, where, perturb=perturb, seed=seed)
    return [m["J"]] + [m[n] for n in syn.METRIC_NAMES]


def state(g, seed):
    J = syn.flat_metrics(g, 1.5, "cell", perturb=0.02, seed=seed + 1000)["J"]
    return syn.channel_state(g, J, seed=seed), J


def flux_case(g, direction, seed=0, ep_values=(0.0, 0.5, 1.0)):
    """32 arrays: U1_..5, MR1..5, ML1..5, J, J_f, 9 face metrics, inF1..5, Ep."""
    rng = np.random.default_rng(seed + 7)
    U, J = state(g, seed)
    fm = metric_set(g, {"x": "u", "y": "v", "z": "w"}[direction], seed + 11)
    MR = [_rand_like(g, rng) for _ in range(5)]
    ML = [_rand_like(g, rng) for _ in range(5)]
    F = [_rand_like(g, rng) for _ in range(5)]
    Ep = rng.choice(np.asarray(ep_values, dtype=np.float64), size=g.shape)
    return U + MR + ML + [J] + fm + F + [Ep]


def copy_case(arrays):
    return [np.array(a, copy=True) for a in arrays]


def viscous_case(g, seed=0):
    """79 arrays in Viscous_terms' order: U1_..5, vF2..5, J, 9 cell metrics,
    J_u + 9, J_v + 9, J_w + 9, then the scratch LR, LL, MR, ML, NR, NL."""
    rng = np.random.default_rng(seed + 5)
    U, J = state(g, seed)
    cm = metric_set(g, "cell", seed + 21)[1:]
    out = U + [_rand_like(g, rng) for _ in range(4)] + [J] + cm
    for w, s in (("u", 31), ("v", 41), ("w", 51)):
        out += metric_set(g, w, seed + s)
    out += [_rand_like(g, rng) for _ in range(30)]
    return out


def filter_case(g, seed=0):
    """10 arrays in Filter's order: U1_..5, Y_point, EpX, EpY, EpZ, J."""
    rng = np.random.default_rng(seed + 9)
    U, J = state(g, seed)
    Yp = syn.y_points(g)
    return U + [Yp] + [_rand_like(g, rng) for _ in range(3)] + [J]


FILTER_ARGS = (0.007, 1.0, 0.0)   # Roe_criterion, E_high, E_low (main.cpp:55-57)


DELTA_T = 0.00000005   # main.cpp:53


def dt_case(g, seed=0, nslots=64):
    """Dual-time / RK3 signature (main.h:653): U1_..5, U1..5, U1q..5, J,
    9 cell metrics, inFx/y/z 1..5, vF2..5, MR1..5 [, NR1..5, NL1..5,
    Residual1..5].  U and Uq are the state with 1e-6 relative noise, the
    fluxes O(1) with 5 % noise."""
    rng = np.random.default_rng(seed + 13)
    U_, J = state(g, seed)
    U = [x * (1 + 1e-6 * rng.uniform(-1, 1, g.shape)) for x in U_]
    Uq = [x * (1 + 1e-6 * rng.uniform(-1, 1, g.shape)) for x in U_]
    cm = metric_set(g, "cell", seed + 21)[1:]
    F = [np.ascontiguousarray((1.0 + 0.05 * rng.uniform(-1, 1, g.shape)) * s)
         for s in (1, 100, 1, 1, 1e5) for _ in range(3)]
    Fx, Fy, Fz = F[0::3], F[1::3], F[2::3]
    vF = [1e-3 * rng.uniform(-1, 1, g.shape) for _ in range(4)]
    out = U_ + U + Uq + [J] + cm + Fx + Fy + Fz + vF
    out += [_rand_like(g, rng) for _ in range(nslots - len(out))]
    return out
