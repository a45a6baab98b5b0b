"""Seeded per-routine cases shared by the parity tests.

Each ``*_case`` function returns the list of field arrays in the reference
routine's argument order (main.h), filled with a seeded channel state,
perturbed curvilinear metrics and random (but identical) initial contents of
the output and scratch arrays, so that two implementations handed copies of
the same list can be compared array by array.

Inputs are built from the seeded PCG64 generator and IEEE-exact arithmetic
(+, -, *, /, sqrt) only, so every machine regenerates them bit for bit; the
golden fixtures can therefore store hashes of the reference's outputs.
"""
from __future__ import annotations

import hashlib
import math

import numpy as np

from channel_flow_gb300 import synthetic as syn

# test grids (X_out, Y_out, Z_out): the second one has Z_out > Y_out + 1 so
# that Flux_Z_limiter takes its 3rd-order branch for k >= ny
GRIDS = [(12, 10, 8), (8, 6, 12), (16, 12, 10)]
GOLDEN_GRID = (6, 6, 8)
DELTA_T = 0.00000005                       # main.cpp:53
FILTER_ARGS = (0.007, 1.0, 0.0)            # Roe_criterion, E_high, E_low (main.cpp:55-57)
METRIC_NAMES = syn.METRIC_NAMES


def grid(dims):
    return syn.reference_grid(*dims)


def _rand_like(g, rng, scale=1.0):
    return scale * rng.uniform(-1, 1, g.shape)


def _eta(g, joff):
    """normalised wall-normal position of row j (0 at the lower wall)"""
    j = np.arange(g.shape[1], dtype=np.float64)
    return (j - joff) * g.deltaET


def metric_set(g, where, seed, perturb=0.02):
    """J and nine metrics of a stretched flat channel (arithmetic stand-in for
    the tanh stretching: dy/deta = high*(0.25 + 4.5 eta (1 - eta))), plus
    seeded relative noise on all ten arrays and noise-filled cross terms."""
    joff = {"cell": 1.5, "u": 0.5, "v": 1.0, "w": 0.5}[where]
    eta = _eta(g, joff)
    ydet = g.high * (0.25 + 4.5 * eta * (1 - eta))
    etdy1 = 1.0 / ydet
    rng = np.random.default_rng(seed)
    J = np.broadcast_to((1.0 / ydet)[None, :, None], g.shape).copy()
    m = {n: np.zeros(g.shape) for n in METRIC_NAMES}
    m["xidx"][:] = 1.0
    m["etdy"][:] = etdy1[None, :, None]
    m["ztdz"][:] = 1.0
    if perturb > 0:
        scale = {"xi": 1.0, "et": float(np.max(etdy1)), "zt": 1.0}
        for n in METRIC_NAMES:
            m[n] *= 1 + perturb * rng.uniform(-1, 1, g.shape)
            m[n] += perturb * scale[n[:2]] * rng.uniform(-1, 1, g.shape)
        J *= 1 + perturb * rng.uniform(-1, 1, g.shape)
    return [J] + [m[n] for n in METRIC_NAMES]


def y_points(g):
    """monotone wall distance with the ghost rule of Grid.cpp:86-108"""
    eta = _eta(g, 1.5)
    yp = 0.5 * g.high * eta * eta * (3 - 2 * eta) + 0.01 * g.high * eta
    ny = g.ny
    yp[1] = -yp[2]
    yp[ny + 1] = yp[ny] + 2 * yp[2]
    yp[0] = 2 * yp[1] - yp[2]
    yp[ny + 2] = 2 * yp[ny + 1] - yp[ny]
    return np.broadcast_to(yp[None, :, None], g.shape).copy()


def state(g, seed, mach=0.5, noise=0.05, jitter=0.01):
    """seeded conserved state U/J and the cell Jacobian J"""
    J = metric_set(g, "cell", seed + 1000)[0]
    rng = np.random.default_rng(seed)
    ub = mach * math.sqrt(g.K * g.R * syn.T_WALL)
    eta = np.clip(_eta(g, 1.5), 0.0, 1.0)
    prof = 1.5 * ub * (1 - (2 * eta - 1) ** 2)
    rho = syn.RHO_REF * (1 + jitter * rng.uniform(-1, 1, g.shape))
    T = syn.T_WALL * (1 + jitter * rng.uniform(-1, 1, g.shape))
    u = prof[None, :, None] + noise * ub * rng.uniform(-1, 1, g.shape)
    v = noise * ub * rng.uniform(-1, 1, g.shape)
    w = noise * ub * rng.uniform(-1, 1, g.shape)
    p = rho * g.R * T
    E = p / (g.K - 1) + 0.5 * rho * (u * u + v * v + w * w)
    return [np.ascontiguousarray(x / J) for x in (rho, rho * u, rho * v, rho * w, E)], J


def copy_case(arrays):
    return [np.array(a, copy=True) for a in arrays]


# --------------------------------------------------------------------------
# per-routine argument lists

def bc_case(g, seed=0):
    """6 arrays: U1_..U5_, J"""
    U, J = state(g, seed)
    return U + [J]


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
    return U + [y_points(g)] + [_rand_like(g, rng) for _ in range(3)] + [J]


def dt_case(g, seed=0, nslots=64):
    """Dual-time / RK3 signature (main.h:653): U1_..5, U1..5, U1q..5, J,
    9 cell metrics, inFx/y/z 1..5, vF2..5, MR1..5 [, NR1..5, NL1..5,
    Residual1..5].  U and Uq are the state with 1e-6 relative noise, the
    fluxes of realistic magnitude with 5 % noise."""
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


def jacobian_case(g, which, seed=0):
    """10 face arrays (J_f + 9), random initial content; Jacobian_v also
    gets J + 9 cell metrics"""
    rng = np.random.default_rng(seed + 17)
    out = [rng.uniform(0.5, 1.5, g.shape) for _ in range(10)]
    if which == "v":
        out += metric_set(g, "cell", seed + 23)
    return out


# --------------------------------------------------------------------------
# which arrays each routine writes (slots compared by the tests)

FLUX_OUT = list(range(26, 31))
VISC_OUT = [5, 6, 7, 8] + [55, 56, 57, 58, 65, 66, 67, 68, 75, 76, 77, 78]
FILTER_OUT = [6, 7, 8]
RK3_OUT = list(range(0, 5)) + list(range(44, 49))
LU_OUT = list(range(0, 5)) + list(range(44, 64))
BC_OUT = list(range(0, 5))
JAC_OUT = list(range(0, 10))


def ylim_undefined_mask(g, slot):
    """Entries of Flux_Y_limiter's outputs that depend on the reference's
    uninitialised jL/jR (Flux_Y_limiter.cpp:120-232): face fluxes at faces
    j = 2, ny-2, ny-1 (all five variables) and at the wall faces 1 and ny
    (the normal-momentum flux, the only one not set to zero there)."""
    m = np.zeros(g.shape, dtype=bool)
    ny = g.ny
    if slot in FLUX_OUT:
        rows = [2, ny - 2, ny - 1] + ([1, ny] if slot == 28 else [])
        for j in rows:
            m[:, j, :] = True
    return m


def digest(a, mask=None):
    a = np.array(a, dtype=np.float64, copy=True)
    if mask is not None:
        a[mask] = 0.0
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def statistic_case(g, seed=0):
    """27 arrays in Statistic's order: U1_..5, J, J_v + 9 face metrics,
    MR1..5, ML1..5 (scratch the routine overwrites), EpY."""
    rng = np.random.default_rng(seed + 13)
    U, J = state(g, seed)
    fm = metric_set(g, "v", seed + 17)
    MR = [_rand_like(g, rng) for _ in range(5)]
    ML = [_rand_like(g, rng) for _ in range(5)]
    Ep = rng.choice(np.asarray([0.0, 1.0]), size=g.shape)
    return U + [J] + fm + MR + ML + [Ep]


def restart_case(g, seed=0):
    """11 arrays in Output's order: U1..U5, U1q..U5q, J."""
    U, J = state(g, seed)
    Uq, _ = state(g, seed + 1)
    return U + Uq + [J]


def step_case(g, seed=0):
    """The fields of one physical step (cf_fields), as numpy arrays: the
    state at three time levels, cell and face metrics, Y_point and zeroed
    outputs and scratch."""
    rng = np.random.default_rng(seed + 29)
    U_, J = state(g, seed)
    U = [x * (1 + 1e-6 * rng.uniform(-1, 1, g.shape)) for x in U_]
    Uq = [x * (1 + 1e-6 * rng.uniform(-1, 1, g.shape)) for x in U_]
    z = lambda: np.zeros(g.shape)
    faces = [metric_set(g, w, seed + s) for w, s in (("u", 31), ("v", 41), ("w", 51))]
    return {"U_": U_, "U": U, "Uq": Uq, "J": J, "Y_point": y_points(g),
            "cell_metric": metric_set(g, "cell", seed + 1000)[1:],
            "face_J": [f[0] for f in faces], "face_metric": [f[1:] for f in faces],
            "Ep": [z() for _ in range(3)], "inF": [[z() for _ in range(5)] for _ in range(3)],
            "vF": [z() for _ in range(4)], "LL": [z() for _ in range(4)], "ML": [z() for _ in range(4)],
            "MR": [z() for _ in range(5)], "NR": [z() for _ in range(5)], "NL": [z() for _ in range(5)],
            "Residual": [z() for _ in range(5)]}


def port_step(port, g, f, deltaT, max_iterations, tolerance, E, crit=(0.007, 1.0, 0.0), scheme="reference"):
    """The same physical step on the C oracle: the loop of main.cpp:143-480
    with Filter and the limited fluxes (face-state scaling ``scheme``); f is
    modified in place, E (running maxima) too.  Returns (iterations, er, Q)."""
    from oracle.cforacle import hyperplane_buffers
    U_, J = f["U_"], f["J"]
    s10 = [np.zeros(g.shape) for _ in range(10)]
    Nijk, ijk = port.Hyperplane(g)
    visc_scratch = [np.zeros(g.shape) for _ in range(30)]
    it = 0
    while True:
        it += 1
        port.x_periodic(g, U_)
        port.Y_boundary_condition(g, U_ + [J])
        port.Z_boundary_condition(g, U_ + [J])
        port.Filter(g, *crit, U_ + [f["Y_point"]] + f["Ep"] + [J])
        for d, name in enumerate(("Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter")):
            port.flux(name, g, U_ + s10 + [J, f["face_J"][d]] + f["face_metric"][d] + f["inF"][d] + [f["Ep"][d]],
                      scheme=scheme)
        visc = U_ + f["vF"] + [J] + f["cell_metric"]
        for d in range(3):
            visc += [f["face_J"][d]] + f["face_metric"][d]
        # LR, LL, MR, ML, NR, NL scratch blocks; LL2..5, ML2..5 and NL2..5 are the
        # driver's shared arrays
        LR, LL1, MR_, ML1, NR_ = visc_scratch[0:5], visc_scratch[5], visc_scratch[10:15], visc_scratch[15], \
            visc_scratch[20:25]
        visc += LR + [LL1] + f["LL"] + MR_ + [ML1] + f["ML"] + NR_ + f["NL"]
        port.Viscous_terms(g, visc)
        dts = U_ + f["U"] + f["Uq"] + [J] + f["cell_metric"] + f["inF"][0] + f["inF"][1] + f["inF"][2] + \
            f["vF"] + f["MR"] + f["NR"] + f["NL"] + f["Residual"]
        er = port.Dual_time_stepping(g, deltaT, Nijk, ijk, dts)
        for n in range(5):
            E[n] = max(E[n], er[n])
            er[n] = er[n] / E[n]
        if (er[0] < tolerance and er[1] < tolerance and er[2] < tolerance and er[3] < tolerance) \
                or it >= max_iterations:
            break
    Q = port.Driven_force(g, f["U"][1], J)
    ix = g.interior
    for n in range(5):
        f["Uq"][n][ix] = f["U"][n][ix]
        f["U"][n][ix] = f["U_"][n][ix]
    return it, np.asarray(er), Q


def channel_step_case(g, gamma=2.0, seed=0, mach=0.5, port=None):
    """The fields of a physical step on the benchmark channel (synthetic.py:
    tanh-stretched flat walls, laminar parabola with wall-damped +-5 % velocity
    noise, +-1 % rho and T jitter), as numpy arrays, U = U_ = Uq; face
    metrics from the oracle's Jacobian_u/v/w."""
    cm = syn.flat_metrics(g, gamma, "cell")
    J = cm["J"]
    U = syn.channel_state(g, J, seed=seed, mach=mach, noise=0.05, jitter=0.01, gamma=gamma, wall_damped=True)
    if port is None:
        from oracle.cforacle import Port
        port = Port()
    faces = []
    for w in ("u", "v", "w"):
        arrs = [np.zeros(g.shape) for _ in range(10)]
        extra = [J] + [cm[n] for n in syn.METRIC_NAMES] if w == "v" else []
        port.Jacobian_face(w, g, gamma, arrs + extra)
        faces.append(arrs)
    z = lambda: np.zeros(g.shape)
    return {"U_": [u.copy() for u in U], "U": [u.copy() for u in U], "Uq": [u.copy() for u in U], "J": J,
            "Y_point": syn.y_points(g, gamma=gamma), "cell_metric": [cm[n] for n in syn.METRIC_NAMES],
            "face_J": [f[0] for f in faces], "face_metric": [f[1:] for f in faces],
            "Ep": [z() for _ in range(3)], "inF": [[z() for _ in range(5)] for _ in range(3)],
            "vF": [z() for _ in range(4)], "LL": [z() for _ in range(4)], "ML": [z() for _ in range(4)],
            "MR": [z() for _ in range(5)], "NR": [z() for _ in range(5)], "NL": [z() for _ in range(5)],
            "Residual": [z() for _ in range(5)]}


def config0_case():
    """The 64^3 plain-FP64 channel schedule of tests/golden/config0_64_run.json
    (made by tests/golden/make_config0_run.py): (grid, fields, fixture).
    The static inputs come from the stored arrays and the state from the
    stored wall-normal profile, so every host builds the same bits."""
    import bz2
    import json
    from pathlib import Path
    here = Path(__file__).resolve().parent / "golden"
    meta = json.loads((here / "config0_64_run.json").read_text())
    g = syn.channel_physics(syn.channel_grid(*meta["dims"]), meta["mach"], meta["re_bulk"])
    raw = bz2.decompress((here / "config0_64_static.bz2").read_bytes())
    n = int(np.prod(g.shape))
    st = np.frombuffer(raw, dtype=np.float64).reshape(len(meta["static_names"]), *g.shape).copy()
    J = st[0]
    yy = np.array([float.fromhex(x) for x in meta["yy"]])
    U = syn.channel_state(g, J, seed=meta["seed"], mach=meta["mach"], noise=0.05, jitter=0.01, gamma=meta["gamma"],
                          wall_damped=True, yy=yy)
    assert st.shape[0] * n * 8 == len(raw)
    z = lambda: np.zeros(g.shape)
    f = {"U_": [u.copy() for u in U], "U": [u.copy() for u in U], "Uq": [u.copy() for u in U], "J": J,
         "Y_point": st[1], "cell_metric": list(st[2:11]),
         "face_J": [st[11 + 10 * d] for d in range(3)],
         "face_metric": [list(st[12 + 10 * d:21 + 10 * d]) for d in range(3)],
         "Ep": [z() for _ in range(3)], "inF": [[z() for _ in range(5)] for _ in range(3)],
         "vF": [z() for _ in range(4)], "LL": [z() for _ in range(4)], "ML": [z() for _ in range(4)],
         "MR": [z() for _ in range(5)], "NR": [z() for _ in range(5)], "NL": [z() for _ in range(5)],
         "Residual": [z() for _ in range(5)]}
    meta["deltaT_value"] = float.fromhex(meta["deltaT"])
    return g, f, meta


def state_digest(fields, to_numpy=np.asarray):
    """SHA-256 over U_, U and Uq (five arrays each, in order)."""
    h = hashlib.sha256()
    for key in ("U_", "U", "Uq"):
        for a in fields[key]:
            h.update(np.ascontiguousarray(to_numpy(a)).tobytes())
    return h.hexdigest()
