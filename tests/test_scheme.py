"""The consistent face-state scaling of the limited fluxes, on the C oracle
(CPU).

The reference's Flux_Y_limiter scales its near-wall states inconsistently
(density by the cell J with an unscaled slope, the other variables by
never-set jL/jR) and its Flux_Z_limiter carries 1/60 of the state on
interior faces with a downwind left slope.  Assembled into the limited
dual-time loop, that diverges on channel states at the configurations'
time step 0.005 h/U_b.  The consistent scheme changes those states only;
these tests pin where it differs from the reference's, that its states are
bounded by their neighbours (what the reference's are not), and that the
assembled loop it gives stays bounded where the reference's diverges.
"""
import numpy as np
import pytest

import cases
import routines
from channel_flow_gb300 import synthetic as syn

ML, MR = 10, 5          # first slots of the ML1..5 and MR1..5 scratch in the flux argument list


def _channel_flux_case(g, direction, seed=4, gamma=2.0):
    """A flux argument list on the benchmark channel (J varies in y only,
    face metrics from the oracle's Jacobian routines)."""
    from oracle.cforacle import Port
    port = Port()
    cm = syn.flat_metrics(g, gamma, "cell")
    J = cm["J"]
    U = syn.channel_state(g, J, seed=seed, gamma=gamma)
    where = {"x": "u", "y": "v", "z": "w"}[direction]
    face = [np.zeros(g.shape) for _ in range(10)]
    extra = [J] + [cm[n] for n in syn.METRIC_NAMES] if where == "v" else []
    port.Jacobian_face(where, g, gamma, face + extra)
    z = lambda: np.zeros(g.shape)
    return U + [z() for _ in range(10)] + [J] + face + [z() for _ in range(5)] + [np.ones(g.shape)]


@pytest.mark.parametrize("dims", cases.GRIDS)
def test_consistent_y_differs_only_next_to_walls(dims, port):
    """Flux_Y_limiter: faces j = 3..ny-3 (both states from interior cells)
    are the reference's bit for bit; faces 1, 2, ny-2, ny-1, ny change."""
    r = routines.BY_NAME["Flux_Y_limiter"]
    g = cases.grid(dims)
    a = r.build(g, 7)
    ref, con = cases.copy_case(a), cases.copy_case(a)
    routines.run_cpu(port, r, g, ref)
    routines.run_cpu(port, r, g, con, scheme="consistent")
    ny = g.ny
    inner = slice(3, ny - 2)
    for i in r.outputs:
        assert np.array_equal(ref[i][:, inner, :], con[i][:, inner, :]), i
    changed = {j for i in r.outputs for j in (1, 2, ny - 2, ny - 1, ny)
               if not np.array_equal(ref[i][2:g.gend, j, 1:g.nz], con[i][2:g.gend, j, 1:g.nz])}
    assert changed == {1, 2, ny - 2, ny - 1, ny}, changed


def _between(x, a, b, rtol=1e-6):
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    tol = rtol * np.maximum(np.abs(lo), np.abs(hi))
    return (x >= lo - tol) & (x <= hi + tol)


def test_consistent_states_bounded_by_neighbours(port):
    """Every state the consistent scheme reconstructs lies between the
    conserved values of the two cells of its face: in Flux_Y_limiter's
    near-wall rows and on every interior z face.  The reference's z states
    (1/60 of the state) and near-wall y states are not."""
    g = syn.channel_grid(12, 16, 14)
    ny, nz, gend = g.ny, g.nz, g.gend
    for direction, name in (("y", "Flux_Y_limiter"), ("z", "Flux_Z_limiter")):
        a = _channel_flux_case(g, direction)
        J = a[15]
        out = {}
        for scheme in ("reference", "consistent"):
            b = cases.copy_case(a)
            port.flux(name, g, b, scheme=scheme)
            out[scheme] = b
        ok = {}
        for scheme, b in out.items():
            good = True
            for n in range(5):
                q = a[n] * J                                    # conserved values of the cells
                if direction == "y":
                    # left state of cell j at face j (cells j, j+1), right state of
                    # cell j at face j-1 (cells j-1, j), for the near-wall cells 2, ny-1
                    for j in (2, ny - 1):
                        i_, k_ = slice(3, gend), slice(2, nz)
                        mL = b[ML + n][2:gend - 1, j, 1:nz - 1]
                        mR = b[MR + n][2:gend - 1, j - 1, 1:nz - 1]
                        good &= bool(np.all(_between(mL, q[i_, j, k_], q[i_, j + 1, k_])))
                        good &= bool(np.all(_between(mR, q[i_, j - 1, k_], q[i_, j, k_])))
                else:
                    # interior z faces k = 3..nz-2: left state from cell k, right from k+1
                    i_, j_ = slice(3, gend), slice(2, ny)
                    mL = b[ML + n][2:gend - 1, 1:ny - 1, 3:nz - 1]
                    mR = b[MR + n][2:gend - 1, 1:ny - 1, 3:nz - 1]
                    good &= bool(np.all(_between(mL, q[i_, j_, 3:nz - 1], q[i_, j_, 4:nz])))
                    good &= bool(np.all(_between(mR, q[i_, j_, 3:nz - 1], q[i_, j_, 4:nz])))
            ok[scheme] = good
        assert ok == {"reference": False, "consistent": True}, (direction, ok)


def _loop(port, g, f, scheme, steps, dt):
    E = [0.0] * 5
    rho_b = syn.RHO_REF
    worst = 0.0
    for _ in range(steps):
        cases.port_step(port, g, f, dt, 10, 1e-12, E, scheme=scheme)
        rho = f["U"][0][g.interior] * f["J"][g.interior]
        if not np.all(np.isfinite(rho)) or np.min(rho) <= 0:
            return float("inf")
        worst = max(worst, float(np.max(np.abs(rho / rho_b - 1))))
    return worst


def test_assembled_limited_loop(port):
    """Three physical steps of 10 sub-iterations of the limited loop with
    the Filter (x halo, ghosts, Filter, limited fluxes, viscous terms,
    Dual_time_stepping) at Mach 0.5, Re_b 2800 and dt = 0.005 h/U_b on a
    16^3 channel: the reference's scaling leaves the physical range
    (non-positive or non-finite density) while the consistent scheme keeps
    the density within 10 % of the bulk value."""
    g = syn.channel_physics(syn.channel_grid(16, 16, 16), 0.5, 2800)
    dt = syn.time_step(g, 0.5)
    worst = {}
    for scheme in ("reference", "consistent"):
        f = cases.channel_step_case(g, port=port)
        worst[scheme] = _loop(port, g, f, scheme, 3, dt)
    assert worst["reference"] == float("inf") or worst["reference"] > 0.5, worst
    assert worst["consistent"] < 0.1, worst
