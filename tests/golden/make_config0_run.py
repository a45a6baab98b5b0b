"""Fixtures of the plain-FP64 channel schedule on 64^3 cells, run on the C oracle.

The schedule: periodic channel 64 x 64 x 64 cells, 2 pi h x 2h x pi h, tanh
stretching 2.0, Mach_bulk 0.5, Re_bulk 2800 (on 2h), laminar parabola with
wall-damped +-5 % velocity noise and +-1 % rho / T jitter (seed 0);
limited MUSCL-5 + Roe with the consistent face-state scaling, viscous
terms, the Filter at every sub-iteration, dual time with
deltaT = 0.005 h / U_b, exactly 10 LU-SGS sub-iterations per step
(main.cpp:380-462 with the tolerance test never met), 100 steps.  The
reference's own face-state scaling makes this schedule diverge in its first
step (the oracle, bit-identical to the reference, gives NaN there), so the
consistent one is used.

Outputs (beside this script):
* ``config0_64_static.bz2``: the static inputs - J, Y_point, the nine cell
  metrics and the three face sets (J_f + nine metrics each) - as raw
  float64 arrays in the order of ``static_names`` in the JSON file.  They
  hold tanh/cosh values from this machine's libm; storing them makes the
  GPU run start from the same bits on any host.
* ``config0_64_run.json``: the wall-normal position profile ``yy`` the
  state is built from (channel_state's ``yy``; the rest of the state is
  seeded random numbers and correctly rounded arithmetic), the time step,
  per-step Q from Driven_force, SHA-256 digests of U_, U, Uq after steps
  10 and 100, and the mean streamwise velocity profile after step 100.

Run from the repository root: ``python tests/golden/make_config0_run.py``
(about three minutes on eight cores).
"""
import bz2
import hashlib
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

DIMS = (64, 64, 64)
MACH, RE, GAMMA, SEED = 0.5, 2800.0, 2.0, 0
STEPS, SUBITERATIONS, DIGEST_AT = 100, 10, (10, 100)


def static_names():
    names = ["J", "Y_point"] + [f"cell_metric{n}" for n in range(9)]
    for d in range(3):
        names += [f"face_J{d}"] + [f"face_metric{d}_{n}" for n in range(9)]
    return names


def static_arrays(f):
    out = [f["J"], f["Y_point"]] + list(f["cell_metric"])
    for d in range(3):
        out += [f["face_J"][d]] + list(f["face_metric"][d])
    return out


def state_digest(f):
    h = hashlib.sha256()
    for key in ("U_", "U", "Uq"):
        for a in f[key]:
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def mean_u(g, f):
    ix = g.interior
    u = f["U"][1][ix] / f["U"][0][ix]
    return u.mean(axis=(0, 2))


def main():
    import cases
    from channel_flow_gb300 import synthetic as syn
    from oracle.cforacle import Port
    port = Port()
    g = syn.channel_physics(syn.channel_grid(*DIMS), MACH, RE)
    f = cases.channel_step_case(g, gamma=GAMMA, seed=SEED, mach=MACH, port=port)
    Y = g.shape[1]
    j = np.arange(Y, dtype=np.float64)
    eta = np.clip(1 - 2 * (j - 1.5) * g.deltaET, -1.0, 1.0)
    yy = 1 - 1.0 / math.tanh(GAMMA) * np.tanh(GAMMA * eta)
    # the fixture's state must be the one channel_step_case built
    U = syn.channel_state(g, f["J"], seed=SEED, mach=MACH, noise=0.05, jitter=0.01, gamma=GAMMA,
                          wall_damped=True, yy=yy)
    assert all(np.array_equal(a, b) for a, b in zip(U, f["U"]))
    raw = b"".join(np.ascontiguousarray(a, dtype=np.float64).tobytes() for a in static_arrays(f))
    (HERE / "config0_64_static.bz2").write_bytes(bz2.compress(raw, 9))
    dt = syn.time_step(g, MACH)
    E = [0.0] * 5
    q, digests = [], {}
    t0 = time.time()
    for s in range(1, STEPS + 1):
        it, er, Q = cases.port_step(port, g, f, dt, SUBITERATIONS, 0.0, E, scheme="consistent")
        assert it == SUBITERATIONS
        q.append(float(Q).hex())
        if s in DIGEST_AT:
            digests[str(s)] = state_digest(f)
        print(f"step {s} {time.time() - t0:.1f}s", file=sys.stderr)
    out = {"dims": list(DIMS), "mach": MACH, "re_bulk": RE, "gamma": GAMMA, "seed": SEED,
           "steps": STEPS, "subiterations": SUBITERATIONS, "scheme": "consistent", "filter": "every sub-iteration",
           "deltaT": dt.hex(), "yy": [float(x).hex() for x in yy], "static_names": static_names(),
           "Q": q, "sha256": digests, "mean_u_100": [float(x).hex() for x in mean_u(g, f)],
           "E": [float(x).hex() for x in E]}
    (HERE / "config0_64_run.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
