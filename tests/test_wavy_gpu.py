"""Wavy-wall metric generator (cf_wavy_metrics, cf_wavy_y_point): against
its numpy restatement on a curved grid, against the reference's flat-wall
metrics at zero amplitude, the discrete geometric conservation law of the
conservative form, and physical steps on a wavy channel."""
import math

import numpy as np
import pytest

from oracle import metric_oracle as mo

GAMMA = 1.5


def _grid(X=16, Y=12, Z=8):
    from channel_flow_gb300 import synthetic as syn
    return syn.channel_grid(X, Y, Z)


def _wall(g, amp_h, conservative, gamma=GAMMA):
    from channel_flow_gb300 import wavy
    return wavy.wall_for(g, amplitude_over_h=amp_h, wavelength_over_h=math.pi, stretching=gamma,
                         conservative=conservative)


def _oracle(g, w, where):
    return mo.metrics(g.shape, g.deltaXI, g.deltaET, g.high, w.amplitude, w.wavelength, w.stretching,
                      w.conservative, where)


def _close(got, want, rtol):
    scale = max(float(np.max(np.abs(want))), 1e-300)
    return float(np.max(np.abs(got - want))) <= rtol * scale


# ---------------------------------------------------------------------------
# oracle alone (CPU)

def test_oracle_flat_limit_is_flat_metrics():
    from channel_flow_gb300 import synthetic as syn
    g = _grid()
    w = type("W", (), {"amplitude": 0.0, "wavelength": math.pi * 0.5 * g.high, "stretching": GAMMA,
                       "conservative": False})()
    for where in ("cell", "u", "v", "w"):
        got = _oracle(g, w, where)
        want = syn.flat_metrics(g, GAMMA, where)
        assert _close(got[0], want["J"], 1e-14), where
        for n, name in enumerate(syn.METRIC_NAMES):
            assert _close(got[1 + n], want[name], 1e-14), (where, name)
    yp = mo.y_point(g.shape, g.deltaXI, g.deltaET, g.high, 0.0, 1.0, GAMMA)
    assert _close(yp, syn.y_points(g, gamma=GAMMA), 1e-14)


@pytest.mark.parametrize("conservative", [True, False])
def test_oracle_free_stream(conservative):
    """The conservative form makes the divergence of a constant flux
    vanish to rounding on the curved grid; the analytic form does not."""
    g = _grid(32, 24, 8)
    w = type("W", (), {"amplitude": 0.2 * 0.5 * g.high, "wavelength": math.pi * 0.5 * g.high,
                       "stretching": GAMMA, "conservative": conservative})()
    f = {s: _oracle(g, w, s) for s in ("u", "v", "w")}
    d = mo.divergence_of_constant_flux(f["u"], f["v"], f["w"], g.deltaXI, g.deltaET, g.deltaZT, 0)
    term = float(np.max(np.abs(f["u"][1] / f["u"][0]))) / g.deltaXI
    if conservative:
        assert float(np.max(np.abs(d))) <= 1e-11 * term
    else:
        assert float(np.max(np.abs(d))) >= 1e-6 * term


# ---------------------------------------------------------------------------
# device generator



@pytest.mark.gpu
@pytest.mark.parametrize("conservative", [True, False])
def test_wavy_metrics_match_oracle(cuda_lib, conservative):
    from channel_flow_gb300 import wavy
    g = _grid()
    w = _wall(g, 0.2, conservative)
    for where in ("cell", "u", "v", "w"):
        got = [t.cpu().numpy() for t in wavy.metrics(g, w, where)]
        want = _oracle(g, w, where)
        for n in range(10):
            assert _close(got[n], want[n], 1e-12), (where, n)
    yp = wavy.y_point(g, w).cpu().numpy()
    assert _close(yp, mo.y_point(g.shape, g.deltaXI, g.deltaET, g.high, w.amplitude, w.wavelength, GAMMA), 1e-13)


@pytest.mark.gpu
def test_wavy_flat_limit_matches_reference_metrics(cuda_lib):
    """Amplitude 0, analytic form: the face metrics of the device
    Jacobian_u/v/w routines (the reference's, Jacobian_?.cpp) on the index
    ranges they write, the v-face wall rows excepted (Jacobian_v.cpp:124-141
    copies cell metrics there)."""
    import torch
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import synthetic as syn, wavy
    g = _grid()
    ctx = cf.Context(g, precision="fp64_exact", gamma=GAMMA)
    w = _wall(g, 0.0, False)
    z = lambda: torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    fu = [z() for _ in range(10)]
    fw = [z() for _ in range(10)]
    fv = [z() for _ in range(10)]
    cell = wavy.metrics(g, w, "cell")
    ctx.Jacobian_u(*fu)
    ctx.Jacobian_w(*fw)
    ctx.Jacobian_v(*fv, *cell)
    for where, ref in (("u", fu), ("w", fw), ("v", fv)):
        got = [t.cpu().numpy() for t in wavy.metrics(g, w, where)]
        want = [t.cpu().numpy() for t in ref]
        mask = want[0] != 0
        if where == "v":
            mask[:, 1, :] = False
            mask[:, g.ny, :] = False
        assert mask.sum() > 0
        for n in range(10):
            assert np.allclose(got[n][mask], want[n][mask], rtol=1e-14, atol=1e-14 * np.abs(want[n]).max()), (where, n)
    want = syn.flat_metrics(g, GAMMA, "cell")
    got = [t.cpu().numpy() for t in cell]
    assert _close(got[0], want["J"], 1e-14)
    for n, name in enumerate(syn.METRIC_NAMES):
        assert _close(got[1 + n], want[name], 1e-14), name
    ctx.close()


@pytest.mark.gpu
def test_wavy_device_free_stream(cuda_lib):
    from channel_flow_gb300 import wavy
    g = _grid(32, 24, 8)
    for conservative, bound in ((True, 1e-11), (False, None)):
        w = _wall(g, 0.2, conservative)
        f = {s: [t.cpu().numpy() for t in wavy.metrics(g, w, s)] for s in ("u", "v", "w")}
        term = float(np.max(np.abs(f["u"][1] / f["u"][0]))) / g.deltaXI
        for d in range(3):
            div = mo.divergence_of_constant_flux(f["u"], f["v"], f["w"], g.deltaXI, g.deltaET, g.deltaZT, d)
            if bound is not None:
                assert float(np.max(np.abs(div))) <= bound * term, d


@pytest.mark.gpu
def test_wavy_channel_steps(cuda_lib):
    """Physical steps of the stable scheme (unlimited fluxes, no filter,
    dt 5e-9) on a channel with a 0.05 h wall wave converge to the
    tolerance and stay finite, in FP64 and in the mixed FP32 path, and the
    two agree (state difference small against the change over the steps,
    the scale that the tolerance sets)."""
    import torch
    import bench
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import stepper, synthetic as syn, wavy
    g = _grid(32, 24, 16)
    w = _wall(g, 0.05, True, gamma=bench.GAMMA)
    finals = {}
    for prec in ("fp64", "fp32"):
        ctx = cf.Context(g, precision=prec, gamma=bench.GAMMA)
        m = wavy.channel_metrics(g, w)
        J = m["J"].cpu().numpy()
        host = {"U": syn.channel_state(g, J, seed=3, mach=0.05, noise=0.01, jitter=0.001, gamma=bench.GAMMA),
                "J": J, "cm": [t.cpu().numpy() for t in m["cm"]], "Yp": m["Yp"].cpu().numpy()}
        dw = bench.DeviceWorkload(ctx, g, host, torch)
        for dst, src in ((dw.fu, m["fu"]), (dw.fv, m["fv"]), (dw.fw, m["fw"])):
            for a, b in zip(dst, src):
                a.copy_(b)
        st = stepper.Stepper(ctx, stepper.fields_from_workload(dw, torch, g), deltaT=5e-9, max_iterations=200,
                             tolerance=1e-6, limiter=False, filter=False)
        start = [u.clone() for u in st.f["U"]]
        its = [st.step("extrapolate")[0] for _ in range(4)]
        assert max(its) < 200, its
        for u in st.f["U"]:
            assert bool(torch.isfinite(u).all())
        finals[prec] = [u.clone() for u in st.f["U"]]
        ctx.close()
    for v in range(5):
        a, b = finals["fp32"][v], finals["fp64"][v]
        assert float((a - b).abs().max()) <= 1e-2 * float((b - start[v]).abs().max()), v


@pytest.mark.gpu
def test_wavy_channel_exact_equals_oracle(cuda_lib, port):
    """The configuration schedule's physics on a wavy lower wall (0.05 h,
    wavelength pi h, metrics of the numpy restatement): limited MUSCL-5 +
    Roe with the consistent face-state scaling, the Filter at every
    sub-iteration, 10 fixed sub-iterations per step, Mach 0.5, Re_b 11000,
    dt = 0.005/8 h/U_b.  After each of four steps the no-FMA GPU state (U_,
    U, Uq) equals the C oracle's bit for bit on the same inputs."""
    import torch
    import cases
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import synthetic as syn
    g = syn.channel_physics(syn.channel_grid(24, 16, 20), 0.5, 11000.0)
    h = 0.5 * g.high
    A, lam, gam = 0.05 * h, math.pi * h, 2.0
    met = {w: mo.metrics(g.shape, g.deltaXI, g.deltaET, g.high, A, lam, gam, True, w) for w in ("cell", "u", "v", "w")}
    J = met["cell"][0]
    U = syn.channel_state(g, J, seed=0, mach=0.5, noise=0.05, jitter=0.01, gamma=gam, wall_damped=True)
    z = lambda: np.zeros(g.shape)
    f = {"U_": [u.copy() for u in U], "U": [u.copy() for u in U], "Uq": [u.copy() for u in U], "J": J,
         "Y_point": mo.y_point(g.shape, g.deltaXI, g.deltaET, g.high, A, lam, gam), "cell_metric": met["cell"][1:],
         "face_J": [met[w][0] for w in ("u", "v", "w")], "face_metric": [met[w][1:] for w in ("u", "v", "w")],
         "Ep": [z() for _ in range(3)], "inF": [[z() for _ in range(5)] for _ in range(3)],
         "vF": [z() for _ in range(4)], "LL": [z() for _ in range(4)], "ML": [z() for _ in range(4)],
         "MR": [z() for _ in range(5)], "NR": [z() for _ in range(5)], "NL": [z() for _ in range(5)],
         "Residual": [z() for _ in range(5)]}
    dev = {k: ([[torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in w] if isinstance(w, list)
                 else torch.from_numpy(np.ascontiguousarray(w)).cuda() for w in v] if isinstance(v, list)
               else torch.from_numpy(np.ascontiguousarray(v)).cuda()) for k, v in f.items()}
    dt = syn.time_step(g, 0.5) / 8
    ctx = cf.Context(g, precision="fp64_exact", gamma=gam, scheme="consistent")
    E = [0.0] * 5
    try:
        for s in range(1, 5):
            ctx.step(dev, step=s, deltaT=dt, max_iterations=10, tolerance=0.0, limiter=True, filter=True,
                     statistic_step=0, static_metrics=True)
            cases.port_step(port, g, f, dt, 10, 0.0, E, scheme="consistent")
            assert cases.state_digest(dev, lambda t: t.cpu().numpy()) == cases.state_digest(f), s
    finally:
        ctx.close()
