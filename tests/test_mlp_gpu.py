"""The learned-guess MLP: forward pass and every gradient of the tcgen05
path against the float64 oracle with the same BF16 roundings
(oracle/mlp_oracle.py), training convergence, and the gain of the trained
guess on the solver's own pseudo-time iterations."""
import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def _net(capacity=512, seed=3):
    from channel_flow_gb300 import mlp
    return mlp, mlp.LearnedGuess(capacity=capacity, seed=seed)


def test_mlp_forward_and_gradients_match_oracle(cuda_lib):
    import torch
    mlp, net = _net()
    rng = np.random.default_rng(7)
    M, Mpad = 300, 512
    X = np.zeros((Mpad, mlp.K1), np.float32)
    X[:M, :mlp.IN] = rng.normal(0, 1, (M, mlp.IN))
    T = np.zeros((Mpad, mlp.N3), np.float32)
    T[:M, :mlp.OUT] = rng.normal(0, 1, (M, mlp.OUT))
    Xb = torch.from_numpy(X).cuda().to(torch.bfloat16)
    net.X.copy_(Xb)
    net.T.copy_(torch.from_numpy(T).cuda())
    net.forward(Mpad)
    net.backward(M, Mpad)
    torch.cuda.synchronize()
    net.check_device()
    p = net.p.cpu().numpy()
    loss, Y, g = mlp_oracle.forward_backward(p, mlp.OFFS, Xb.float().cpu().numpy(), T, M)
    Yg = net.Y.cpu().numpy()
    assert np.max(np.abs(Yg[:M, :5] - Y[:M, :5])) <= 1e-2 * np.max(np.abs(Y[:M, :5]))
    assert abs(net.loss(Mpad) - loss) <= 1e-2 * loss
    gg = net.g.cpu().numpy()
    for name, (o, s) in mlp.OFFS.items():
        n = int(np.prod(s))
        want, got = g[o:o + n], gg[o:o + n]
        err = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-30)
        assert err <= 1e-2, (name, err)


def test_mlp_training_reduces_loss(cuda_lib):
    """Fit a smooth function of the features: the loss falls by 10x."""
    import torch
    mlp, net = _net(capacity=4096, seed=1)
    net.lr = 3e-3
    rng = np.random.default_rng(2)
    M = 4096
    X = np.zeros((M, mlp.K1), np.float32)
    X[:, :mlp.IN] = rng.normal(0, 1, (M, mlp.IN))
    A = rng.normal(0, 1.0 / np.sqrt(mlp.IN), (mlp.IN, 5))
    T = np.zeros((M, mlp.N3), np.float32)
    T[:, :5] = np.tanh(X[:, :mlp.IN] @ A)
    net.X.copy_(torch.from_numpy(X).cuda().to(torch.bfloat16))
    net.T.copy_(torch.from_numpy(T).cuda())
    first = net.step(M, M)
    for _ in range(150):
        last = net.step(M, M)
    net.check_device()
    assert last < 0.1 * first, (first, last)


def _guess_study(dims, harvest, evals, precision="fp64", epochs=30, batch=None, online=None):
    """Harvest FP64 steps from a seeded channel (unlimited fluxes, dt 5e-9,
    where the assembled loop is stable), train the network on them, then
    run `evals` steps from the same start with each initial guess at the
    residual tolerance 1e-6 (er_n / max er_n, fields 1-4).  Returns the
    sub-iteration counts, the final states, the start and the network."""
    import torch
    import bench
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import mlp, stepper, synthetic as syn
    g = syn.channel_grid(*dims)
    cm = syn.flat_metrics(g, bench.GAMMA, "cell")
    J = cm["J"]
    host = {"U": syn.channel_state(g, J, seed=1, mach=0.05, noise=0.01, jitter=0.001, gamma=bench.GAMMA),
            "J": J, "cm": [cm[n] for n in syn.METRIC_NAMES], "Yp": syn.y_points(g, gamma=bench.GAMMA)}
    kw = dict(deltaT=5e-9, max_iterations=200, tolerance=1e-6, limiter=False, filter=False)
    ctx = cf.Context(g, precision="fp64", gamma=bench.GAMMA)
    w = bench.DeviceWorkload(ctx, g, host, torch)
    st = stepper.Stepper(ctx, stepper.fields_from_workload(w, torch, g), **kw)
    hist = [[u.clone() for u in st.f["U"]]]
    for _ in range(harvest):
        st.step()
        hist.append([u.clone() for u in st.f["U"]])
    E = ctx.step_scale()
    net = mlp.LearnedGuess(capacity=g.cells, seed=0, lr=2e-3, batch=batch)
    losses = net.train(g, hist, epochs=epochs, batch=batch)
    start = hist[-3:]
    its, final = {}, {}
    ctx.set_precision(precision)
    for name, guess in (("plain", None), ("extrapolate", "extrapolate"), ("learned", net)):
        st.restore(start, step=harvest)
        st.online = online if name == "learned" else None
        ctx.step_scale(E)
        its[name] = [st.step(guess)[0] for _ in range(evals)]
        final[name] = [u.clone() for u in st.f["U"]]
    net.check_device()
    ctx.close()
    return its, final, start, net, losses


def _state_err(a, b, start):
    return max(float((a[v] - b[v]).abs().max()) / float((b[v] - start[-1][v]).abs().max()) for v in range(5))


def test_learned_guess_cuts_subiterations(cuda_lib):
    """What the trained network gains, in the mixed-precision loop on a
    64^3 channel at the tolerance 1e-6: against the method without it (the
    plain start from U^n) at most half the sub-iterations, against the
    quadratic extrapolation at least 15% fewer, with the same answer (state
    difference small against the change over the steps); out of sample (the
    held-out window) its correction shrinks the error of the fitted linear
    predictor it corrects for density and energy, the fields whose updates
    converge last.  (The loss falls by half at least: the fitted predictor
    already removes most of what a correction of the plain extrapolation
    would learn.)"""
    its, final, start, net, losses = _guess_study((64, 64, 64), harvest=12, evals=4, precision="fp32",
                                                  epochs=40, batch=65536)
    print(its, net.coef, net.validation)
    assert losses[-1] < 0.5 * losses[0]
    plain, extra, learned = (np.mean(its[k]) for k in ("plain", "extrapolate", "learned"))
    assert learned <= 0.5 * plain, its
    assert learned <= 0.85 * extra, its
    assert _state_err(final["learned"], final["plain"], start) < 1e-2, its
    raw = net.validation["err_over_extrapolation_raw"]
    assert raw[0] < 0.8 and raw[4] < 0.8, net.validation


def test_mlp_data_kernels_match_oracle(cuda_lib):
    """Scalings, feature rows (all cells and a row subset), targets and the
    guess of the device kernels against the numpy restatement."""
    import torch
    from channel_flow_gb300 import mlp
    X, Y, Z = 6, 5, 7
    shape = (X + 6, Y + 4, Z + 4)
    rng = np.random.default_rng(11)
    base = [rng.uniform(0.5, 2.0, shape) for _ in range(5)]
    lv = [[b + 1e-3 * t * rng.normal(size=shape) + 1e-4 * t * t for b in base] for t in range(4)]
    nxt, un, u1, u2 = lv[3], lv[2], lv[1], lv[0]
    dev = lambda L: [torch.from_numpy(a.copy()).cuda() for a in L]
    g = type("G", (), {"X_out": X, "Y_out": Y, "Z_out": Z, "cells": X * Y * Z})()
    net = mlp.LearnedGuess(capacity=256, seed=0)
    Dn, D1, D2, Dx = dev(un), dev(u1), dev(u2), dev(nxt)
    net.set_scale_device(g, Dn, D1, D2)
    sc_dev = net.scale.cpu().numpy()
    sc = net.set_scale(g, Dn, D1, D2)
    want = mlp_oracle.rms([un, u1, u2], X, Y, Z)
    assert np.allclose(sc, want, rtol=1e-12), (sc, want)
    assert np.allclose(sc_dev, want.astype(np.float32), rtol=1e-6), (sc_dev, want)
    net.oscale.copy_(torch.tensor([0.5, 1.5, 2.0, 0.25, 1.0]))
    osc = net.oscale.cpu().numpy()
    # the sums of the predictor fit, and a predictor with mixed coefficients
    sums = net._base_sums(g, [D2, D1, Dn, Dx], 2).copy()
    assert np.allclose(sums, mlp_oracle.base_sums([nxt, un, u1, u2], X, Y, Z), rtol=1e-12, atol=0)
    net.coef[:] = [0.3, 1.0, -0.2, 0.0, 1.7, 0.9, 0.0, 0.4, 1.0, -0.5]
    coef = net.coef.copy()
    M, Mpad = net.load_features(g, Dn, D1, D2)
    F = net.X[:Mpad].float().cpu().numpy()
    Fw = mlp_oracle.features([un, u1, u2], sc.astype(np.float32), X, Y, Z)
    assert np.array_equal(F[:M], Fw) and not F[M:].any()
    rows = np.array([5, 0, 209, 17, 17, 100], np.int32)
    M, Mpad = net.load_features(g, Dn, D1, D2, rows=torch.from_numpy(rows).cuda())
    assert np.array_equal(net.X[:M].float().cpu().numpy(), Fw[rows])
    M, Mpad = net.load_targets(g, Dx, Dn, D1, D2)
    T = net.T[:M].cpu().numpy()
    Tw = mlp_oracle.targets(nxt, [un, u1, u2], sc, osc, X, Y, Z, coef10=coef)
    assert np.allclose(T, Tw, rtol=1e-6, atol=1e-6 * np.abs(Tw).max())
    Yc = rng.normal(size=(M, 16)).astype(np.float32)
    net.Y[:M].copy_(torch.from_numpy(Yc))
    out = dev([np.zeros(shape)] * 5)
    net._ok(net.lib.cf_mlp_apply(net._s(), X, Y, Z, (mlp.C.c_void_p * 15)(*[t.data_ptr() for t in Dn + D1 + D2]),
                                 coef.ctypes.data, net.scale.data_ptr(), net.oscale.data_ptr(), net.Y.data_ptr(),
                                 (mlp.C.c_void_p * 5)(*[t.data_ptr() for t in out])), "cf_mlp_apply")
    got = [o.cpu().numpy()[3:3 + X, 2:2 + Y, 2:2 + Z].reshape(-1) for o in out]
    want = mlp_oracle.apply([un, u1, u2], sc, osc, Yc, X, Y, Z, coef10=coef)
    for v in range(5):
        assert np.allclose(got[v], want[v], rtol=1e-14, atol=0), v
    mlp.LearnedGuess.extrapolate(g, Dn, D1, D2, out)
    want = mlp_oracle.apply([un, u1, u2], None, None, None, X, Y, Z)
    for v in range(5):
        assert np.allclose(out[v].cpu().numpy()[3:3 + X, 2:2 + Y, 2:2 + Z].reshape(-1), want[v], rtol=1e-14), v
