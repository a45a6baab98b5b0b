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


def test_learned_guess_cuts_subiterations(cuda_lib):
    """Train on the solver's own steps (unlimited fluxes, dt 5e-9, where
    the assembled loop is stable), then continue the run: with the learned
    guess the held-out steps reach the same residual tolerance in at most
    half the sub-iterations of the plain start."""
    import torch
    import bench
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import mlp, stepper, synthetic as syn
    g = syn.channel_grid(24, 24, 24)
    cm = syn.flat_metrics(g, bench.GAMMA, "cell")
    J = cm["J"]
    host = {"U": syn.channel_state(g, J, seed=1, mach=0.05, noise=0.01, jitter=0.001, gamma=bench.GAMMA),
            "J": J, "cm": [cm[n] for n in syn.METRIC_NAMES], "Yp": syn.y_points(g, gamma=bench.GAMMA)}
    kw = dict(deltaT=5e-9, max_iterations=60, tolerance=1e-3, limiter=False, filter=False)

    def run(n_warm, guess, n_eval):
        ctx = cf.Context(g, precision="fp32", gamma=bench.GAMMA)
        w = bench.DeviceWorkload(ctx, g, host, torch)
        st = stepper.Stepper(ctx, stepper.fields_from_workload(w, torch, g), **kw)
        hist = [[u.clone() for u in w.U]]
        for _ in range(n_warm):
            st.step()
            hist.append([u.clone() for u in st.f["U"]])
        its = [st.step(guess)[0] for _ in range(n_eval)]
        ctx.close()
        return hist, its

    hist, plain = run(12, None, 4)
    net = mlp.LearnedGuess(capacity=g.cells, seed=0, lr=2e-3)
    losses = net.train(g, hist, epochs=30)
    assert losses[-1] < losses[0]
    _, learned = run(12, net, 4)
    assert np.mean(learned) <= 0.5 * np.mean(plain), (plain, learned)
