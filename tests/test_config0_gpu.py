"""The 64^3 plain-FP64 channel schedule run end to end on the GPU.

100 physical steps of 10 LU-SGS sub-iterations each (main.cpp:143-498 with
the limited fluxes, the Filter at every sub-iteration, Driven_force and the
level shift), Mach 0.5, Re_bulk 2800, deltaT = 0.005 h/U_b, consistent
face-state scaling (the reference's own diverges in the first step), from
the stored inputs of tests/golden/config0_64_run.json:

* no-FMA build: after steps 10 and 100 the state (U_, U, Uq) equals the C
  oracle's run bit for bit (SHA-256 of the arrays); Q of every step agrees
  to 1e-12 (a reduction summed in another order);
* FMA build: the mean streamwise velocity after 100 steps within 1e-9 of
  the oracle's;
* FP32 path (FP32 kernels, FP64 state and norms): within 0.5 % of it.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _to_dev(f):
    import torch
    out = {}
    for k, v in f.items():
        if isinstance(v, list):
            out[k] = [[torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in w] if isinstance(w, list)
                      else torch.from_numpy(np.ascontiguousarray(w)).cuda() for w in v]
        else:
            out[k] = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    return out


def _run(precision, stop_at):
    """Run the schedule in `precision`; returns ({step: digest}, [Q], mean u)."""
    import channel_flow_gb300 as cf
    g, f, meta = cases.config0_case()
    dev = _to_dev(f)
    ctx = cf.Context(g, precision=precision, gamma=meta["gamma"], scheme=meta["scheme"])
    digests, q = {}, []
    try:
        for s in range(1, meta["steps"] + 1):
            it, er, Q = ctx.step(dev, step=s, deltaT=meta["deltaT_value"], max_iterations=meta["subiterations"],
                                 tolerance=0.0, limiter=True, filter=True, statistic_step=0, static_metrics=True)
            assert it == meta["subiterations"]
            q.append(Q)
            if s in stop_at:
                digests[s] = cases.state_digest(dev, lambda t: t.cpu().numpy())
        ix = g.interior
        U = [dev["U"][n].cpu().numpy() for n in (0, 1)]
        mean_u = (U[1][ix] / U[0][ix]).mean(axis=(0, 2))
    finally:
        ctx.close()
    return digests, q, mean_u, meta


def test_config0_exact_equals_oracle_run(cuda_lib):
    digests, q, mean_u, meta = _run("fp64_exact", (10, 100))
    for s, want in meta["sha256"].items():
        assert digests[int(s)] == want, f"state after step {s} differs from the oracle's"
    want_q = [float.fromhex(x) for x in meta["Q"]]
    np.testing.assert_allclose(q, want_q, rtol=1e-12, atol=0)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-9), ("fp32", 5e-3)])
def test_config0_mean_velocity(precision, rtol, cuda_lib):
    _, _, mean_u, meta = _run(precision, ())
    want = np.array([float.fromhex(x) for x in meta["mean_u_100"]])
    err = float(np.max(np.abs(mean_u - want))) / float(np.max(np.abs(want)))
    assert np.isfinite(mean_u).all()
    assert err <= rtol, f"{precision}: mean u after 100 steps differs by {err:.3e} of its maximum"
