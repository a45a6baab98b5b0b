"""The consistent face-state scaling (cf_set_scheme(CF_SCHEME_CONSISTENT))
on the GPU against the C oracle's consistent variant: bit for bit in the
no-FMA build, within 1e-12 in the contracted FP64 build, within the
mixed-precision bound in FP32; and the physical-step driver with it against
the oracle's limited loop."""
import numpy as np
import pytest

import cases
import routines
from channel_flow_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu
NAMES = ["Flux_Y_limiter", "Flux_Z_limiter"]


@pytest.fixture(scope="module")
def ctx_factory(cuda_lib):
    import channel_flow_gb300 as cf
    made = {}

    def get(dims, precision):
        key = (dims, precision)
        if key not in made:
            made[key] = cf.Context(cases.grid(dims), precision=precision, scheme="consistent")
        return made[key]
    yield get
    for c in made.values():
        c.close()


def _run(port, ctx, r, g, seed=3):
    a = r.build(g, seed)
    want, got = cases.copy_case(a), cases.copy_case(a)
    routines.run_cpu(port, r, g, want, scheme="consistent")
    routines.run_gpu(ctx, r, got)
    return want, got


@pytest.mark.parametrize("dims", cases.GRIDS)
@pytest.mark.parametrize("name", NAMES)
def test_consistent_exact_equals_oracle(dims, name, port, ctx_factory):
    r = routines.BY_NAME[name]
    g = cases.grid(dims)
    want, got = _run(port, ctx_factory(dims, "fp64_exact"), r, g)
    diff = routines.compare(r, g, got, want)
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("dims", cases.GRIDS[:2])
@pytest.mark.parametrize("name", NAMES)
def test_consistent_fp64_within_1e12(dims, name, port, ctx_factory):
    r = routines.BY_NAME[name]
    g = cases.grid(dims)
    want, got = _run(port, ctx_factory(dims, "fp64"), r, g)
    diff = routines.compare(r, g, got, want, rtol=1)
    assert max(diff.values()) <= 1e-12, diff


@pytest.mark.parametrize("name", NAMES)
def test_consistent_fp32_error_bounded(name, port, ctx_factory):
    r = routines.BY_NAME[name]
    dims = cases.GRIDS[0]
    g = cases.grid(dims)
    want, got = _run(port, ctx_factory(dims, "fp32"), r, g)
    diff = routines.compare(r, g, got, want, rtol=1)
    assert max(diff.values()) <= 2e-3, diff


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


def test_consistent_step_equals_oracle_loop(port, cuda_lib):
    """cf_step (limited fluxes with the Filter) with the consistent scheme,
    no-FMA build, at Mach 0.5, Re_b 2800 and dt = 0.005 h/U_b on a 14x12x16
    channel: every field after two steps equals the oracle's loop bit for
    bit; norms and Q to 1e-12."""
    import channel_flow_gb300 as cf
    g = syn.channel_physics(syn.channel_grid(14, 12, 16), 0.5, 2800)
    dt = syn.time_step(g, 0.5)
    f = cases.channel_step_case(g, port=port)
    dev = _to_dev(f)
    ctx = cf.Context(g, precision="fp64_exact", gamma=2.0, scheme="consistent")
    try:
        E = [0.0] * 5
        for step in (1, 2):
            it_g, er_g, q_g = ctx.step(dev, step=step, deltaT=dt, max_iterations=3, tolerance=1e-9,
                                       statistic_step=0)
            it_p, er_p, q_p = cases.port_step(port, g, f, dt, 3, 1e-9, E, scheme="consistent")
            assert it_g == it_p
            np.testing.assert_allclose(er_g, er_p, rtol=1e-12, atol=0)
            assert abs(q_g - q_p) <= 1e-12 * abs(q_p)
        for key in ("U_", "U", "Uq"):
            for n in range(5):
                assert np.array_equal(dev[key][n].cpu().numpy(), f[key][n], equal_nan=True), (key, n)
    finally:
        ctx.close()
