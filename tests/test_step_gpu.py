"""The physical-step driver (cf_step) against the same loop on the C
oracle: in the no-FMA build every field after the step equals the
oracle's bit for bit; the residual norms and Q agree to 1e-12."""
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


@pytest.mark.parametrize("dims", [(12, 10, 8), (13, 9, 17)])
def test_gpu_step_equals_oracle_loop(dims, port, cuda_lib):
    import channel_flow_gb300 as cf
    g = cases.grid(dims)
    f = cases.step_case(g, seed=2)
    dev = _to_dev(f)
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        E = [0.0] * 5
        for step in (1, 2):
            it_g, er_g, q_g = ctx.step(dev, step=step, max_iterations=2, tolerance=1e-3, statistic_step=0)
            it_p, er_p, q_p = cases.port_step(port, g, f, 0.00000005, 2, 1e-3, E)
            assert it_g == it_p
            np.testing.assert_allclose(er_g, er_p, rtol=1e-12, atol=0)
            assert abs(q_g - q_p) <= 1e-12 * abs(q_p)
        for key in ("U_", "U", "Uq"):
            for n in range(5):
                assert np.array_equal(dev[key][n].cpu().numpy(), f[key][n], equal_nan=True), (key, n)
    finally:
        ctx.close()
