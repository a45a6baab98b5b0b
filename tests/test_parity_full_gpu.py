"""Parity at the mixed-precision configuration's full grid, 256 x 192 x 192
(9.4 M cells): the no-FMA build of every hot-path routine against the C
oracle on the same seeded inputs, bit for bit on every written array
(the residual norms, summed in another order, to 1e-12; the tanh/cosh
metrics of Jacobian_u/v/w to 1e-13).  At this size the wavefront runs
36 864 tiles in 110 tile diagonals and the Filter's levels and the flux
launches fill many waves, so the scheduling that only large grids exercise
is checked against the reference's plane-ordered loop.  The whole file
runs in about 70 s (the oracle on the host cores, the case set-up)."""
import numpy as np
import pytest

import cases
import routines

pytestmark = pytest.mark.gpu
FULL = (256, 192, 192)


@pytest.fixture(scope="module")
def ctx_full(cuda_lib):
    import channel_flow_gb300 as cf
    ctx = cf.Context(cases.grid(FULL), precision="fp64_exact")
    yield ctx
    ctx.close()


@pytest.mark.parametrize("name", [r.name for r in routines.ROUTINES])
def test_exact_equals_oracle_full_grid(name, port, ctx_full):
    import torch
    r = routines.BY_NAME[name]
    g = cases.grid(FULL)
    a = r.build(g, 41)
    want = cases.copy_case(a)
    e_want = routines.run_cpu(port, r, g, want)
    e_got = routines.run_gpu(ctx_full, r, a)          # a: inputs copied to the device, outputs back into a
    if r.libm:
        # tanh/cosh metrics: CUDA's and the host's libm agree to 1e-13
        diff = routines.compare(r, g, a, want, rtol=1)
        assert max(diff.values()) <= 1e-13, diff
    else:
        diff = routines.compare(r, g, a, want)
        assert all(v == 0 for v in diff.values()), f"{name}: differing entries per slot {diff}"
    if r.scalars:
        np.testing.assert_allclose(e_got, e_want, rtol=1e-12, atol=0)
    del a, want
    torch.cuda.empty_cache()
