"""Failure detection on the GPU in the allowed forms: a bounded device wait
made to run out on purpose (a short wait limit; nothing faults or hangs),
and a non-finite value injected on the host.

* With the sweeps' dependency-wait limit set to one poll, tiles (or
  pencils) stop waiting for their upstream neighbours: Dual_time_stepping returns
  CF_ERR_TIMEOUT (its results are then invalid) instead of hanging, and
  the next call on the same context at the default limit equals the
  oracle bit for bit again.
* A NaN written into a registered host array and uploaded is reported by
  cf_check_finite, and a physical step on that state ends with
  CF_ERR_NONFINITE (its residual norms are not finite).
"""
import numpy as np
import pytest

import cases
import routines
from channel_flow_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("schedule", ["wavefront", "pencil"])
def test_wavefront_wait_runs_out_then_recovers(schedule, port, cuda_lib):
    import channel_flow_gb300 as cf
    r = routines.BY_NAME["Dual_time_stepping"]
    g = cases.grid((32, 24, 40))
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        ctx.set_lu_schedule(schedule)
        a = r.build(g, 23)
        ctx.set_wait_limit(1)
        with pytest.raises(cf.CFError) as exc:
            routines.run_gpu(ctx, r, cases.copy_case(a))
        assert exc.value.code == _lib.CF_ERR_TIMEOUT, exc.value
        ctx.set_wait_limit(0)
        want, got = cases.copy_case(a), cases.copy_case(a)
        e_want = routines.run_cpu(port, r, g, want)
        e_got = routines.run_gpu(ctx, r, got)
        diff = routines.compare(r, g, got, want)
        assert all(v == 0 for v in diff.values()), diff
        np.testing.assert_allclose(e_got, e_want, rtol=1e-12, atol=0)
    finally:
        ctx.close()


def test_nonfinite_state_detected(cuda_lib):
    import torch
    import channel_flow_gb300 as cf
    g = cases.grid((12, 10, 8))
    f = cases.step_case(g, seed=3)
    ctx = cf.Context(g, precision="fp64")
    try:
        host = f["U_"][1]                  # rho u / J, a registered host array
        ctx.register(host)
        ctx.upload(host)
        ctx.check_finite(host)             # finite: no error
        host[5, 4, 3] = np.nan             # an interior cell
        ctx.upload(host)
        with pytest.raises(cf.CFError) as exc:
            ctx.check_finite(host)
        assert exc.value.code == _lib.CF_ERR_NONFINITE
        dev = {}
        for k, v in f.items():
            if isinstance(v, list):
                dev[k] = [[torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in w] if isinstance(w, list)
                          else torch.from_numpy(np.ascontiguousarray(w)).cuda() for w in v]
            else:
                dev[k] = torch.from_numpy(np.ascontiguousarray(v)).cuda()
        with pytest.raises(cf.CFError) as exc:
            ctx.step(dev, step=1, max_iterations=3, tolerance=1e-3)
        assert exc.value.code == _lib.CF_ERR_NONFINITE, exc.value
        assert "not finite" in str(exc.value)
    finally:
        ctx.close()
