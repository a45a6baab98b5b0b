"""GPU kernels against the C oracle and the reference's golden digests.

* FP64 exact mode (no FMA): every written array equals the oracle bit for
  bit, i.e. equals the reference (the oracle is pinned to it bit for bit);
  only the residual norms, summed in a different order, are compared at
  1e-12 relative, and the tanh/cosh metrics at 1e-13.
* FP64 mode (FMA contraction): within 1e-12 normwise relative.
* FP32 mode: within the stated mixed-precision bound.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import cases
import routines

pytestmark = pytest.mark.gpu
GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_outputs.json").read_text())
RTOL_FP64 = 1e-12
RTOL_FP32 = {"Filter": None}   # FP32 switch decisions may differ: test_gpu_fp32_filter_switch
CONFIG0_GRID = (64, 64, 64)


@pytest.fixture(scope="module")
def ctx_factory(cuda_lib):
    import channel_flow_gb300 as cf
    made = {}

    def get(dims, precision):
        key = (dims, precision)
        if key not in made:
            made[key] = cf.Context(cases.grid(dims), precision=precision)
        return made[key]
    yield get
    for c in made.values():
        c.close()


def _run_both(port, ctx, r, g, seed=3):
    a = r.build(g, seed)
    want, got = cases.copy_case(a), cases.copy_case(a)
    e_want = routines.run_cpu(port, r, g, want)
    e_got = routines.run_gpu(ctx, r, got)
    return want, got, e_want, e_got


@pytest.mark.parametrize("dims", cases.GRIDS)
@pytest.mark.parametrize("name", [r.name for r in routines.ROUTINES])
def test_gpu_exact_equals_oracle(dims, name, port, ctx_factory):
    r = routines.BY_NAME[name]
    g = cases.grid(dims)
    want, got, e_want, e_got = _run_both(port, ctx_factory(dims, "fp64_exact"), r, g)
    if r.libm:
        diff = routines.compare(r, g, got, want, rtol=1)
        assert max(diff.values()) <= 1e-13, diff
    else:
        diff = routines.compare(r, g, got, want)
        assert all(v == 0 for v in diff.values()), f"{name}: differing entries per slot {diff}"
    if r.scalars:
        np.testing.assert_allclose(e_got, e_want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("seed", GOLDEN["seeds"])
@pytest.mark.parametrize("name", [r.name for r in routines.ROUTINES if not r.libm])
def test_gpu_exact_matches_reference_golden(name, seed, ctx_factory):
    r = routines.BY_NAME[name]
    dims = tuple(GOLDEN["grid"])
    g = cases.grid(dims)
    a = r.build(g, seed)
    er = routines.run_gpu(ctx_factory(dims, "fp64_exact"), r, a)
    rec = GOLDEN["routines"][name][str(seed)]
    for i in r.outputs:
        assert cases.digest(a[i], r.mask(g, i)) == rec["digests"][str(i)], f"{name} slot {i}"
    if "er" in rec:
        np.testing.assert_allclose(er, [float.fromhex(x) for x in rec["er"]], rtol=1e-12, atol=0)


@pytest.mark.parametrize("dims", cases.GRIDS[:2])
@pytest.mark.parametrize("name", [r.name for r in routines.ROUTINES])
def test_gpu_fp64_fma_within_1e12(dims, name, port, ctx_factory):
    r = routines.BY_NAME[name]
    g = cases.grid(dims)
    want, got, e_want, e_got = _run_both(port, ctx_factory(dims, "fp64"), r, g)
    diff = routines.compare(r, g, got, want, rtol=1)
    assert max(diff.values()) <= RTOL_FP64, diff
    if r.scalars:
        np.testing.assert_allclose(e_got, e_want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ["Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter", "Flux_X", "Flux_Y",
                                  "Flux_Z", "Viscous_terms", "RK3NODT", "DPLUSGS", "Dual_time_stepping"])
def test_gpu_fp32_error_bounded(name, port, ctx_factory):
    """FP32 kernels (FP64 state, FP32 changes): normwise error against the FP64
    oracle stays at single-precision level."""
    r = routines.BY_NAME[name]
    dims = cases.GRIDS[0]
    g = cases.grid(dims)
    want, got, e_want, e_got = _run_both(port, ctx_factory(dims, "fp32"), r, g)
    diff = routines.compare(r, g, got, want, rtol=1)
    print(name, {k: f"{v:.2e}" for k, v in diff.items()})
    assert max(diff.values()) <= 2e-3, diff


def _tied_case(r, g, seed=5):
    """A flux case whose state has tied neighbours in x, y and z: one plane,
    row and column of every variable copied from its lower neighbour."""
    a = r.build(g, seed)
    for n in range(5):
        U = a[n]
        U[5] = U[4]
        U[:, 5] = U[:, 4]
        U[:, :, 5] = U[:, :, 4]
    return a


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "fp32"])
@pytest.mark.parametrize("name", ["Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter"])
def test_gpu_limiter_ties(name, precision, port, ctx_factory):
    """Tied neighbours make the reference's limiter ratio 0/0 or x/0, and
    its state NaN there.  The exact build reproduces that bit for bit; the
    contracted and FP32 builds take the reciprocal of a zero difference as
    0, so every face is finite and the faces where the reference is finite
    agree with it."""
    r = routines.BY_NAME[name]
    dims = cases.GRIDS[0]
    g = cases.grid(dims)
    a = _tied_case(r, g)
    want, got = cases.copy_case(a), cases.copy_case(a)
    routines.run_cpu(port, r, g, want)
    routines.run_gpu(ctx_factory(dims, precision), r, got)
    nan_faces = 0
    for i in r.outputs:
        w, o = want[i], got[i]
        keep = np.ones(w.shape, bool)
        if precision == "fp64_exact":
            same = (w == o) | (np.isnan(w) & np.isnan(o))
            assert np.all(same[keep]), (i, int(np.count_nonzero(~same[keep])))
            continue
        nan_faces += int(np.count_nonzero(np.isnan(w) & keep))
        assert np.all(np.isfinite(o[keep])), (i, int(np.count_nonzero(~np.isfinite(o[keep]))))
        fin = keep & np.isfinite(w)
        scale = float(np.max(np.abs(w[fin])))
        err = float(np.max(np.abs(o[fin] - w[fin]))) / scale
        assert err <= (RTOL_FP64 if precision == "fp64" else 2e-3), (i, err)
    if precision != "fp64_exact":
        assert nan_faces > 0   # the case does reach the reference's 0/0


def test_gpu_fp32_filter_switch(port, ctx_factory):
    """FP32 sensor: the Ep switch agrees with the FP64 oracle except on
    faces whose sensor ratio lies within FP32 rounding of Roe_criterion
    (at most 1 % of the faces on the test case)."""
    r = routines.BY_NAME["Filter"]
    dims = cases.GRIDS[0]
    g = cases.grid(dims)
    want, got, _, _ = _run_both(port, ctx_factory(dims, "fp32"), r, g)
    for i in r.outputs:
        frac = np.count_nonzero(want[i] != got[i]) / want[i].size
        assert frac <= 0.01, (i, frac)


@pytest.mark.parametrize("schedule", ["wavefront", "pencil", "planes"])
@pytest.mark.parametrize("dims", cases.GRIDS + [(13, 9, 17), (6, 6, 7), (20, 7, 9), CONFIG0_GRID])
def test_gpu_dts_schedules_exact(dims, schedule, port, cuda_lib):
    """Every sweep schedule of Dual_time_stepping (tiled wavefront, pencils,
    one launch per hyperplane) equals the oracle bit for bit, on grids with
    partial tiles and pencils."""
    import channel_flow_gb300 as cf
    r = routines.BY_NAME["Dual_time_stepping"]
    g = cases.grid(dims)
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        ctx.set_lu_schedule(schedule)
        want, got, e_want, e_got = _run_both(port, ctx, r, g, seed=11)
        diff = routines.compare(r, g, got, want)
        assert max(diff.values()) == 0, diff
        np.testing.assert_allclose(e_got, e_want, rtol=1e-12, atol=0)
    finally:
        ctx.close()


@pytest.mark.parametrize("other", ["planes", "pencil"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_dts_schedules_agree(precision, other, cuda_lib):
    """The schedules agree in the contracted and FP32 builds to the
    rounding of those builds (FMA contraction may pair the per-direction
    sums differently in different kernels)."""
    import channel_flow_gb300 as cf
    r = routines.BY_NAME["Dual_time_stepping"]
    dims = (13, 9, 17)
    g = cases.grid(dims)
    outs = []
    for schedule in ("wavefront", other):
        ctx = cf.Context(g, precision=precision)
        try:
            ctx.set_lu_schedule(schedule)
            a = cases.copy_case(r.build(g, 4))
            er = routines.run_gpu(ctx, r, a)
            outs.append((a, er))
        finally:
            ctx.close()
    (a0, e0), (a1, e1) = outs
    tol = RTOL_FP64 if precision == "fp64" else 1e-5
    for i in r.outputs:
        scale = max(float(np.max(np.abs(a1[i]))), 1e-300)
        assert float(np.max(np.abs(a0[i] - a1[i]))) / scale <= tol, i
    np.testing.assert_allclose(np.asarray(e0), np.asarray(e1), rtol=tol * 10, atol=0)


@pytest.mark.parametrize("name", [r.name for r in routines.ROUTINES])
def test_gpu_exact_equals_oracle_config0_grid(name, port, cuda_lib):
    """Every routine at the 64^3 grid of the CPU-runnable configuration
    (many wavefront tiles, grids of several waves, the filter's full
    level sizes), no-FMA build against the oracle: bit for bit on every
    written array and every face, norms to 1e-12, tanh/cosh metrics to
    1e-13."""
    import channel_flow_gb300 as cf
    r = routines.BY_NAME[name]
    g = cases.grid(CONFIG0_GRID)
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        want, got, e_want, e_got = _run_both(port, ctx, r, g, seed=17)
    finally:
        ctx.close()
    if r.libm:
        diff = routines.compare(r, g, got, want, rtol=1)
        assert max(diff.values()) <= 1e-13, diff
    else:
        diff = routines.compare(r, g, got, want)
        assert all(v == 0 for v in diff.values()), f"{name}: differing entries per slot {diff}"
    if r.scalars:
        np.testing.assert_allclose(e_got, e_want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ["Flux_Y_limiter", "Flux_Z_limiter"])
def test_gpu_consistent_exact_equals_oracle_config0_grid(name, port, cuda_lib):
    """The consistent face-state scaling at 64^3, no-FMA build, bit for bit."""
    import channel_flow_gb300 as cf
    r = routines.BY_NAME[name]
    g = cases.grid(CONFIG0_GRID)
    a = r.build(g, 19)
    want, got = cases.copy_case(a), cases.copy_case(a)
    routines.run_cpu(port, r, g, want, scheme="consistent")
    ctx = cf.Context(g, precision="fp64_exact", scheme="consistent")
    try:
        routines.run_gpu(ctx, r, got)
    finally:
        ctx.close()
    diff = routines.compare(r, g, got, want)
    assert all(v == 0 for v in diff.values()), diff


@pytest.mark.parametrize("dims", cases.GRIDS + [(13, 9, 17), CONFIG0_GRID])
def test_gpu_hyperplane_tables_equal_oracle(dims, port, cuda_lib):
    """cf_Hyperplane's plane tables Nijk and ijk (Hyperplane.cpp:50-78)
    equal the oracle's, whose tables equal the reference's."""
    import channel_flow_gb300 as cf
    g = cases.grid(dims)
    ctx = cf.Context(g, precision="fp64_exact")
    try:
        n_gpu, i_gpu = ctx.Hyperplane()
    finally:
        ctx.close()
    n_cpu, i_cpu = port.Hyperplane(g)
    assert np.array_equal(n_gpu, n_cpu) and np.array_equal(i_gpu, i_cpu)
