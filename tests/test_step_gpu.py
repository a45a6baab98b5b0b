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


def _routine_loop(ctx, dev, deltaT, max_iterations, tolerance, E, limiter=True, filt=True):
    """One physical step composed of the drop-in routine calls (FP64
    arrays between them), in the context's precision: the loop of cf_step
    written out.  E (running maxima) is updated in place."""
    import torch
    U_, J = dev["U_"], dev["J"]
    Nijk, ijk = ctx.Hyperplane()
    names = ("Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter") if limiter else ("Flux_X", "Flux_Y", "Flux_Z")
    visc = [None] * 79
    visc[0:5] = U_
    visc[5:9] = dev["vF"]
    visc[9] = J
    visc[10:19] = dev["cell_metric"]
    for s in range(3):
        visc[19 + 10 * s] = dev["face_J"][s]
        visc[20 + 10 * s:29 + 10 * s] = dev["face_metric"][s]
    visc[55:59] = dev["LL"]
    visc[65:69] = dev["ML"]
    visc[75:79] = dev["NL"][1:5]
    dts = U_ + dev["U"] + dev["Uq"] + [J] + dev["cell_metric"] + dev["inF"][0] + dev["inF"][1] + dev["inF"][2] + \
        dev["vF"] + dev["MR"] + dev["NR"] + dev["NL"] + dev["Residual"]
    it = 0
    while True:
        it += 1
        ctx.X_periodic(*U_)
        ctx.Y_boundary_condition(*U_, J)
        ctx.Z_boundary_condition(*U_, J)
        if filt:
            ctx.Filter(0.007, 1.0, 0.0, *U_, dev["Y_point"], *dev["Ep"], J)
        for d in range(3):
            ctx.flux(names[d], U_ + [None] * 10 + [J, dev["face_J"][d]] + dev["face_metric"][d] + dev["inF"][d] +
                     [dev["Ep"][d]])
        ctx.Viscous_terms(*visc)
        er = ctx.Dual_time_stepping(deltaT, *dts, Nijk=Nijk, ijk=ijk)
        for n in range(5):
            E[n] = max(E[n], er[n])
        ern = [er[n] / E[n] for n in range(5)]
        if all(ern[n] < tolerance for n in range(4)) or it >= max_iterations:
            break
    q, _ = ctx.Driven_force(dev["U"][1], J)
    g = ctx.grid
    box = (slice(3, g.gend + 1), slice(2, g.ny + 1), slice(2, g.nz + 1))
    for n in range(5):
        dev["Uq"][n][box] = dev["U"][n][box]
        dev["U"][n][box] = U_[n][box]
    torch.cuda.synchronize()
    return it, np.array(ern), q


@pytest.mark.parametrize("static_metrics", [False, True])
def test_gpu_fp32_step_equals_routine_loop(static_metrics, cuda_lib):
    """In FP32 the step driver passes its intermediate arrays as FP32 values
    and (static_metrics) reads FP32 copies of the fixed metrics; the drop-in
    routines exchange FP64 arrays.  Every FP32 value is exact in FP64, so
    with the same kernels the two give the same state bit for bit.  With
    static metrics the step driver runs the kernels compiled for its FP32
    layout (namespace cf_drv), whose FP32 instruction selection differs:
    the two then agree to FP32 rounding (the same iteration counts, norms
    to 1e-3, states to 1e-3 of their change over the steps)."""
    import channel_flow_gb300 as cf
    g = cases.grid((13, 9, 17))
    f = cases.step_case(g, seed=5)
    a, b = _to_dev(f), _to_dev(f)
    start = [u.clone() for u in a["U"]]
    ctx_a = cf.Context(g, precision="fp32")
    ctx_b = cf.Context(g, precision="fp32")
    bitwise = not static_metrics
    try:
        E = [0.0] * 5
        for step in (1, 2):
            it_a, er_a, q_a = ctx_a.step(a, step=step, max_iterations=3, tolerance=1e-3,
                                         static_metrics=static_metrics)
            it_b, er_b, q_b = _routine_loop(ctx_b, b, 0.00000005, 3, 1e-3, E)
            assert it_a == it_b
            np.testing.assert_allclose(er_a, er_b, rtol=1e-12 if bitwise else 1e-3, atol=0)
            assert abs(q_a - q_b) <= (1e-12 if bitwise else 1e-6) * abs(q_b)
        for key in ("U_", "U", "Uq"):
            for n in range(5):
                x, y = a[key][n].cpu().numpy(), b[key][n].cpu().numpy()
                if bitwise:
                    assert np.array_equal(x, y, equal_nan=True), (key, n)
                else:
                    change = float((b[key][n] - start[n]).abs().max())
                    assert float(np.max(np.abs(x - y))) <= 1e-3 * change, (key, n)
    finally:
        ctx_a.close()
        ctx_b.close()


def test_gpu_fp32_static_metrics_first_step_after_poisoned_memory(cuda_lib):
    """The first FP32 step with static metrics makes the FP32 metric copies;
    Flux_Y/Flux_Z (side stream) and the viscous terms (main stream) both
    read the y- and z-face copies, so they must exist before the loop forks.
    Device memory is first filled with NaN and released, so a read of a copy
    before it is written shows as NaN.  On the 256 x 192 x 192 channel one
    sub-iteration with the copies equals one without them to FP32 rounding,
    and every value of the state is finite."""
    import torch
    import channel_flow_gb300 as cf
    from channel_flow_gb300 import stepper, synthetic as syn
    import bench

    g = syn.channel_physics(syn.channel_grid(256, 192, 192), 0.5, 5600)
    cm = syn.flat_metrics(g, 2.0, "cell")
    host = {"U": syn.channel_state(g, cm["J"], seed=2800, gamma=2.0, wall_damped=True), "J": cm["J"],
            "cm": [cm[n] for n in syn.METRIC_NAMES], "Yp": syn.y_points(g, gamma=2.0)}
    dt = syn.time_step(g, 0.5) / 4
    ers = {}
    for static in (True, False):
        x = torch.full((2 ** 30,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        del x
        torch.cuda.empty_cache()
        ctx = cf.Context(g, precision="fp32", gamma=2.0, scheme="consistent")
        try:
            w = bench.DeviceWorkload(ctx, g, host, torch)
            f = stepper.fields_from_workload(w, torch, g)
            ctx.step_reset()
            ctx.step(f, step=1, deltaT=dt, max_iterations=2, tolerance=1e-9, limiter=True, filter="per_step",
                     static_metrics=static)
            assert all(bool(torch.isfinite(u).all()) for u in f["U_"]), static
            ers[static] = ctx.step_residuals()
        finally:
            ctx.close()
        del w, f
        torch.cuda.empty_cache()
    np.testing.assert_allclose(ers[True], ers[False], rtol=1e-3, atol=0)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_step_statistic_beside_next_step(precision, cuda_lib, tmp_path):
    """cf_step's Statistic adds the rows of a copy of the final U_ on a
    stream of its own, beside the next call's work, and its host part waits
    for the next flush.  Three steps with statistic_step 2 (step 2 writes the
    ND/st files and clears the accumulators) give the same files and
    accumulators, bit for bit, as the same steps without the Statistic
    followed each by the drop-in cf_Statistic on U_."""
    import channel_flow_gb300 as cf
    import torch
    g = cases.grid((13, 9, 17))
    f = cases.step_case(g, seed=5)
    a, b = _to_dev(f), _to_dev(f)
    da, db = tmp_path / "a", tmp_path / "b"
    da.mkdir()
    db.mkdir()
    ctx_a = cf.Context(g, precision=precision)
    ctx_b = cf.Context(g, precision=precision)
    try:
        ctx_a.set_output_dir(str(da))
        ctx_b.set_output_dir(str(db))
        scratch = [torch.zeros_like(b["J"]) for _ in range(10)]
        for step in (1, 2, 3):
            ctx_a.step(a, step=step, max_iterations=2, tolerance=1e-3, statistic_step=2)
            ctx_b.step(b, step=step, max_iterations=2, tolerance=1e-3, statistic_step=0)
            ctx_b.Statistic(step, 0, 2, *b["U_"], b["J"], b["face_J"][1], *b["face_metric"][1], *scratch,
                            b["Ep"][1])
        got = ctx_a.statistic_read()          # flushes step 3's host part first
        want = ctx_b.statistic_read()
        assert np.array_equal(got, want)
        assert np.any(got[:17 * (g.Y_out + 4)])   # step 3 accumulated after the clearing at step 2
        for name in ("Shear_stress.dat", "ND00002.dat", "st00002.dat"):
            assert (da / name).read_bytes() == (db / name).read_bytes(), name
        assert len((da / "Shear_stress.dat").read_text().splitlines()) == 3
        for key in ("U_", "U", "Uq"):
            for n in range(5):
                assert torch.equal(a[key][n], b[key][n]), (key, n)
    finally:
        ctx_a.close()
        ctx_b.close()
