"""GPU Statistic, Driven_force and restart IO against the C oracle (which
is pinned to the reference's own Statistic / Output / Initial_condition in
test_oracle_stat_io.py).  Sums are FP64 in every precision mode and differ
from the oracle's serial loops only in summation order (1e-12 relative);
the restart image is exact."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _dev(arrays):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


def _rel(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


@pytest.mark.parametrize("precision", ["fp64_exact", "fp64", "fp32"])
@pytest.mark.parametrize("dims", cases.GRIDS)
def test_gpu_statistic(dims, precision, port, cuda_lib, tmp_path):
    import channel_flow_gb300 as cf
    g = cases.grid(dims)
    ctx = cf.Context(g, precision=precision)
    try:
        ctx.set_output_dir(tmp_path)
        acc = port.statistic_state(g)
        Ym, ny = g.Y_out + 4, g.ny
        for step in (1, 2):
            a = cases.statistic_case(g, seed=step)
            ctx.Statistic(step, 3, 2, *_dev(a))
            wrote, shear, nd, st = port.Statistic(g, acc, step, 3, 2, cases.copy_case(a))
            if step == 1:
                got = ctx.statistic_read()
                for r in range(17):
                    assert _rel(got[r * Ym:(r + 1) * Ym], acc[r * Ym:(r + 1) * Ym]) <= 1e-12, r
            lines = [l.split() for l in open(tmp_path / "Shear_stress.dat")]
            assert len(lines) == step
            np.testing.assert_allclose([float(x) for x in lines[-1]], shear, rtol=1e-5, atol=1e-6)
        assert wrote
        ndf = np.array([float(x) for x in open(tmp_path / "ND00002.dat")]).reshape(10, ny)
        stf = np.array([float(x) for x in open(tmp_path / "st00002.dat")]).reshape(7, ny - 1)
        for b in range(10):
            assert _rel(ndf[b], nd[b, 1:ny + 1]) <= 1e-12, b
        for b in range(7):
            assert _rel(stf[b], st[b, 2:ny + 1]) <= 1e-12, b
        assert not np.any(ctx.statistic_read()[:17 * Ym])      # cleared after the output step
    finally:
        ctx.close()


@pytest.mark.parametrize("dims", cases.GRIDS)
def test_gpu_driven_force(dims, port, cuda_lib):
    import channel_flow_gb300 as cf
    g = cases.grid(dims)
    ctx = cf.Context(g, precision="fp64")
    try:
        U, J = cases.state(g, 9)
        q, er = ctx.Driven_force(*_dev([U[1], J]))
        want = port.Driven_force(g, U[1], J)
        assert abs(q - want) <= 1e-12 * abs(want)
        assert abs(er - abs(g.Q0 - want) / g.Q0) <= 1e-12 * max(er, 1e-300) + 1e-15
    finally:
        ctx.close()


@pytest.mark.parametrize("dims", cases.GRIDS)
def test_gpu_restart_roundtrip(dims, port, cuda_lib, tmp_path):
    import channel_flow_gb300 as cf
    g = cases.grid(dims)
    ctx = cf.Context(g, precision="fp64")
    try:
        ctx.set_output_dir(tmp_path)
        a = cases.restart_case(g, seed=6)
        ctx.Output(12, *_dev(a))
        img = port.restart_pack(g, a)
        assert (tmp_path / "LES00012.bin").read_bytes() == img.tobytes()
        (tmp_path / "initial.bin").write_bytes(img.tobytes())
        z = [np.zeros(g.shape) for _ in range(15)]
        dev = _dev(z + [a[10]])
        ctx.Initial_condition(*dev)
        want = [x.copy() for x in z] + [a[10]]
        port.restart_unpack(g, img, want)
        for i in range(15):
            assert np.array_equal(dev[i].cpu().numpy(), want[i]), i
    finally:
        ctx.close()
