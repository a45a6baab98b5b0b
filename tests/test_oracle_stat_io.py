"""The C oracle's Statistic and restart image against the reference's own
Statistic, Output and Initial_condition (compiled from the reference
sources).  The reference writes its results to files in the current
directory; its printed values (%.16f) must equal the oracle's values
printed the same way, and the restart files byte for byte."""
import os

import numpy as np
import pytest

import cases
from oracle import cforacle

pytestmark = pytest.mark.skipif(not cforacle.reference_available(),
                                reason="reference sources not present on this machine")


def _read_blocks(path, nblocks, n):
    vals = [line.strip() for line in open(path) if line.strip()]
    assert len(vals) == nblocks * n, (path, len(vals))
    return [vals[b * n:(b + 1) * n] for b in range(nblocks)]


@pytest.mark.parametrize("dims", cases.GRIDS)
@pytest.mark.parametrize("stat_step", [1, 2])
def test_statistic_port_equals_reference(dims, stat_step, port, tmp_path, monkeypatch):
    g = cases.grid(dims)
    ref = cforacle.Reference(g)
    monkeypatch.chdir(tmp_path)
    acc = port.statistic_state(g)
    ny = g.ny
    for step in range(1, stat_step + 1):
        a = cases.statistic_case(g, seed=step)
        want, got = cases.copy_case(a), cases.copy_case(a)
        ref.Statistic(step, 3, stat_step, want)
        wrote, shear, nd, st = port.Statistic(g, acc, step, 3, stat_step, got)
        # the scratch the routine writes (ML, MR) equals the reference's
        for i in range(16, 26):
            assert np.array_equal(got[i], want[i], equal_nan=True), i
        lines = [l.split() for l in open(tmp_path / "Shear_stress.dat")]
        assert lines[-1] == ["%f" % shear[0], "%f" % shear[1]]
    assert wrote
    ndf = _read_blocks(tmp_path / ("ND%05d.dat" % stat_step), 10, ny)
    stf = _read_blocks(tmp_path / ("st%05d.dat" % stat_step), 7, ny - 1)
    for b in range(10):
        assert ndf[b] == ["%.16f" % v for v in nd[b, 1:ny + 1]], b
    for b in range(7):
        assert stf[b] == ["%.16f" % v for v in st[b, 2:ny + 1]], b


@pytest.mark.parametrize("dims", cases.GRIDS)
def test_restart_image_equals_reference(dims, port, tmp_path, monkeypatch):
    g = cases.grid(dims)
    ref = cforacle.Reference(g)
    monkeypatch.chdir(tmp_path)
    a = cases.restart_case(g, seed=4)
    ref.Output(7, cases.copy_case(a))
    img = port.restart_pack(g, a)
    assert (tmp_path / "LES00007.bin").read_bytes() == img.tobytes()
    # Initial_condition reads initial.bin back into U and Uq
    (tmp_path / "initial.bin").write_bytes(img.tobytes())
    z = [np.zeros(g.shape) for _ in range(15)]
    want = z[:5] + [x.copy() for x in z[5:]] + [a[10]]
    got = [x.copy() for x in z] + [a[10]]
    ref.Initial_condition(want)
    port.restart_unpack(g, img, got)
    for i in range(15):
        assert np.array_equal(want[i], got[i]), i
