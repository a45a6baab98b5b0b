"""Exact operation counts of the oracle's restatement (oracle/flop_count.cpp):
the counting build computes the same results as the oracle, and its counts
on the seeded cases equal the committed fixture (tests/golden/flop_counts.json,
made by tests/golden/make_flop_counts.py)."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

import cases
import routines

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_flop_counts as mfc  # noqa: E402


@pytest.fixture(scope="module")
def counter():
    from oracle.flopcount import Counter
    return Counter()


@pytest.mark.parametrize("name", ["Flux_Y_limiter", "Viscous_terms", "Filter", "Dual_time_stepping"])
def test_counting_build_computes_the_oracle(port, counter, name):
    r = routines.BY_NAME[name]
    g = cases.grid((16, 12, 8))
    a = r.build(g, 3)
    b = [x.copy() for x in a]
    ea = routines.run_cpu(port, r, g, a)
    eb = routines.run_cpu(counter, r, g, b)
    for s in r.outputs:
        assert np.array_equal(a[s], b[s], equal_nan=True), (name, s)
    if ea is not None:
        assert np.array_equal(ea, eb)


def test_counts_match_fixture(counter):
    want = json.loads(mfc.FIXTURE.read_text())
    got = mfc.count(counter)
    assert got["grid"] == want["grid"] and got["cells"] == want["cells"]
    for name, w in want["routines"].items():
        g = got["routines"][name]
        for k in ("add", "mul", "div", "sqrt", "libm"):
            assert g[k] == w[k], (name, k)


def test_counts_scale_with_the_grid(counter):
    """Per-cell counts are grid-independent up to the wall and seam faces:
    halving every extent changes them by under 15 %, and the smaller grid,
    with more boundary faces per cell, does not count fewer (to rounding of
    the per-cell quotient's data-dependent branches)."""
    names = ["Flux_X_limiter", "Viscous_terms", "Filter", "Dual_time_stepping"]
    a = mfc.count(counter, dims=(16, 12, 8), names=names)["routines"]
    b = mfc.count(counter, dims=(32, 24, 16), names=names)["routines"]
    for name in a:
        r = a[name]["flops_per_cell"] / b[name]["flops_per_cell"]
        assert 0.999 <= r < 1.15, (name, r)


def test_bench_flop_constants_match_fixture():
    """The benchmark's FP64 roofline uses these counts per cell."""
    import bench
    want = json.loads(mfc.FIXTURE.read_text())["routines"]
    for name, v in bench.ALG_FLOPS_PER_CELL.items():
        assert abs(v - want[name]["flops_per_cell"]) < 0.05, name
