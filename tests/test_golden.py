"""The C oracle against the golden fixture made from the reference solver
(tests/golden/make_golden.py): digests of every written array must match
bit for bit; routines that call tanh/cosh match to 1e-14 along a line."""
import json
from pathlib import Path

import numpy as np
import pytest

import cases
import routines

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_outputs.json").read_text())


def check_against_golden(r, g, arrays, er, seed):
    rec = GOLDEN["routines"][r.name][str(seed)]
    if r.libm:
        for i in r.outputs:
            want = np.array([float.fromhex(x) for x in rec["lines"][str(i)]])
            np.testing.assert_allclose(arrays[i][3, :, 3], want, rtol=1e-14, atol=0)
        return
    for i in r.outputs:
        assert cases.digest(arrays[i], r.mask(g, i)) == rec["digests"][str(i)], f"{r.name} slot {i}"
    if "er" in rec:
        assert [float(x).hex() for x in er] == rec["er"]


@pytest.mark.parametrize("seed", GOLDEN["seeds"])
@pytest.mark.parametrize("name", [r.name for r in routines.ROUTINES])
def test_port_matches_golden(name, seed, port):
    r = routines.BY_NAME[name]
    g = cases.grid(tuple(GOLDEN["grid"]))
    a = r.build(g, seed)
    er = routines.run_cpu(port, r, g, a)
    check_against_golden(r, g, a, er, seed)


def test_golden_covers_every_routine():
    assert set(GOLDEN["routines"]) == {r.name for r in routines.ROUTINES}
