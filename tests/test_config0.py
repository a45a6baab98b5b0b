"""The 64^3 plain-FP64 schedule fixture (tests/golden/config0_64_run.json):
the inputs rebuilt from it give the oracle's first step as recorded (Q of
Driven_force bit for bit), so the GPU run of the schedule starts from the
state the oracle started from."""
import numpy as np

import cases


def test_config0_fixture_reproduces_first_step(port):
    g, f, meta = cases.config0_case()
    assert g.shape == (70, 68, 68)
    E = [0.0] * 5
    it, er, Q = cases.port_step(port, g, f, meta["deltaT_value"], meta["subiterations"], 0.0, E,
                                scheme=meta["scheme"])
    assert it == meta["subiterations"]
    assert float(Q) == float.fromhex(meta["Q"][0])
    assert all(np.isfinite(a).all() for a in f["U"])
