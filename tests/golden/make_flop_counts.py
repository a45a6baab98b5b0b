"""Generate flop_counts.json: the exact floating-point operations that the
CPU oracle's restatement of each hot-path routine performs on the seeded
cases of tests/cases.py (oracle/flop_count.cpp counts every add/subtract,
multiply, divide, sqrt and libm call), in total and per interior cell.

The counts depend on the data only through the branches (limiter cases,
the filter threshold, wall and seam stencils), and the inputs are rebuilt
bit for bit from the seeds, so the fixture is exact on any machine.

Run from the repository root:  python tests/golden/make_flop_counts.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent))

import cases  # noqa: E402
import routines  # noqa: E402
from oracle.flopcount import Counter  # noqa: E402

DIMS = (64, 48, 32)
SEED = 0
ROUTINES = ["Filter", "Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter", "Flux_X", "Flux_Y", "Flux_Z",
            "Viscous_terms", "RK3NODT", "Dual_time_stepping", "DPLUSGS"]
FIXTURE = HERE / "flop_counts.json"


def count(counter=None, dims=DIMS, names=ROUTINES):
    counter = counter or Counter()
    g = cases.grid(dims)
    cells = dims[0] * dims[1] * dims[2]
    out = {}
    for name in names:
        r = routines.BY_NAME[name]
        arrays = r.build(g, SEED)
        if name == "Dual_time_stepping":
            # the plane tables are set-up work, outside the counted call
            Nijk, ijk = counter.Hyperplane(g)
            counter.reset()
            counter.Dual_time_stepping(g, cases.DELTA_T, Nijk, ijk, arrays)
        else:
            counter.reset()
            routines.run_cpu(counter, r, g, arrays)
        n = counter.read()
        flops = n["add"] + n["mul"] + n["div"] + n["sqrt"]
        out[name] = dict(n, flops=flops, flops_per_cell=flops / cells,
                         div_per_cell=n["div"] / cells, sqrt_per_cell=n["sqrt"] / cells)
    return {"grid": list(dims), "cells": cells, "seed": SEED, "routines": out}


def main():
    data = count()
    FIXTURE.write_text(json.dumps(data, indent=1) + "\n")
    for k, v in data["routines"].items():
        print(f"{k:20s} {v['flops_per_cell']:9.1f} flop/cell  div {v['div_per_cell']:6.1f}  "
              f"sqrt {v['sqrt_per_cell']:5.2f}  libm {v['libm']}")


if __name__ == "__main__":
    main()
