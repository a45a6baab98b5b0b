"""Generate the golden fixture reference_outputs.json from the reference
solver itself (its own routine sources compiled by oracle/build_ref.py).

For every hot-path routine, the seeded case of tests/cases.py on the golden
grid is run through the compiled reference; the fixture stores a SHA-256
digest of every array the routine writes (entries that depend on the
reference's uninitialised variables zeroed first), the residual norms of the
dual-time routines as exact hex floats, and for the two routines that call
tanh/cosh (whose last bits depend on the libm) the written values along one
wall-normal line.

The inputs are regenerated bit for bit from the seeds on any machine, so the
C oracle and the GPU can be checked against these digests where the
reference cannot be compiled.

Run from the repository root:  python tests/golden/make_golden.py
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
from oracle.cforacle import Reference  # noqa: E402

SEEDS = [3, 11]


def main():
    g = cases.grid(cases.GOLDEN_GRID)
    ref = Reference(g)
    out = {"grid": list(cases.GOLDEN_GRID), "seeds": SEEDS, "routines": {}}
    for r in routines.ROUTINES:
        rec = {}
        for seed in SEEDS:
            a = r.build(g, seed)
            er = routines.run_cpu(ref, r, g, a)
            entry = {"digests": {str(i): cases.digest(a[i], r.mask(g, i)) for i in r.outputs}}
            if er is not None:
                entry["er"] = [float(x).hex() for x in er]
            if r.libm:
                entry["lines"] = {str(i): [float(x).hex() for x in a[i][3, :, 3]] for i in r.outputs}
            rec[str(seed)] = entry
        out["routines"][r.name] = rec
    path = HERE / "reference_outputs.json"
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
