"""Build recipe for the reference-solver oracle library (test infrastructure).

Compiles the reference's own routine sources IN PLACE from the read-only
reference checkout (default ``/root/reference``, override with
``CF_REFERENCE_DIR``) into ``oracle/_ref/<tag>/libcfref.so``, one build per
grid because the reference fixes its grid at compile time.  Nothing is copied
out of the reference tree; the only generated file is the grid header
``Resolution.h`` written into the per-grid build directory.

Include order (GCC ``-I-``): quoted includes look first in the per-grid
directory (``Resolution.h``) and in ``oracle/ref_overrides`` (``MPI_prm.h``
with one rank), then in the reference tree; ``<mpi.h>`` resolves to the
single-rank stand-in.  ``-I-`` also stops GCC from searching the reference
directory first for quoted includes, which is what lets the generated grid
header replace the reference's 96x128x72 one without editing any source.

Flags: ``-O2 -fopenmp -ffp-contract=off``: IEEE double arithmetic with no
fused multiply-add, so the C restatement in ``cf_oracle.c`` (built with the
same contraction rule) can be compared bit for bit.

Usage::

    python oracle/build_ref.py 12 10 8          # X_out Y_out Z_out
    python oracle/build_ref.py 128 128 128 --lx 0.0157 --lz 0.0079
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import math
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OVERRIDES = HERE / "ref_overrides"
REF_OUT = HERE / "_ref"

# Reference sources on the hot path and its set-up (X_boundary_condition.cpp
# does not compile: it uses undeclared X_memory/Y_memory/Z_memory; main.cpp
# is replaced by ref_harness.cpp).
SOURCES = [
    "Y_boundary_condition.cpp", "Z_boundary_condition.cpp",
    "Flux_X.cpp", "Flux_Y.cpp", "Flux_Z.cpp",
    "Flux_X_limiter.cpp", "Flux_Y_limiter.cpp", "Flux_Z_limiter.cpp",
    "Viscous_terms.cpp", "Filter.cpp", "RK3NODT.cpp",
    "Dual_time_stepping.cpp", "DPLUSGS.cpp", "Hyperplane.cpp",
    "Grid.cpp", "Jacobian.cpp", "Jacobian_u.cpp", "Jacobian_v.cpp", "Jacobian_w.cpp",
    "Driven_force.cpp", "Statistic.cpp", "Output.cpp", "Initial_condition.cpp",
]


def reference_dir() -> Path:
    return Path(os.environ.get("CF_REFERENCE_DIR", "/root/reference"))


def default_deltas(X_out: int, Y_out: int, Z_out: int, high: float = 0.005,
                   lx: float | None = None, lz: float | None = None):
    """Reference conventions (Resolution.h:13-15): deltaXI = Lx/X_out with
    Lx = 4*pi*(high/2), deltaET = 1/Y_out (normalised wall-normal
    coordinate), deltaZT = Lz/Z_out with Lz = 2*pi*(high/2)."""
    h = 0.5 * high
    lx = 4.0 * math.pi * h if lx is None else lx
    lz = 2.0 * math.pi * h if lz is None else lz
    return lx / X_out, 1.0 / Y_out, lz / Z_out


def grid_tag(X_out, Y_out, Z_out, dxi, det, dzt) -> str:
    return f"g{X_out}x{Y_out}x{Z_out}_{dxi.hex()}_{det.hex()}_{dzt.hex()}".replace(".", "p").replace("+", "")


def resolution_header(X_out, Y_out, Z_out, dxi, det, dzt) -> str:
    # Same macro set and the same unparenthesised style as the reference
    # header, so every expression in the routines expands identically.
    return f"""/* generated by oracle/build_ref.py */
#define X_out {X_out}
#define Y_out {Y_out}
#define Z_out {Z_out}

#define X_m {X_out + 4}
#define Y_m {Y_out + 4}
#define Z_m {Z_out + 4}

#define nx X_out+1
#define ny Y_out+1
#define nz Z_out+1

#define deltaXI {dxi!r}
#define deltaET {det!r}
#define deltaZT {dzt!r}

#define nxx nx+1
#define nyy ny+1
#define nzz nz+1

#define nxxx nxx+1
#define nyyy nyy+1
#define nzzz nzz+1
"""


def build(X_out: int, Y_out: int, Z_out: int, deltas=None, jobs: int = 8,
          verbose: bool = False) -> Path:
    """Compile the reference routines for one grid; return the .so path.
    Rebuilds when the library is missing or older than the harness, the
    stand-in headers or this recipe."""
    ref = reference_dir()
    if not (ref / "Flux_X_limiter.cpp").exists():
        raise FileNotFoundError(f"reference sources not found under {ref}")
    dxi, det, dzt = deltas if deltas is not None else default_deltas(X_out, Y_out, Z_out)
    out = REF_OUT / grid_tag(X_out, Y_out, Z_out, dxi, det, dzt)
    lib = out / "libcfref.so"
    deps = [HERE / "ref_harness.cpp", Path(__file__)] + sorted(OVERRIDES.rglob("*.h"))
    if lib.exists() and all(lib.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return lib
    out.mkdir(parents=True, exist_ok=True)
    (out / "Resolution.h").write_text(resolution_header(X_out, Y_out, Z_out, dxi, det, dzt))
    inc = [f"-I{out}", f"-I{OVERRIDES}", "-I-", f"-I{OVERRIDES}", f"-I{ref}"]
    flags = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-w", "-std=gnu++14"]

    def cc(src: Path) -> Path:
        obj = out / (src.stem + ".o")
        cmd = ["g++", *flags, *inc, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")
        return obj

    def cc_defined(src: Path) -> Path:
        # second build of DPLUSGS.cpp with its two unassigned indices defined
        # (see ref_overrides/dplusgs_defined.h)
        obj = out / "DPLUSGS_defined.o"
        inc_d = [f"-I{out}", f"-I{OVERRIDES / 'defined_indices'}", f"-I{OVERRIDES}", "-I-",
                 f"-I{OVERRIDES}", f"-I{ref}"]
        fl = [f for f in flags if f != "-fopenmp"]
        cmd = ["g++", *fl, "-include", str(OVERRIDES / "dplusgs_defined.h"), *inc_d,
               "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")
        return obj

    srcs = [ref / s for s in SOURCES] + [HERE / "ref_harness.cpp"]
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(cc, s) for s in srcs] + [ex.submit(cc_defined, ref / "DPLUSGS.cpp")]
        objs = [f.result() for f in futs]
    tmp = out / "libcfref.so.tmp"
    cmd = ["g++", "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {r.stderr[-4000:]}")
    for o in objs:
        o.unlink()
    tmp.rename(lib)
    if verbose:
        print(lib)
    return lib


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("X_out", type=int)
    ap.add_argument("Y_out", type=int)
    ap.add_argument("Z_out", type=int)
    ap.add_argument("--lx", type=float, default=None)
    ap.add_argument("--lz", type=float, default=None)
    a = ap.parse_args(argv)
    d = default_deltas(a.X_out, a.Y_out, a.Z_out, lx=a.lx, lz=a.lz)
    print(build(a.X_out, a.Y_out, a.Z_out, d, verbose=False))


if __name__ == "__main__":
    sys.exit(main())
