"""Build the CUDA library ``channel_flow_gb300/libcfgb300.so`` (sm_103a).

Translation units, compiled in parallel with nvcc:

* ``cf_variant.cu`` as namespace ``cf_exact`` with ``--fmad=false``: the FP64
  kernels without fused multiply-add, whose results equal the reference's
  bit for bit;
* ``cf_variant.cu`` as namespace ``cf_fast`` with contraction on, the
  reduced-division face fluxes (CF_FAST_MATH) and the FP32 instantiations,
  whose divisions and square roots take the approximate hardware forms
  (``-prec-div=false -prec-sqrt=false``; these flags leave FP64 alone);
* ``cf_variant.cu`` as namespace ``cf_drv``: the ``cf_fast`` kernels with
  the step driver's FP32 array layout fixed at compile time (CF_STEP_LAYOUT);
* ``cf_api.cu``: the C-ABI layer (include/channel_flow_gb300.h);
* ``cf_noalloc.cu``: the allocation-free DPLUSGS entry point (its scratch is
  a file-scope device array);
* ``cf_mlp.cu``: the learned initial guess (tcgen05 BF16 GEMMs, TMA) and
  its training kernels;
* ``cf_metrics.cu``: the wavy-wall metric generator (no FMA contraction).

Usage: ``python -m channel_flow_gb300.build [--verbose] [--ptxas]``
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "libcfgb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        [PKG.parent / "include" / "channel_flow_gb300.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources())


def build(verbose: bool = False, ptxas: bool = False, force: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    out = PKG / "_build"
    out.mkdir(exist_ok=True)
    base = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "--expt-relaxed-constexpr", f"-I{CSRC}"]
    if ptxas:
        base += ["-Xptxas", "-v"]
    units = [
        ("cf_variant.cu", "cf_exact.o", ["-DCF_NS=cf_exact", "--fmad=false"]),
        ("cf_variant.cu", "cf_fast.o", ["-DCF_NS=cf_fast", "-DCF_WITH_FLOAT", "-DCF_FAST_MATH", "--fmad=true",
                                         "-prec-div=false", "-prec-sqrt=false"]),
        ("cf_variant.cu", "cf_drv.o", ["-DCF_NS=cf_drv", "-DCF_WITH_FLOAT", "-DCF_FAST_MATH", "-DCF_STEP_LAYOUT",
                                         "--fmad=true", "-prec-div=false", "-prec-sqrt=false"]),
        ("cf_api.cu", "cf_api.o", ["-DCF_NS=cf_api_unused"]),
        ("cf_noalloc.cu", "cf_noalloc.o", ["-DCF_NS=cf_noalloc", "--fmad=false"]),
        ("cf_mlp.cu", "cf_mlp.o", []),
        ("cf_metrics.cu", "cf_metrics.o", ["--fmad=false"]),
    ]

    def cc(u):
        src, obj, extra = u
        cmd = base + extra + ["-c", str(CSRC / src), "-o", str(out / obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({src} {' '.join(extra)}):\n{r.stderr[-6000:]}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=6) as ex:
        logs = list(ex.map(cc, units))
    if verbose or ptxas:
        for log in logs:
            sys.stderr.write(log)
    tmp = PKG / f"libcfgb300.{os.getpid()}.tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp)] + [str(out / u[1]) for u in units] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser(description="build libcfgb300.so for sm_103a")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print register/spill usage (-Xptxas -v)")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build(a.verbose, a.ptxas, a.force))


if __name__ == "__main__":
    main()
