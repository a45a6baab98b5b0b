"""Exact floating-point operation counts of the CPU oracle (test
infrastructure).

``flop_count.cpp`` compiles the oracle's C sources as C++ with every double
replaced by a counting wrapper (same layout, same results, serial), into
``oracle/_build/libcfoflops.so``.  ``Counter`` is a ``cforacle.Port`` on that
library: call a routine through it, then ``read()`` returns the operations
the call performed.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

from . import cforacle

KINDS = ("add", "mul", "div", "sqrt", "libm")
SOURCES = ["flop_count.cpp", "cf_oracle_flux.c", "cf_oracle_visc.c", "cf_oracle_filter.c", "cf_oracle_lusgs.c",
           "cf_oracle.h", "cf_oracle_common.h"]


def build(force: bool = False):
    lib = cforacle.BUILD / "libcfoflops.so"
    srcs = [cforacle.HERE / s for s in SOURCES]
    with cforacle._lock:
        if not force and lib.exists() and all(lib.stat().st_mtime >= s.stat().st_mtime for s in srcs):
            return lib
        cforacle.BUILD.mkdir(exist_ok=True)
        tmp = cforacle.BUILD / f"libcfoflops.{os.getpid()}.tmp"
        # -fpermissive: the C sources assign calloc's void * without a cast
        cmd = ["g++", "-O1", "-std=gnu++17", "-fpermissive", "-w", "-ffp-contract=off", "-fPIC", "-shared",
               "-o", str(tmp), str(srcs[0]), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"flop-count build failed:\n{r.stderr[-4000:]}")
        tmp.rename(lib)
    return lib


class Counter(cforacle.Port):
    def __init__(self):
        self.lib = C.CDLL(str(build()))

    def reset(self):
        self.lib.cfo_flops_reset()

    def read(self) -> dict:
        out = (C.c_ulonglong * 5)()
        self.lib.cfo_flops_read(out)
        return dict(zip(KINDS, (int(v) for v in out)))
