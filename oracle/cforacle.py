"""ctypes front end of the CPU oracle (test infrastructure).

Two libraries share one calling convention (grid description + list of
field pointers in the reference routine's argument order):

* ``Port``: the C restatement in this directory (``cf_oracle_*.c``), built
  into ``oracle/_build/libcforacle.so`` with ``-O2 -fopenmp
  -ffp-contract=off``.  It exists on every machine that has gcc.
* ``Reference``: the reference solver's own sources compiled per grid by
  ``build_ref.py`` into ``oracle/_ref``; only where the reference checkout
  exists.

Only tests, ``__graft_entry__.smoke`` and the bench's CPU-baseline arm use
this module, as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
PORT_SOURCES = ["cf_oracle_flux.c", "cf_oracle_visc.c", "cf_oracle_filter.c", "cf_oracle_lusgs.c",
                "cf_oracle_stat.c", "cf_oracle_io.c"]
_lock = threading.Lock()


class cfo_grid(C.Structure):
    _fields_ = [("X_out", C.c_int), ("Y_out", C.c_int), ("Z_out", C.c_int),
                ("deltaXI", C.c_double), ("deltaET", C.c_double), ("deltaZT", C.c_double),
                ("K", C.c_double), ("R", C.c_double), ("e", C.c_double),
                ("Cv", C.c_double), ("mu_L", C.c_double), ("Pr_L", C.c_double),
                ("f", C.c_double), ("high", C.c_double), ("scheme", C.c_int)]

# limited-flux face-state scaling (cfo_grid.scheme)
SCHEMES = {"reference": 0, "consistent": 1}


def grid_struct(g, scheme: str = "reference") -> cfo_grid:
    return cfo_grid(g.X_out, g.Y_out, g.Z_out, g.deltaXI, g.deltaET, g.deltaZT,
                    g.K, g.R, g.e, g.Cv, g.mu_L, g.Pr_L, g.f, g.high, SCHEMES[scheme])


def build_port(force: bool = False) -> Path:
    """Compile the C restatement (seconds).  Rebuilds when a source is newer."""
    lib = BUILD / "libcforacle.so"
    srcs = [HERE / s for s in PORT_SOURCES]
    with _lock:
        if not force and lib.exists() and all(lib.stat().st_mtime >= s.stat().st_mtime for s in
                                              srcs + [HERE / "cf_oracle.h", HERE / "cf_oracle_common.h"]):
            return lib
        BUILD.mkdir(exist_ok=True)
        tmp = BUILD / f"libcforacle.{os.getpid()}.tmp"
        cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11",
               "-Wall", "-Wno-unused-variable", "-o", str(tmp), *map(str, srcs), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr[-4000:]}")
        tmp.rename(lib)
    return lib


def _ptrs(arrays):
    for x in arrays:
        assert x.dtype == np.float64 and x.flags["C_CONTIGUOUS"], "oracle fields are C-contiguous float64"
    return (C.POINTER(C.c_double) * len(arrays))(*[x.ctypes.data_as(C.POINTER(C.c_double)) for x in arrays])


class Port:
    """The C restatement; every method mirrors one reference routine."""

    def __init__(self):
        self.lib = C.CDLL(str(build_port()))

    def _call(self, name, g, arrays, *scalars, scheme="reference"):
        fn = getattr(self.lib, "cfo_" + name)
        gs = grid_struct(g, scheme)
        fn(C.byref(gs), *scalars, _ptrs(arrays))

    def x_periodic(self, g, U):
        self._call("x_periodic", g, U)

    def Y_boundary_condition(self, g, arrays):
        self._call("Y_boundary_condition", g, arrays)

    def Z_boundary_condition(self, g, arrays):
        self._call("Z_boundary_condition", g, arrays)

    def flux(self, name, g, arrays, scheme="reference"):
        self._call(name, g, arrays, scheme=scheme)

    def Viscous_terms(self, g, arrays):
        self._call("Viscous_terms", g, arrays)

    def Filter(self, g, crit, hi, lo, arrays):
        self._call("Filter", g, arrays, C.c_double(crit), C.c_double(hi), C.c_double(lo))

    def RK3NODT(self, g, RK, dt, arrays):
        er = np.zeros(5)
        self._call("RK3NODT", g, arrays, C.c_int(RK), C.c_double(dt),
                   er.ctypes.data_as(C.POINTER(C.c_double)))
        return er

    def Dual_time_stepping(self, g, dt, Nijk, ijk, arrays):
        er = np.zeros(5)
        self._call("Dual_time_stepping", g, arrays, C.c_double(dt),
                   er.ctypes.data_as(C.POINTER(C.c_double)),
                   Nijk.ctypes.data_as(C.POINTER(C.c_int)), ijk.ctypes.data_as(C.POINTER(C.c_int)))
        return er

    def DPLUSGS(self, g, dt, arrays):
        er = np.zeros(5)
        self._call("DPLUSGS", g, arrays, C.c_double(dt), er.ctypes.data_as(C.POINTER(C.c_double)))
        return er

    def Hyperplane(self, g):
        Nijk, ijk = hyperplane_buffers(g)
        gs = grid_struct(g)
        self.lib.cfo_Hyperplane(C.byref(gs), Nijk.ctypes.data_as(C.POINTER(C.c_int)),
                                ijk.ctypes.data_as(C.POINTER(C.c_int)))
        return Nijk, ijk

    def Jacobian_face(self, which, g, gamma, arrays):
        fn = getattr(self.lib, "cfo_Jacobian_" + which)
        gs = grid_struct(g)
        fn(C.byref(gs), C.c_double(gamma), _ptrs(arrays))

    def Driven_force(self, g, U2, J):
        self.lib.cfo_Driven_force.restype = C.c_double
        gs = grid_struct(g)
        return self.lib.cfo_Driven_force(C.byref(gs), _ptrs([U2, J]))

    @staticmethod
    def statistic_state(g):
        """Accumulators of Statistic (17 rows of Y_m, then SXY_bottom, SXY_up)."""
        return np.zeros(17 * (g.Y_out + 4) + 2)

    def Statistic(self, g, acc, step, iteration, statistic_step, arrays):
        """One Statistic call; returns (written, shear[2], nd[10][Y_m], st[7][Y_m])."""
        Ym = g.Y_out + 4
        shear = np.zeros(2)
        nd = np.zeros((10, Ym))
        st = np.zeros((7, Ym))
        gs = grid_struct(g)
        dp = C.POINTER(C.c_double)
        w = self.lib.cfo_Statistic(C.byref(gs), acc.ctypes.data_as(dp), C.c_int(step), C.c_int(iteration),
                                   C.c_int(statistic_step), _ptrs(arrays), shear.ctypes.data_as(dp),
                                   nd.ctypes.data_as(dp), st.ctypes.data_as(dp))
        return bool(w), shear, nd, st

    def restart_pack(self, g, arrays):
        """The LES%05d.bin image of U1..U5, U1q..U5q (times J), as float64."""
        out = np.zeros(10 * g.X_out * g.Y_out * g.Z_out)
        gs = grid_struct(g)
        self.lib.cfo_restart_pack(C.byref(gs), _ptrs(arrays), out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def restart_unpack(self, g, image, arrays):
        """Initial_condition's fill of U1..U5, U1q..U5q (divided by J)."""
        gs = grid_struct(g)
        img = np.ascontiguousarray(image, dtype=np.float64)
        self.lib.cfo_restart_unpack(C.byref(gs), img.ctypes.data_as(C.POINTER(C.c_double)), _ptrs(arrays))


def hyperplane_buffers(g):
    X_np = g.X_out + 6
    ny, nz = g.Y_out + 1, g.Z_out + 1
    nplanes = (X_np - 3) + ny + nz + 7      # Array.h:182
    ncells = (X_np - 6) * g.Y_out * g.Z_out * 3 + 1
    return np.zeros((nplanes, 2), np.int32), np.zeros((ncells, 3), np.int32)


def reference_available() -> bool:
    from . import build_ref
    return (build_ref.reference_dir() / "Flux_X_limiter.cpp").exists()


class Reference:
    """The reference's own routines for one grid (compiled on demand)."""

    def __init__(self, g):
        from . import build_ref
        lib = build_ref.build(g.X_out, g.Y_out, g.Z_out, (g.deltaXI, g.deltaET, g.deltaZT))
        self.lib = C.CDLL(str(lib))
        dims = (C.c_int * 6)()
        d = (C.c_double * 3)()
        self.lib.ref_grid(dims, d)
        assert tuple(dims[:3]) == (g.X_out, g.Y_out, g.Z_out)
        assert tuple(d) == (g.deltaXI, g.deltaET, g.deltaZT)
        self.g = g

    def _call(self, name, arrays, *scalars):
        getattr(self.lib, "ref_" + name)(*scalars, _ptrs(arrays))

    def Y_boundary_condition(self, g, arrays):
        self._call("Y_boundary_condition", arrays)

    def Z_boundary_condition(self, g, arrays):
        self._call("Z_boundary_condition", arrays)

    def Statistic(self, step, iteration, statistic_step, arrays):
        """The reference's Statistic; writes its files in the current directory."""
        self.lib.ref_Statistic(C.c_int(step), C.c_int(iteration), C.c_int(statistic_step), _ptrs(arrays))

    def Output(self, step, arrays):
        """The reference's Output (U1..U5, U1q..U5q, J): LES%05d.bin in the current directory."""
        self.lib.ref_Output(C.c_int(step), _ptrs(arrays))

    def Initial_condition(self, arrays):
        """The reference's Initial_condition (16 arrays): reads initial.bin in the current directory."""
        self.lib.ref_Initial_condition(_ptrs(arrays))

    def flux(self, name, g, arrays):
        self._call(name, arrays)

    def Viscous_terms(self, g, arrays):
        self._call("Viscous_terms", arrays)

    def Filter(self, g, crit, hi, lo, arrays):
        self._call("Filter", arrays, C.c_double(crit), C.c_double(hi), C.c_double(lo))

    def RK3NODT(self, g, RK, dt, arrays):
        er = np.zeros(5)
        self._call("RK3NODT", arrays, C.c_int(RK), C.c_double(dt),
                   er.ctypes.data_as(C.POINTER(C.c_double)))
        return er

    def Dual_time_stepping(self, g, dt, Nijk, ijk, arrays):
        er = np.zeros(5)
        self._call("Dual_time_stepping", arrays, C.c_double(dt),
                   er.ctypes.data_as(C.POINTER(C.c_double)),
                   Nijk.ctypes.data_as(C.POINTER(C.c_int)), ijk.ctypes.data_as(C.POINTER(C.c_int)))
        return er

    def DPLUSGS(self, g, dt, arrays):
        er = np.zeros(5)
        self._call("DPLUSGS", arrays, C.c_double(dt), er.ctypes.data_as(C.POINTER(C.c_double)))
        return er

    def DPLUSGS_defined(self, g, dt, arrays):
        er = np.zeros(5)
        self._call("DPLUSGS_defined", arrays, C.c_double(dt), er.ctypes.data_as(C.POINTER(C.c_double)))
        return er

    def Hyperplane(self, g):
        Nijk, ijk = hyperplane_buffers(g)
        self.lib.ref_Hyperplane(Nijk.ctypes.data_as(C.POINTER(C.c_int)),
                                ijk.ctypes.data_as(C.POINTER(C.c_int)))
        return Nijk, ijk

    def Jacobian_face(self, which, g, gamma, arrays):
        assert gamma == 1.5, "the reference hard-codes gamma = 1.5 (Jacobian_u.cpp:19)"
        self._call("Jacobian_" + which, arrays)

    def Jacobian(self, arrays):
        self._call("Jacobian", arrays)

    def Grid(self, arrays):
        self._call("Grid", arrays)
