"""GB300-native hot path of the compressible channel-flow solver.

``Context`` mirrors the reference solver's per-step routines
(ricklee209/Channel_Flow, main.h): each method has the reference routine's
name and takes the reference's arrays in the reference's order, as CUDA
float64 tensors of shape (X_out+6, Y_out+4, Z_out+4) or raw device
pointers.  The work runs in hand-written sm_103a kernels behind the C-ABI of
``libcfgb300.so``; a missing library is an error, never a CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .synthetic import Grid, channel_grid, reference_grid  # noqa: F401

__all__ = ["Context", "Grid", "channel_grid", "reference_grid", "CFError", "FieldSet", "dplusgs_noalloc"]
CFError = _lib.CFError


def _ptr(x):
    if isinstance(x, int):
        return x
    if x is None:
        return None
    import torch
    if isinstance(x, torch.Tensor):
        if x.dtype != torch.float64 or not x.is_cuda or not x.is_contiguous():
            raise ValueError("fields must be contiguous float64 CUDA tensors")
        return x.data_ptr()
    if isinstance(x, np.ndarray):          # a registered host array
        return x.ctypes.data
    raise TypeError(f"unsupported field argument {type(x)}")


class Context:
    """One device context for one grid (the reference's one MPI rank)."""

    def __init__(self, grid: Grid, precision: str = "fp64", stream=None, gamma: float = 1.5,
                 scheme: str = "reference"):
        self.lib = _lib.load()
        self.grid = grid
        g = _lib.grid_struct(grid)
        h = C.c_void_p()
        rc = self.lib.cf_create(C.byref(g), _lib.PREC[precision], C.byref(h))
        _lib.check(self.lib, None, rc)
        self.h = h.value
        self.precision = precision
        if stream is None:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        self.set_stream(stream)
        if gamma != 1.5:
            self._ok(self.lib.cf_set_stretching(self.h, gamma))
        self.scheme = "reference"
        if scheme != "reference":
            self.set_scheme(scheme)

    def close(self):
        if getattr(self, "h", None):
            self.lib.cf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc):
        _lib.check(self.lib, self.h, rc)

    # -- context ---------------------------------------------------------
    def set_stream(self, stream):
        self._ok(self.lib.cf_set_stream(self.h, stream if isinstance(stream, int) else int(stream)))

    def set_lu_schedule(self, schedule: str):
        """'wavefront' (default), 'pencil' or 'planes': how the hyperplane
        sweeps of Dual_time_stepping are launched; all give the same results."""
        self._ok(self.lib.cf_set_lu_schedule(self.h, {"wavefront": _lib.CF_LU_WAVEFRONT,
                                                      "planes": _lib.CF_LU_PLANES,
                                                      "pencil": _lib.CF_LU_PENCIL}[schedule]))

    def set_scheme(self, scheme: str):
        """'reference' (default: the reference's face-state scaling of the
        limited fluxes, bit for bit) or 'consistent' (Flux_Y_limiter's
        near-wall rows reconstruct the conserved variables, Flux_Z_limiter's
        weights are normalised and its left state upwind)."""
        self._ok(self.lib.cf_set_scheme(self.h, _lib.SCHEME[scheme]))
        self.scheme = scheme

    def set_wait_limit(self, polls: int = 0):
        """Polls of a wavefront dependency wait before it gives up and the
        call returns CF_ERR_TIMEOUT (0: the default); a test hook."""
        self._ok(self.lib.cf_set_wait_limit(self.h, polls))

    def lu_trace(self, enable: bool = True):
        """Record per-tile timer stamps of the wavefront sweeps."""
        self._ok(self.lib.cf_lu_trace(self.h, 1 if enable else 0))

    def lu_trace_read(self) -> np.ndarray:
        """Stamps of the last Dual_time_stepping call, shape (2, tiles, 4):
        forward/backward sweep; claimed, inputs ready, staged, done (ns)."""
        g = self.grid
        tiles = -(-g.X_out // 4) * -(-g.Y_out // 8) * -(-g.Z_out // 8)
        out = np.zeros((2, tiles, 4), np.int64)
        self._ok(self.lib.cf_lu_trace_read(self.h, out.ctypes.data, out.size))
        return out

    def set_output_dir(self, path):
        """Directory of Statistic's, Output's and Initial_condition's files."""
        self._ok(self.lib.cf_set_output_dir(self.h, None if path is None else str(path).encode()))

    def Driven_force(self, U2_, J, myid=0):
        """Bulk-flow integral: returns (Q, ER_Q)."""
        q = np.zeros(2)
        self._ok(self.lib.cf_Driven_force(self.h, myid, _ptr(U2_), _ptr(J), q[0:].ctypes.data,
                                          q[1:].ctypes.data))
        return float(q[0]), float(q[1])

    def Statistic(self, step, iteration, statistic_step, *arrays, myid=0):
        if len(arrays) != 27:
            raise ValueError("Statistic takes 27 arrays")
        self._ok(self.lib.cf_Statistic(self.h, myid, step, iteration, statistic_step,
                                       _lib.ptr_array([_ptr(a) for a in arrays])))

    def statistic_read(self) -> np.ndarray:
        out = np.zeros(17 * (self.grid.Y_out + 4) + 2)
        self._ok(self.lib.cf_statistic_read(self.h, out.ctypes.data))
        return out

    def statistic_reset(self):
        self._ok(self.lib.cf_statistic_reset(self.h))

    def statistic_flush(self):
        """Completes the Statistic the last step left running (host part)."""
        self._ok(self.lib.cf_statistic_flush(self.h))

    def Output(self, step, *arrays, myid=0):
        """U1..U5, U1q..U5q, J -> LES%05d.bin"""
        if len(arrays) != 11:
            raise ValueError("Output takes 11 arrays")
        self._ok(self.lib.cf_Output(self.h, step, myid, *[_ptr(a) for a in arrays]))

    def Initial_condition(self, *arrays, myid=0):
        """U1_..U5_, U1..U5, U1q..U5q, J <- initial.bin"""
        if len(arrays) != 16:
            raise ValueError("Initial_condition takes 16 arrays")
        self._ok(self.lib.cf_Initial_condition(self.h, myid, *[_ptr(a) for a in arrays]))

    def step(self, fields: dict, step: int = 1, deltaT: float = 0.00000005, max_iterations: int = 200,
             tolerance: float = 0.001, limiter: bool = True, filter: bool = True, roe_criterion: float = 0.007,
             e_high: float = 1.0, e_low: float = 0.0, statistic_step: int = 0, static_metrics: bool = False):
        """One physical time step (cf_step).  ``fields`` maps the cf_fields
        member names to device tensors (lists for the multi-array members,
        a list of three lists for face_metric and inF).  Returns
        (iterations, er[5], Q).  ``static_metrics``: the metric arrays stay
        unchanged between calls (the FP32 path then converts them once).
        ``filter``: True (every sub-iteration), False, or "per_step" (the
        sensor at the first sub-iteration only)."""
        f = _lib.cf_fields()
        for name, val in fields.items():
            slot = getattr(f, name)
            if isinstance(val, (list, tuple)):
                for i, v in enumerate(val):
                    if isinstance(v, (list, tuple)):
                        for k, x in enumerate(v):
                            slot[i][k] = _ptr(x)
                    else:
                        slot[i] = _ptr(v)
            else:
                setattr(f, name, _ptr(val))
        filt = 2 if filter == "per_step" else int(bool(filter))
        prm = _lib.cf_step_params(deltaT, max_iterations, tolerance, int(limiter), filt, roe_criterion,
                                  e_high, e_low, statistic_step, int(static_metrics))
        it = C.c_int(0)
        er = np.zeros(5)
        q = np.zeros(1)
        self._ok(self.lib.cf_step(self.h, C.byref(prm), step, C.byref(f), C.byref(it), er.ctypes.data,
                                  q.ctypes.data))
        return it.value, er, float(q[0])

    def step_reset(self):
        self._ok(self.lib.cf_step_reset(self.h))

    def step_scale(self, E=None) -> np.ndarray:
        """The running residual maxima E1..E5; with ``E`` given, set them."""
        e = np.zeros(5) if E is None else np.ascontiguousarray(E, dtype=np.float64).copy()
        self._ok(self.lib.cf_step_scale(self.h, e.ctypes.data, 0 if E is None else 1))
        return e

    def step_residuals(self) -> np.ndarray:
        """[iterations x 5] normalised er1..er5 of the last step's iterations."""
        n = C.c_int(0)
        self._ok(self.lib.cf_step_residuals(self.h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 5))
        if n.value:
            self._ok(self.lib.cf_step_residuals(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def set_precision(self, precision: str):
        self._ok(self.lib.cf_set_precision(self.h, _lib.PREC[precision]))
        self.precision = precision

    def synchronize(self):
        self._ok(self.lib.cf_synchronize(self.h))

    def register(self, host: np.ndarray):
        assert host.dtype == np.float64 and host.flags["C_CONTIGUOUS"] and host.size == self.field_count
        self._ok(self.lib.cf_register(self.h, host.ctypes.data))

    def upload(self, host: np.ndarray):
        self._ok(self.lib.cf_upload(self.h, host.ctypes.data))

    def download(self, host: np.ndarray):
        self._ok(self.lib.cf_download(self.h, host.ctypes.data))

    def upload_async(self, host: np.ndarray, stream):
        """Queue the upload of a registered (pinned) host array on `stream`."""
        self._ok(self.lib.cf_upload_async(self.h, host.ctypes.data, stream if isinstance(stream, int) else int(stream)))

    def download_async(self, host: np.ndarray, stream):
        """Queue the download into a registered (pinned) host array on `stream`."""
        self._ok(self.lib.cf_download_async(self.h, host.ctypes.data,
                                            stream if isinstance(stream, int) else int(stream)))

    @property
    def field_count(self) -> int:
        return int(self.lib.cf_field_count(self.h))

    def check_finite(self, field):
        self._ok(self.lib.cf_check_finite(self.h, _ptr(field)))

    # -- boundary conditions (Y_/Z_boundary_condition.cpp, main.cpp:156-244)
    def Y_boundary_condition(self, U1_, U2_, U3_, U4_, U5_, J, myid=0):
        self._ok(self.lib.cf_Y_boundary_condition(self.h, myid, *map(_ptr, (U1_, U2_, U3_, U4_, U5_, J))))

    def Z_boundary_condition(self, U1_, U2_, U3_, U4_, U5_, J, myid=0):
        self._ok(self.lib.cf_Z_boundary_condition(self.h, myid, *map(_ptr, (U1_, U2_, U3_, U4_, U5_, J))))

    def X_periodic(self, U1_, U2_, U3_, U4_, U5_, myid=0):
        self._ok(self.lib.cf_X_periodic(self.h, myid, *map(_ptr, (U1_, U2_, U3_, U4_, U5_))))

    # -- fluxes: the reference's 32 arrays ---------------------------------
    def _flux(self, name, arrays, myid):
        if len(arrays) != 32:
            raise ValueError(f"{name} takes 32 arrays, got {len(arrays)}")
        self._ok(getattr(self.lib, "cf_" + name)(self.h, myid, *map(_ptr, arrays)))

    def Flux_X_limiter(self, *arrays, myid=0): self._flux("Flux_X_limiter", arrays, myid)
    def Flux_Y_limiter(self, *arrays, myid=0): self._flux("Flux_Y_limiter", arrays, myid)
    def Flux_Z_limiter(self, *arrays, myid=0): self._flux("Flux_Z_limiter", arrays, myid)
    def Flux_X(self, *arrays, myid=0): self._flux("Flux_X", arrays, myid)
    def Flux_Y(self, *arrays, myid=0): self._flux("Flux_Y", arrays, myid)
    def Flux_Z(self, *arrays, myid=0): self._flux("Flux_Z", arrays, myid)

    def flux(self, name, arrays, myid=0):
        self._flux(name, arrays, myid)

    # -- viscous terms and sensor -----------------------------------------
    def Viscous_terms(self, *arrays, myid=0):
        if len(arrays) != 79:
            raise ValueError("Viscous_terms takes 79 arrays")
        self._ok(self.lib.cf_Viscous_terms(self.h, myid, _lib.ptr_array([_ptr(a) for a in arrays])))

    def Filter(self, Roe_criterion, E_high, E_low, U1_, U2_, U3_, U4_, U5_, Y_point, EpX, EpY, EpZ, J, myid=0):
        self._ok(self.lib.cf_Filter(self.h, myid, Roe_criterion, E_high, E_low,
                                    *map(_ptr, (U1_, U2_, U3_, U4_, U5_, Y_point, EpX, EpY, EpZ, J))))

    # -- time integration --------------------------------------------------
    def RK3NODT(self, RK, deltaT, *arrays, myid=0):
        if len(arrays) != 49:
            raise ValueError("RK3NODT takes 49 arrays")
        self._ok(self.lib.cf_RK3NODT(self.h, myid, RK, deltaT, None, None, None, None, None,
                                     _lib.ptr_array([_ptr(a) for a in arrays])))

    def Hyperplane(self):
        g = self.grid
        X_np = g.X_out + 6
        Nijk = np.zeros(((X_np - 3) + g.ny + g.nz + 7, 2), np.int32)
        ijk = np.zeros(((X_np - 6) * g.Y_out * g.Z_out * 3 + 1, 3), np.int32)
        self._ok(self.lib.cf_Hyperplane(self.h, 0, Nijk.ctypes.data, ijk.ctypes.data))
        return Nijk, ijk

    def Dual_time_stepping(self, deltaT, *arrays, Nijk=None, ijk=None, myid=0):
        if len(arrays) != 64:
            raise ValueError("Dual_time_stepping takes 64 arrays")
        er = np.zeros(5)
        e = [er[n:].ctypes.data for n in range(5)]
        self._ok(self.lib.cf_Dual_time_stepping(
            self.h, myid, deltaT, *e, None if Nijk is None else Nijk.ctypes.data,
            None if ijk is None else ijk.ctypes.data, _lib.ptr_array([_ptr(a) for a in arrays])))
        return er

    def DPLUSGS(self, deltaT, *arrays, myid=0):
        if len(arrays) != 64:
            raise ValueError("DPLUSGS takes 64 arrays")
        er = np.zeros(5)
        e = [er[n:].ctypes.data for n in range(5)]
        self._ok(self.lib.cf_DPLUSGS(self.h, myid, deltaT, *e, _lib.ptr_array([_ptr(a) for a in arrays])))
        return er

    # -- face metrics ------------------------------------------------------
    def Jacobian_u(self, *arrays, myid=0):
        self._ok(self.lib.cf_Jacobian_u(self.h, myid, _lib.ptr_array([_ptr(a) for a in arrays])))

    def Jacobian_v(self, *arrays, myid=0):
        self._ok(self.lib.cf_Jacobian_v(self.h, myid, _lib.ptr_array([_ptr(a) for a in arrays])))

    def Jacobian_w(self, *arrays, myid=0):
        self._ok(self.lib.cf_Jacobian_w(self.h, myid, _lib.ptr_array([_ptr(a) for a in arrays])))


def dplusgs_noalloc(grid: Grid, deltaT, *arrays, stream=None):
    """DPLUSGS through the allocation-free entry point (no context, scratch in
    a fixed file-scope device array): for callers that may not allocate
    device memory (a host memory manager owns the device, or the loop cannot
    absorb an allocation's device-wide synchronisation).  The call
    synchronises the stream.  Returns the residual norms er1..er5."""
    lib = _lib.load()
    if len(arrays) != 64:
        raise ValueError("DPLUSGS takes 64 arrays")
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    g = _lib.grid_struct(grid)
    er = np.zeros(5)
    e = [er[n:].ctypes.data for n in range(5)]
    rc = lib.cf_DPLUSGS_noalloc(C.byref(g), stream, deltaT, *e, _lib.ptr_array([_ptr(a) for a in arrays]))
    if rc != _lib.CF_OK:
        raise CFError(rc, "cf_DPLUSGS_noalloc: " + lib.cf_error_string(rc).decode())
    return er


class FieldSet:
    """Device fields of one grid, allocated as one (n, X_np, Y_m, Z_m) float64
    block so that related arrays are adjacent in HBM."""

    def __init__(self, grid: Grid, n: int, device="cuda"):
        import torch
        self.block = torch.zeros((n,) + grid.shape, dtype=torch.float64, device=device)

    def __getitem__(self, i):
        return self.block[i]

    def __len__(self):
        return self.block.shape[0]

    def list(self):
        return [self.block[i] for i in range(self.block.shape[0])]
