"""Channels with a wavy lower wall: metrics and Y_point on the device.

The reference builds analytic flat-wall metrics only (Grid.cpp:49-141,
Jacobian.cpp, Jacobian_u/v/w.cpp).  ``cf_wavy_metrics`` generalises them
to the lower wall y_w(x) = A sin(2 pi x / lambda) with the upper wall flat
and the same tanh wall-normal stretching; ``channel_metrics`` fills every
metric array a step needs (cells and the three face sets, each J plus the
nine metrics xidx..ztdz, and Y_point) in the reference layout.  The default
is the conservative form, whose face metrics are differences between cell
corners, so the finite-volume divergence of a uniform flux vanishes to
rounding on the curved grid.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

from . import _lib

WHERE = {"cell": 0, "u": 1, "v": 2, "w": 3}


@dataclass(frozen=True)
class WavyWall:
    amplitude: float
    wavelength: float
    stretching: float = 2.0
    conservative: bool = True

    def struct(self):
        return _lib.cf_wavy_wall(self.amplitude, self.wavelength, self.stretching, int(self.conservative))


def wall_for(grid, amplitude_over_h: float = 0.05, wavelength_over_h: float = math.pi, stretching: float = 2.0,
             conservative: bool = True) -> WavyWall:
    """The wall of a channel of half-height h = high / 2: amplitude and
    wavelength in units of h (defaults 0.05 h and pi h)."""
    h = 0.5 * grid.high
    return WavyWall(amplitude_over_h * h, wavelength_over_h * h, stretching, conservative)


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


def metrics_into(grid, wall: WavyWall, where: str, out10) -> None:
    """Write J and the nine metrics at ``where`` ('cell', 'u', 'v', 'w')
    into ten float64 CUDA tensors of the grid's shape."""
    import torch
    lib = _lib.load()
    if len(out10) != 10:
        raise ValueError("ten arrays: J then xidx..ztdz")
    for t in out10:
        if t.dtype != torch.float64 or not t.is_cuda or tuple(t.shape) != grid.shape or not t.is_contiguous():
            raise ValueError("metric arrays must be contiguous float64 CUDA tensors of the grid's shape")
    g = _lib.grid_struct(grid)
    w = wall.struct()
    arr = _lib.ptr_array([t.data_ptr() for t in out10])
    rc = lib.cf_wavy_metrics(C.byref(g), _stream(torch), C.byref(w), WHERE[where], arr)
    _lib.check(lib, None, rc)


def metrics(grid, wall: WavyWall, where: str):
    """[J, xidx, ..., ztdz] at ``where`` as new float64 CUDA tensors."""
    import torch
    out = [torch.empty(grid.shape, dtype=torch.float64, device="cuda") for _ in range(10)]
    metrics_into(grid, wall, where, out)
    return out


def y_point(grid, wall: WavyWall):
    import torch
    lib = _lib.load()
    out = torch.empty(grid.shape, dtype=torch.float64, device="cuda")
    g = _lib.grid_struct(grid)
    w = wall.struct()
    _lib.check(lib, None, lib.cf_wavy_y_point(C.byref(g), _stream(torch), C.byref(w), C.c_void_p(out.data_ptr())))
    return out


def channel_metrics(grid, wall: WavyWall) -> dict:
    """Every metric array of a step: {'J', 'cm' (9), 'fu', 'fv', 'fw'
    (10 each: J then 9), 'Yp'} on the device."""
    cell = metrics(grid, wall, "cell")
    return {"J": cell[0], "cm": cell[1:], "fu": metrics(grid, wall, "u"), "fv": metrics(grid, wall, "v"),
            "fw": metrics(grid, wall, "w"), "Yp": y_point(grid, wall)}
