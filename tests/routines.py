"""Table of the hot-path routines for the parity tests: how to build a case,
which arrays the routine writes, and how to call it on the compiled
reference, on the C oracle and on the GPU context."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import numpy as np

import cases


@dataclass
class Routine:
    name: str
    build: Callable          # (grid, seed) -> list of arrays
    outputs: list            # written slots
    scalars: bool = False    # returns the five residual norms
    libm: bool = False       # uses tanh/cosh: compare with a tolerance across libms

    def mask(self, g, slot):
        if self.name == "Flux_Y_limiter":
            return cases.ylim_undefined_mask(g, slot)
        return None


def _flux(d):
    return lambda g, s: cases.flux_case(g, d, seed=s)


ROUTINES = [
    Routine("Y_boundary_condition", lambda g, s: cases.bc_case(g, s), cases.BC_OUT),
    Routine("Z_boundary_condition", lambda g, s: cases.bc_case(g, s), cases.BC_OUT),
    Routine("Flux_X_limiter", _flux("x"), cases.FLUX_OUT),
    Routine("Flux_Y_limiter", _flux("y"), cases.FLUX_OUT),
    Routine("Flux_Z_limiter", _flux("z"), cases.FLUX_OUT),
    Routine("Flux_X", _flux("x"), cases.FLUX_OUT),
    Routine("Flux_Y", _flux("y"), cases.FLUX_OUT),
    Routine("Flux_Z", _flux("z"), cases.FLUX_OUT),
    Routine("Viscous_terms", lambda g, s: cases.viscous_case(g, s), cases.VISC_OUT),
    Routine("Filter", lambda g, s: cases.filter_case(g, s), cases.FILTER_OUT),
    Routine("RK3NODT", lambda g, s: cases.dt_case(g, s, nslots=49), cases.RK3_OUT),
    Routine("Dual_time_stepping", lambda g, s: cases.dt_case(g, s), cases.LU_OUT, scalars=True),
    Routine("DPLUSGS", lambda g, s: cases.dt_case(g, s), cases.LU_OUT, scalars=True),
    Routine("Jacobian_u", lambda g, s: cases.jacobian_case(g, "u", s), cases.JAC_OUT, libm=True),
    Routine("Jacobian_v", lambda g, s: cases.jacobian_case(g, "v", s), cases.JAC_OUT, libm=True),
    Routine("Jacobian_w", lambda g, s: cases.jacobian_case(g, "w", s), cases.JAC_OUT, libm=True),
]
BY_NAME = {r.name: r for r in ROUTINES}
RK_STAGE = 2


def run_cpu(impl, r: Routine, g, arrays, scheme="reference"):
    """Run routine r on the compiled reference or the C oracle (in place);
    returns the residual norms for the dual-time routines, else None.
    ``scheme``: the oracle's face-state scaling of the limited fluxes (the
    reference itself has only its own)."""
    n = r.name
    if n in ("Y_boundary_condition", "Z_boundary_condition", "Viscous_terms"):
        getattr(impl, n)(g, arrays)
    elif n.startswith("Flux"):
        if scheme == "reference":
            impl.flux(n, g, arrays)
        else:
            impl.flux(n, g, arrays, scheme=scheme)
    elif n == "Filter":
        impl.Filter(g, *cases.FILTER_ARGS, arrays)
    elif n == "RK3NODT":
        impl.RK3NODT(g, RK_STAGE, cases.DELTA_T, arrays)
    elif n == "Dual_time_stepping":
        Nijk, ijk = impl.Hyperplane(g)
        return impl.Dual_time_stepping(g, cases.DELTA_T, Nijk, ijk, arrays)
    elif n == "DPLUSGS":
        # the reference's own DPLUSGS reads two uninitialised indices; its
        # defined-index build is the one to compare with (see oracle/)
        fn = getattr(impl, "DPLUSGS_defined", impl.DPLUSGS)
        return fn(g, cases.DELTA_T, arrays)
    elif n.startswith("Jacobian_"):
        impl.Jacobian_face(n[-1], g, 1.5, arrays)
    else:
        raise KeyError(n)
    return None


def run_gpu(ctx, r: Routine, arrays):
    """Same on the GPU context: arrays (numpy) are copied to the device,
    the routine runs through the C-ABI, and the written arrays come back."""
    import torch
    dev = [torch.from_numpy(a).cuda() for a in arrays]
    n = r.name
    er = None
    if n in ("Y_boundary_condition", "Z_boundary_condition"):
        getattr(ctx, n)(*dev)
    elif n.startswith("Flux"):
        ctx.flux(n, dev)
    elif n == "Viscous_terms":
        ctx.Viscous_terms(*dev)
    elif n == "Filter":
        ctx.Filter(*cases.FILTER_ARGS, *dev)
    elif n == "RK3NODT":
        ctx.RK3NODT(RK_STAGE, cases.DELTA_T, *dev)
    elif n == "Dual_time_stepping":
        Nijk, ijk = ctx.Hyperplane()
        er = ctx.Dual_time_stepping(cases.DELTA_T, *dev, Nijk=Nijk, ijk=ijk)
    elif n == "DPLUSGS":
        er = ctx.DPLUSGS(cases.DELTA_T, *dev)
    elif n.startswith("Jacobian_"):
        getattr(ctx, n)(*dev)
    else:
        raise KeyError(n)
    torch.cuda.synchronize()
    for i in r.outputs:
        arrays[i][...] = dev[i].cpu().numpy()
    return er


def compare(r: Routine, g, got, want, rtol=0.0, masked=False):
    """Largest normwise relative difference per written array (0 = equal
    bit for bit where rtol == 0).  ``masked``: skip the entries that depend
    on the reference's undefined values (only for comparisons with the
    reference itself; the GPU and the oracle define them alike and are
    compared everywhere)."""
    worst = {}
    for i in r.outputs:
        a, b = got[i], want[i]
        m = r.mask(g, i) if masked else None
        if m is not None:
            a = np.where(m, 0.0, a)
            b = np.where(m, 0.0, b)
        both_nan = np.isnan(a) & np.isnan(b)
        a = np.where(both_nan, 0.0, a)
        b = np.where(both_nan, 0.0, b)
        if rtol == 0.0:
            worst[i] = float(np.count_nonzero(a != b))
        else:
            scale = max(float(np.max(np.abs(b))), 1e-300)
            worst[i] = float(np.max(np.abs(a - b))) / scale
    return worst
