"""ctypes binding of libcfgb300.so (the C-ABI in include/channel_flow_gb300.h).

The library is built in-tree by ``channel_flow_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libcfgb300.so"

CF_OK, CF_ERR_ARG, CF_ERR_CUDA, CF_ERR_NONFINITE, CF_ERR_NOMEM, CF_ERR_STATE, CF_ERR_TIMEOUT = range(7)
CF_LU_WAVEFRONT, CF_LU_PLANES, CF_LU_PENCIL = 0, 1, 2
PREC = {"fp64_exact": 0, "fp64": 1, "fp32": 2}
SCHEME = {"reference": 0, "consistent": 1}


class cf_grid(C.Structure):
    _fields_ = [("cells_x", C.c_int), ("cells_y", C.c_int), ("cells_z", C.c_int),
                ("d_xi", C.c_double), ("d_eta", C.c_double), ("d_zeta", C.c_double),
                ("gamma_gas", C.c_double), ("r_gas", C.c_double), ("beta_min", C.c_double),
                ("cv", C.c_double), ("mu", C.c_double), ("prandtl", C.c_double),
                ("body_force", C.c_double), ("height", C.c_double), ("bulk_flux", C.c_double)]


_VP = C.c_void_p


class cf_fields(C.Structure):
    _fields_ = [("U_", _VP * 5), ("U", _VP * 5), ("Uq", _VP * 5), ("J", _VP), ("Y_point", _VP),
                ("cell_metric", _VP * 9), ("face_J", _VP * 3), ("face_metric", (_VP * 9) * 3), ("Ep", _VP * 3),
                ("inF", (_VP * 5) * 3), ("vF", _VP * 4), ("LL", _VP * 4), ("ML", _VP * 4),
                ("MR", _VP * 5), ("NR", _VP * 5), ("NL", _VP * 5), ("Residual", _VP * 5)]


class cf_step_params(C.Structure):
    _fields_ = [("deltaT", C.c_double), ("max_iterations", C.c_int), ("tolerance", C.c_double),
                ("limiter", C.c_int), ("filter", C.c_int), ("roe_criterion", C.c_double),
                ("e_high", C.c_double), ("e_low", C.c_double), ("statistic_step", C.c_int),
                ("static_metrics", C.c_int)]


class cf_wavy_wall(C.Structure):
    _fields_ = [("amplitude", C.c_double), ("wavelength", C.c_double), ("stretching", C.c_double),
                ("conservative", C.c_int)]


def grid_struct(grid) -> "cf_grid":
    return cf_grid(grid.X_out, grid.Y_out, grid.Z_out, grid.deltaXI, grid.deltaET, grid.deltaZT,
                   grid.K, grid.R, grid.e, grid.Cv, grid.mu_L, grid.Pr_L, grid.f, grid.high, grid.Q0)


class CFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()

P = C.c_void_p
_SIGS = {
    "cf_library_version": ([], C.c_int),
    "cf_error_string": ([C.c_int], C.c_char_p),
    "cf_last_error": ([P], C.c_char_p),
    "cf_grid_reference": ([C.POINTER(cf_grid), C.c_int, C.c_int, C.c_int], C.c_int),
    "cf_create": ([C.POINTER(cf_grid), C.c_int, C.POINTER(P)], C.c_int),
    "cf_destroy": ([P], None),
    "cf_set_precision": ([P, C.c_int], C.c_int),
    "cf_set_stream": ([P, P], C.c_int),
    "cf_set_stretching": ([P, C.c_double], C.c_int),
    "cf_set_lu_schedule": ([P, C.c_int], C.c_int),
    "cf_set_scheme": ([P, C.c_int], C.c_int),
    "cf_fp64_peak_probe": ([P, C.c_int, C.c_int, P], C.c_int),
    "cf_reciprocal_check": ([P, P, P, C.c_size_t], C.c_int),
    "cf_set_wait_limit": ([P, C.c_uint], C.c_int),
    "cf_lu_trace": ([P, C.c_int], C.c_int),
    "cf_lu_trace_read": ([P, P, C.c_size_t], C.c_int),
    "cf_synchronize": ([P], C.c_int),
    "cf_field_count": ([P], C.c_size_t),
    "cf_register": ([P, P], C.c_int),
    "cf_unregister": ([P, P], C.c_int),
    "cf_upload": ([P, P], C.c_int),
    "cf_download": ([P, P], C.c_int),
    "cf_device_ptr": ([P, P], P),
    "cf_upload_async": ([P, P, P], C.c_int),
    "cf_download_async": ([P, P, P], C.c_int),
    "cf_check_finite": ([P, P], C.c_int),
    "cf_Y_boundary_condition": ([P, C.c_int] + [P] * 6, C.c_int),
    "cf_Z_boundary_condition": ([P, C.c_int] + [P] * 6, C.c_int),
    "cf_X_periodic": ([P, C.c_int] + [P] * 5, C.c_int),
    "cf_Viscous_terms": ([P, C.c_int, C.POINTER(P)], C.c_int),
    "cf_Filter": ([P, C.c_int, C.c_double, C.c_double, C.c_double] + [P] * 10, C.c_int),
    "cf_RK3NODT": ([P, C.c_int, C.c_int, C.c_double] + [P] * 5 + [C.POINTER(P)], C.c_int),
    "cf_Hyperplane": ([P, C.c_int, P, P], C.c_int),
    "cf_Dual_time_stepping": ([P, C.c_int, C.c_double] + [P] * 5 + [P, P, C.POINTER(P)], C.c_int),
    "cf_DPLUSGS": ([P, C.c_int, C.c_double] + [P] * 5 + [C.POINTER(P)], C.c_int),
    "cf_DPLUSGS_noalloc": ([C.POINTER(cf_grid), P, C.c_double] + [P] * 5 + [C.POINTER(P)], C.c_int),
    "cf_Jacobian_u": ([P, C.c_int, C.POINTER(P)], C.c_int),
    "cf_Jacobian_v": ([P, C.c_int, C.POINTER(P)], C.c_int),
    "cf_Jacobian_w": ([P, C.c_int, C.POINTER(P)], C.c_int),
    "cf_wavy_metrics": ([P, P, P, C.c_int, C.POINTER(P)], C.c_int),
    "cf_wavy_y_point": ([P, P, P, P], C.c_int),
    "cf_set_output_dir": ([P, C.c_char_p], C.c_int),
    "cf_Driven_force": ([P, C.c_int, P, P, P, P], C.c_int),
    "cf_Statistic": ([P, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(P)], C.c_int),
    "cf_statistic_read": ([P, P], C.c_int),
    "cf_statistic_reset": ([P], C.c_int),
    "cf_statistic_flush": ([P], C.c_int),
    "cf_Output": ([P, C.c_int, C.c_int] + [P] * 11, C.c_int),
    "cf_Initial_condition": ([P, C.c_int] + [P] * 16, C.c_int),
    "cf_step": ([P, P, C.c_int, P, P, P, P], C.c_int),
    "cf_step_reset": ([P], C.c_int),
    "cf_step_scale": ([P, P, C.c_int], C.c_int),
    "cf_step_residuals": ([P, P, C.c_int, P], C.c_int),
    "cf_gemm_bf16": ([P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, C.c_int, P], C.c_int),
    "cf_gemm_bf16_splitk": ([P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P], C.c_int),
    "cf_mlp_features": ([P, C.c_int, C.c_int, C.c_int, P, P, P, C.c_longlong, C.c_longlong, P], C.c_int),
    "cf_mlp_targets": ([P, C.c_int, C.c_int, C.c_int, P, P, P, P, P, C.c_longlong, C.c_longlong, P], C.c_int),
    "cf_mlp_apply": ([P, C.c_int, C.c_int, C.c_int, P, P, P, P, P, P], C.c_int),
    "cf_mlp_features_grid": ([P, C.c_int, C.c_int, C.c_int, P, P, C.c_longlong, P, P], C.c_int),
    "cf_mlp_base_sums": ([P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, P], C.c_int),
    "cf_mlp_scale": ([P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, P], C.c_int),
    "cf_mlp_dot": ([P, P, P, C.c_longlong, P, C.c_int, P], C.c_int),
    "cf_mlp_rms": ([P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, P], C.c_int),
    "cf_mlp_rms3": ([P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, P], C.c_int),
    "cf_mlp_loss_grad": ([P, P, P, C.c_longlong, C.c_longlong, P, P, P], C.c_int),
    "cf_mlp_silu_bwd": ([P, P, P, C.c_longlong, P, P], C.c_int),
    "cf_transpose_bf16": ([P, P, C.c_longlong, C.c_int, P], C.c_int),
    "cf_colsum_bf16": ([P, P, C.c_longlong, C.c_int, P], C.c_int),
    "cf_adam": ([P, P, P, P, P, C.c_longlong, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int], C.c_int),
    "cf_mlp_pack": ([P, P, P, P, P, P, P, P, P], C.c_int),
}
for _n in ("Flux_X_limiter", "Flux_Y_limiter", "Flux_Z_limiter", "Flux_X", "Flux_Y", "Flux_Z"):
    _SIGS["cf_" + _n] = ([P, C.c_int] + [P] * 32, C.c_int)

EXPORTED = sorted(_SIGS)


def load():
    """Load (not build) the library; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -m channel_flow_gb300.build` "
                    "(the channel-flow kernels have no CPU fallback)")
            lib = C.CDLL(str(LIB_PATH))
            for name, (args, res) in _SIGS.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = res
            _lib = lib
    return _lib


def check(lib, ctx, rc):
    if rc != CF_OK:
        msg = lib.cf_last_error(ctx).decode() if ctx else lib.cf_error_string(rc).decode()
        raise CFError(rc, msg or lib.cf_error_string(rc).decode())


def ptr_array(ptrs):
    return (P * len(ptrs))(*ptrs)
