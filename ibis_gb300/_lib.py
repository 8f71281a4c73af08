"""ctypes binding of libibisgb.so (the C ABI declared in include/ibisgb.h).

The library is built in-tree by ibis_gb300.build; loading fails loudly when it
is missing: there is no CPU fallback for the residual path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

IBISGB_OK = 0
ERRORS = {
    -1: "IBISGB_ERR_CONFIG", -2: "IBISGB_ERR_GRID", -3: "IBISGB_ERR_CUDA",
    -4: "IBISGB_ERR_BAD_CELLS", -5: "IBISGB_ERR_ARG", -6: "IBISGB_ERR_TIMEOUT",
    -7: "IBISGB_ERR_STATE",
}
PRECISION = {"f64": 0, "mixed": 1, "f64_exact": 2, "mixed_grad": 3, "mixed_ff": 4}


class IbisgbError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


class Sizes(C.Structure):
    _fields_ = [("num_cells", C.c_int64), ("num_ghost_cells", C.c_int64), ("num_faces", C.c_int64),
                ("dim", C.c_int32), ("max_faces_per_cell", C.c_int32), ("n_conserved", C.c_int32),
                ("num_boundaries", C.c_int32)]


class NewtonStatus(C.Structure):
    _fields_ = [("relative_residual", C.c_double), ("residual_norms", C.c_double * 6),
                ("gmres_iterations", C.c_int32), ("gmres_converged", C.c_int32),
                ("gmres_residual", C.c_double), ("dt_star", C.c_double), ("cfl", C.c_double),
                ("step", C.c_int64), ("initial_norms", C.c_double * 6)]


class AdjointStatus(C.Structure):
    _fields_ = [("residual_norm", C.c_double), ("gmres_iterations", C.c_int32), ("gmres_converged", C.c_int32),
                ("gmres_residual", C.c_double), ("dt_star", C.c_double), ("scaled_residual_norm", C.c_double)]


class RkStatus(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("stable_dt", C.c_double),
                ("steps", C.c_int64), ("bad_cells", C.c_int64), ("device_ms", C.c_double)]


_lib = None
_P = C.c_void_p


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libibisgb.so (building it first when allowed and missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise RuntimeError(f"libibisgb.so not built ({_build.LIB}); run ibis_gb300.build.build()")
        _build.build()
    L = C.CDLL(_build.LIB)
    L.ibisgb_create.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(_P)]
    L.ibisgb_create_from_arrays.argtypes = [C.c_char_p, C.c_int32, C.c_int64, _P, C.c_int64, _P, _P, _P,
                                            C.c_int32, C.c_char_p, _P, _P, _P, _P, C.POINTER(_P)]
    L.ibisgb_destroy.argtypes = [_P]
    L.ibisgb_destroy.restype = None
    L.ibisgb_last_error.argtypes = [_P]
    L.ibisgb_last_error.restype = C.c_char_p
    L.ibisgb_get_sizes.argtypes = [_P, C.POINTER(Sizes)]
    L.ibisgb_set_primitives.argtypes = [_P, _P, _P, _P, _P, _P]
    L.ibisgb_get_primitives.argtypes = [_P] + [_P] * 7
    L.ibisgb_get_conserved.argtypes = [_P, _P]
    L.ibisgb_residual.argtypes = [_P, C.c_int32, _P]
    L.ibisgb_residual_device.argtypes = [_P, C.c_int32, _P, _P]
    L.ibisgb_estimate_dt.argtypes = [_P, C.POINTER(C.c_double)]
    L.ibisgb_count_bad_cells.argtypes = [_P, C.POINTER(C.c_int64)]
    L.ibisgb_rk_run.argtypes = [_P, C.c_int32, C.c_int64, C.POINTER(RkStatus)]
    L.ibisgb_l2_norms.argtypes = [_P, _P]
    L.ibisgb_get_dump.argtypes = [_P, C.c_int32, _P, C.c_int64]
    L.ibisgb_set_geometry.argtypes = [_P, _P, _P]
    L.ibisgb_set_flow_state.argtypes = [_P, C.c_char_p, _P]
    L.ibisgb_shared_tables.argtypes = [_P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.ibisgb_get_flow_state.argtypes = [_P, C.c_char_p, _P]
    L.ibisgb_vjp_flow_state.argtypes = [_P, _P, _P, C.c_int32]
    L.ibisgb_vjp_flow_state_device.argtypes = [_P, _P, _P, C.c_int32, _P]
    L.ibisgb_jvp_flow_state.argtypes = [_P, _P, _P, C.c_int32]
    L.ibisgb_set_scratch_poison.argtypes = [_P, C.c_int32]
    L.ibisgb_jvp_flow_state_device.argtypes = [_P, _P, _P, C.c_int32, _P]
    L.ibisgb_numbering.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.ibisgb_synchronize.argtypes = [_P]
    L.ibisgb_set_conserved.argtypes = [_P, _P]
    L.ibisgb_set_conserved_device.argtypes = [_P, _P, _P]
    L.ibisgb_get_stream.argtypes = [_P, C.POINTER(_P)]
    L.ibisgb_kernel_times.argtypes = [_P, C.c_int32, C.c_int32, _P]
    L.ibisgb_l2_norms_noalloc.argtypes = [_P, C.c_int64, C.c_int32, _P, _P]
    L.ibisgb_jvp.argtypes = [_P, _P, _P, C.c_double, C.c_int32]
    L.ibisgb_jvp_device.argtypes = [_P, _P, _P, C.c_double, C.c_int32, _P]
    L.ibisgb_vjp.argtypes = [_P, _P, _P, _P, C.c_int32]
    L.ibisgb_vjp_device.argtypes = [_P, _P, _P, _P, C.c_int32, _P]
    L.ibisgb_vjp_geometry.argtypes = [_P, _P, _P, _P, C.c_int32]
    L.ibisgb_set_adjoint_krylov.argtypes = [_P, C.c_int32]
    L.ibisgb_jvp_geometry.argtypes = [_P, _P, _P, _P, C.c_int32]
    L.ibisgb_jvp_geometry_device.argtypes = [_P, _P, _P, _P, C.c_int32, _P]
    L.ibisgb_rk_run_host.argtypes = [_P, C.c_int32, C.c_int64, C.c_int64, _P, _P, _P]
    L.ibisgb_vjp_geometry_device.argtypes = [_P, _P, _P, _P, C.c_int32, _P]
    L.ibisgb_adjoint_step.argtypes = [_P, _P, _P, C.c_double, C.POINTER(AdjointStatus)]
    L.ibisgb_steady_initialise.argtypes = [_P, C.c_int32]
    L.ibisgb_newton_step.argtypes = [_P, C.c_int32, C.POINTER(NewtonStatus)]
    L.ibisgb_steady_norms.argtypes = [_P, _P, _P]
    L.ibisgb_autotune.argtypes = [_P, C.c_int32, _P, _P]
    L.ibisgb_set_launch_variants.argtypes = [_P, C.c_int32, _P]
    L.ibisgb_launch_variants.argtypes = [C.POINTER(C.c_int32), _P, _P]
    L.ibisgb_set_fused.argtypes = [_P, C.c_int32]
    L.ibisgb_check_conversions.argtypes = [C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]
    L.ibisgb_fused_info.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P, C.c_char_p, C.c_int32]
    L.ibisgb_set_fused_kind.argtypes = [_P, C.c_int32, C.c_int32]
    L.ibisgb_fused_kind.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P,
                                    C.c_char_p, C.c_int32]
    L.ibisgb_set_cell_flux.argtypes = [_P, C.c_int32]
    L.ibisgb_cell_flux_info.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), _P]
    L.ibisgb_batch_create.argtypes = [_P, C.c_int32, C.POINTER(_P)]
    L.ibisgb_batch_layout.argtypes = [_P, C.POINTER(C.c_int32), _P, _P, _P]
    L.ibisgb_batch_status.argtypes = [_P, _P]
    _lib = L
    return L


def check(rc: int, ctx=None) -> None:
    if rc != IBISGB_OK:
        msg = load().ibisgb_last_error(ctx).decode()
        raise IbisgbError(rc, msg)


def header_symbols() -> list:
    """Function names declared in include/ibisgb.h."""
    import re
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ibisgb.h")
    text = open(path).read()
    return sorted(set(re.findall(r"\b(ibisgb_[a-z0-9_]+)\s*\(", text)))
