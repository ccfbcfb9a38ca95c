"""ctypes binding of libcycasgpu.so (declarations in include/cycasgpu.h).

The shared library is the product; this module only marshals numpy arrays across the C
ABI.  Loading fails loudly when the library is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

CYCAS_OK = 0
CYCAS_NOT_CONVERGED = 1
CYCAS_NAN_DETECTED = 2
CYCAS_ERR_INVALID = 3
CYCAS_ERR_CUDA = 4
CYCAS_ERR_ALLOC = 5
CYCAS_ERR_IO = 6
CYCAS_ERR_TIMEOUT = 7
CYCAS_ERR_MESH = 8
CYCAS_ERR_UNSUPPORTED = 9

PC_NONE, PC_JACOBI, PC_ILU0, PC_AMG, PC_POLY1, PC_POLY2, PC_POLY3, PC_POLY4, PC_POLY5 = 0, 1, 2, 3, 4, 5, 6, 7, 8
LOAD_MSH_BINARY = 1
DUMP_TECPLOT, DUMP_DATA, DUMP_BACKUP = 1, 2, 4
KSP_DEFAULT, KSP_GMRES, KSP_CG = 0, 1, 2
SYS_VELOCITY, SYS_PRESSURE, SYS_SCALAR = 0, 1, 2

_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_F64P = C.POINTER(C.c_double)


class MeshView(C.Structure):
    _fields_ = [("ncel", C.c_int32), ("nfac", C.c_int32), ("nbnd", C.c_int32), ("nvrt", C.c_int32)] + [
        (name, _P) for name in (
            "face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_face", "cell_cell",
            "cell_vertices", "bnd_face", "bnd_type", "vert", "face_x", "face_n", "face_area", "face_lambda",
            "face_rlencos", "face_xpac", "face_xnac", "cell_vol", "cell_x", "bnd_distance")]


class Params(C.Structure):
    _fields_ = [("turb_model", C.c_int32), ("density_model", C.c_int32), ("cell_pressure_ref", C.c_int32),
                ("urf", C.c_double * 8), ("gravity", C.c_double * 3), ("transient", C.c_int32),
                ("time_scheme", C.c_int32), ("dt", C.c_double), ("max_outer", C.c_int32),
                ("solve_energy", C.c_int32), ("pressure_reference", C.c_double)]


class KspOptions(C.Structure):
    _fields_ = [("type", C.c_int32), ("restart", C.c_int32), ("pc", C.c_int32), ("rtol", C.c_double),
                ("maxit", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("ksp", KspOptions * 3), ("device", C.c_int32), ("mixed", C.c_int32), ("inner_rtol", C.c_double),
                ("amg_omega", C.c_float), ("amg_alpha", C.c_float), ("amg_gamma", C.c_int32), ("reserved", C.c_int32)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("iterations", C.c_int32), ("ncel", C.c_int32),
                ("pad", C.c_int32), ("t_arrival", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("resmax", C.c_double)]


REQ_CONVERGED, REQ_FAILED, REQ_MAX_ITERS = 1, 2, 3


class IterStats(C.Structure):
    _fields_ = [("its", C.c_int32 * 8), ("reason", C.c_int32 * 8), ("rnorm", C.c_double * 8),
                ("nsolves", C.c_int32), ("failed_solve", C.c_int32)]


class Profile(C.Structure):
    _fields_ = [("kernel_launches", C.c_int64), ("krylov_launches", C.c_int64 * 3), ("krylov_iters", C.c_int64 * 3),
                ("krylov_ms", C.c_double * 3), ("assembly_ms", C.c_double)]


class SolveStats(C.Structure):
    _fields_ = [("its", C.c_int32), ("reason", C.c_int32), ("rnorm", C.c_double)]


# every exported symbol declared in include/cycasgpu.h
EXPORTS = (
    "cycas_last_error", "cycas_options_default", "cycas_case_load", "cycas_case_load_ex", "cycas_case_free",
    "cycas_case_dims", "cycas_case_params", "cycas_case_get_int", "cycas_case_output", "cycas_case_get_field",
    "cycas_write_grid", "cycas_write_tecplot", "cycas_write_data", "cycas_write_backup", "cycas_read_backup",
    "cycas_dump_begin", "cycas_dump_wait",
    "cycas_create", "cycas_create_from_case", "cycas_destroy",
    "cycas_get_field", "cycas_set_field", "cycas_get_int", "cycas_simple_iteration", "cycas_simple_iteration_io", "cycas_simple_iterations",
    "cycas_solve_steady", "cycas_restart_point", "cycas_time_step", "cycas_case_physics", "cycas_set_fields", "cycas_get_fields", "cycas_solve_velocity", "cycas_solve_pressure", "cycas_solve_scalar",
    "cycas_run_stage", "cycas_csr_solve", "cycas_get_stream", "cycas_set_profiling", "cycas_get_profile",
    "cycas_reset_profile", "cycas_csr_solve_noalloc", "cycas_get_amg_levels", "cycas_batch_create",
    "cycas_batch_size", "cycas_batch_offsets", "cycas_batch_iteration", "cycas_batch_residuals",
    "cycas_batch_copy_case", "cycas_batch_case_field", "cycas_server_create", "cycas_server_destroy", "cycas_server_set_graph", "cycas_server_set_max_cells",
    "cycas_server_set_async_rebuild",
    "cycas_server_clock", "cycas_server_submit", "cycas_server_step", "cycas_server_poll",
    "cycas_server_result_field", "cycas_server_last_error", "cycas_server_stats", "cycas_footprint_estimate",
    "cycas_set_graph", "cycas_batch_autotune",
)

_lib = None


class CycasError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cycas error {code}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libcycasgpu.so (building it first when missing and allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"libcycasgpu.so not built at {path}")
        _build.build()
    L = C.CDLL(path)
    L.cycas_last_error.restype = C.c_char_p
    L.cycas_options_default.argtypes = [C.POINTER(Options)]
    L.cycas_options_default.restype = None
    L.cycas_case_load.argtypes = [C.c_char_p, C.POINTER(_P)]
    L.cycas_case_load_ex.argtypes = [C.c_char_p, C.c_int32, C.POINTER(_P)]
    L.cycas_case_free.argtypes = [_P]
    L.cycas_case_free.restype = None
    L.cycas_case_dims.argtypes = [_P, C.POINTER(C.c_int64)]
    L.cycas_case_params.argtypes = [_P, _F64P, _F64P, _F64P]
    L.cycas_case_get_int.argtypes = [_P, C.c_char_p, _P, C.c_int64]
    L.cycas_case_output.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.cycas_case_get_field.argtypes = [_P, C.c_char_p, _P, C.c_int64]
    L.cycas_write_grid.argtypes = [_P, C.c_char_p, C.c_int32]
    L.cycas_write_tecplot.argtypes = [_P, C.c_int32, _P, C.c_char_p]
    L.cycas_write_data.argtypes = [_P, C.c_int32, C.c_char_p]
    L.cycas_write_backup.argtypes = [_P, C.c_int32, C.c_char_p]
    L.cycas_read_backup.argtypes = [_P, C.c_int32, C.c_char_p]
    L.cycas_dump_begin.argtypes = [_P, C.c_int32, _P, C.c_int32, C.c_char_p, C.c_char_p, C.c_char_p]
    L.cycas_dump_wait.argtypes = [_P]
    L.cycas_create.argtypes = [C.POINTER(MeshView), C.POINTER(Params), C.POINTER(Options), C.POINTER(_P)]
    L.cycas_create_from_case.argtypes = [_P, C.POINTER(Options), C.POINTER(_P)]
    L.cycas_destroy.argtypes = [_P]
    L.cycas_destroy.restype = None
    L.cycas_get_field.argtypes = [_P, C.c_char_p, _P, C.c_int64]
    L.cycas_set_field.argtypes = [_P, C.c_char_p, _P, C.c_int64]
    L.cycas_get_int.argtypes = [_P, C.c_char_p, _P, C.c_int64]
    L.cycas_set_fields.argtypes = [_P, C.c_int32, _P, _P, _P]
    L.cycas_get_fields.argtypes = [_P, C.c_int32, _P, _P, _P]
    L.cycas_simple_iteration.argtypes = [_P, _F64P, _F64P, C.POINTER(IterStats)]
    L.cycas_simple_iteration_io.argtypes = [_P, C.c_int32, _P, _P, _P, C.c_int32, _P, _P, _P, _F64P, _F64P,
                                            C.POINTER(IterStats)]
    L.cycas_simple_iterations.argtypes = [_P, C.c_int32, _P, _P, _P, _P]
    L.cycas_solve_steady.argtypes = [_P, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_int32), _P, _P, _P, _P]
    L.cycas_restart_point.argtypes = [_P, C.c_int32]
    L.cycas_run_stage.argtypes = [_P, C.c_char_p]
    L.cycas_solve_velocity.argtypes = [_P, C.c_double, C.c_int32, _P, _P, _P, C.POINTER(IterStats)]
    L.cycas_solve_pressure.argtypes = [_P, C.c_double, C.c_int32, _P, C.c_int32, C.POINTER(IterStats)]
    L.cycas_solve_scalar.argtypes = [_P, C.c_double, C.c_int32, _P, C.POINTER(IterStats)]
    L.cycas_time_step.argtypes = [_P, C.c_int32, C.POINTER(C.c_int32), _P, _P, _P, _P, C.POINTER(C.c_double)]
    L.cycas_case_physics.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    L.cycas_csr_solve.argtypes = [C.c_int32, _P, _P, _P, _P, _P, C.POINTER(KspOptions), C.c_double, C.c_int32,
                                  C.c_int32, C.POINTER(SolveStats)]
    L.cycas_get_stream.argtypes = [_P, C.POINTER(_P)]
    L.cycas_set_profiling.argtypes = [_P, C.c_int32]
    L.cycas_get_profile.argtypes = [_P, C.POINTER(Profile)]
    L.cycas_reset_profile.argtypes = [_P]
    L.cycas_get_amg_levels.argtypes = [_P, C.c_int32, C.POINTER(C.c_int32), _P, _P]
    L.cycas_batch_create.argtypes = [_P, C.c_int32, C.POINTER(Options), C.POINTER(_P)]
    L.cycas_batch_size.argtypes = [_P, C.POINTER(C.c_int32)]
    L.cycas_batch_offsets.argtypes = [_P, C.c_int32, _P]
    L.cycas_batch_iteration.argtypes = [_P, _P, _P, _P]
    L.cycas_batch_residuals.argtypes = [_P, _P]
    L.cycas_batch_copy_case.argtypes = [_P, C.c_int32, _P, C.c_int32]
    L.cycas_batch_case_field.argtypes = [_P, C.c_int32, C.c_char_p, _P, C.c_int64]
    L.cycas_server_create.argtypes = [C.POINTER(Options), C.c_double, C.c_double, C.c_int32, C.c_int32, C.POINTER(_P)]
    L.cycas_server_set_graph.argtypes = [_P, C.c_int32]
    L.cycas_server_set_max_cells.argtypes = [_P, C.c_double]
    L.cycas_server_set_async_rebuild.argtypes = [_P, C.c_int32]
    L.cycas_server_destroy.argtypes = [_P]
    L.cycas_server_destroy.restype = None
    L.cycas_server_clock.argtypes = []
    L.cycas_server_clock.restype = C.c_double
    L.cycas_server_submit.argtypes = [_P, C.c_char_p, C.POINTER(C.c_int64)]
    L.cycas_server_step.argtypes = [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.cycas_server_poll.argtypes = [_P, C.POINTER(RequestResult), C.c_int32, C.POINTER(C.c_int32)]
    L.cycas_server_result_field.argtypes = [_P, C.c_int64, C.c_char_p, _P, C.c_int64]
    L.cycas_set_graph.argtypes = [_P, C.c_int32]
    L.cycas_batch_autotune.argtypes = [_P, C.c_int32, C.POINTER(C.c_int32), _F64P, _F64P]
    L.cycas_footprint_estimate.argtypes = [_P]
    L.cycas_footprint_estimate.restype = C.c_double
    L.cycas_server_last_error.argtypes = [_P]
    L.cycas_server_last_error.restype = C.c_char_p
    L.cycas_server_stats.argtypes = [_P, _P]
    L.cycas_csr_solve_noalloc.argtypes = [C.c_int32, _P, _P, _P, _P, _P, C.POINTER(KspOptions), C.c_double,
                                          C.c_int32, C.c_int32, _P, C.POINTER(SolveStats)]
    _lib = L
    return L


def last_error() -> str:
    return load().cycas_last_error().decode(errors="replace")


def check(rc: int):
    if rc != CYCAS_OK:
        raise CycasError(rc, last_error())


def ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def default_options(pc=PC_JACOBI, restart=30, device=0) -> Options:
    o = Options()
    load().cycas_options_default(C.byref(o))
    for s in range(3):
        o.ksp[s].pc = pc
        o.ksp[s].restart = restart
    o.device = device
    return o
