"""ctypes binding of libcfdgpu.so (include/cfdgpu.h).

The library is the only compute path: if it is missing or no CUDA device is
usable, the calls raise; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcfdgpu.so")

CFDG_OK = 0
CFDG_E031, CFDG_E032, CFDG_E033, CFDG_E034, CFDG_E035, CFDG_E036 = 31, 32, 33, 34, 35, 36
CFDG_CANCELLED, CFDG_WALL_TIME = 100, 101
CFDG_ERR_CUDA, CFDG_ERR_ADMISSION, CFDG_ERR_TIMEOUT, CFDG_ERR_INVALID, CFDG_ERR_UNSUPPORTED = 200, 201, 202, 203, 204
CFDG_PENDING = 3
PRECOND = {"ic0": 0, "multigrid": 1}
PRECISION = {"plain": 0, "mixed": 1}

# Every symbol include/cfdgpu.h declares.
EXPORTS = (
    "cfdg_context_create", "cfdg_context_destroy", "cfdg_grid_open", "cfdg_grid_close",
    "cfdg_grid_update_faces", "cfdg_grid_configure", "cfdg_project", "cfdg_solve_scaled", "cfdg_apply",
    "cfdg_center_nullspaces", "cfdg_multigrid_stats_json", "cfdg_last_error", "cfdg_project_device",
    "cfdg_grid_device_bytes", "cfdg_debug_precondition", "cfdg_debug_projection_rhs", "cfdg_grid_set_stream",
    "cfdg_launch_count", "cfdg_debug_time_kernel", "cfdg_residual_norm_noalloc", "cfdg_batch_create",
    "cfdg_batch_destroy", "cfdg_batch_set_stream", "cfdg_batch_size", "cfdg_batch_project", "cfdg_batch_project_device",
    "cfdg_batch_time_kernel", "cfdg_batch_stats_json", "cfdg_server_create", "cfdg_server_destroy", "cfdg_server_set_stream",
    "cfdg_server_submit", "cfdg_server_progress", "cfdg_server_result", "cfdg_server_pending", "cfdg_server_stats_json", "cfdg_server_set_chunk", "cfdg_grid_set_cycle", "cfdg_grid_set_coarse_scale", "cfdg_grid_set_flow", "cfdg_step_device", "cfdg_scalar_step_device", "cfdg_receptors_set", "cfdg_receptors_sample", "cfdg_debug_momentum_update",
    "cfdg_debug_wave_stall", "cfdg_grid_set_sweep_tile", "cfdg_server_submit_host", "cfdg_batch_debug_rhs",
    "cfdg_debug_div_check", "cfdg_grid_set_coarse_layout", "cfdg_scalar_step_budget", "cfdg_scalar_rates",
    "cfdg_grid_set_advection",
)


class GridDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3),
        ("dx", C.c_double * 3),
        ("volume", C.c_double),
        ("periodic", C.c_int32 * 3),
        ("n_faces", C.c_int64),
        ("fluid", C.c_void_p),
        ("face_kind", C.c_void_p),
        ("face_lo", C.c_void_p),
        ("face_hi", C.c_void_p),
        ("face_area", C.c_void_p),
        ("face_distance", C.c_void_p),
        ("component", C.c_void_p),
        ("n_components", C.c_int32),
        ("anchored", C.c_void_p),
        ("preconditioner", C.c_int32),
        ("precision", C.c_int32),
    ]


class Info(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint64),
        ("relative_residual", C.c_double),
        ("work_units", C.c_uint64),
        ("operator_applications", C.c_uint64),
        ("preconditioner_applications", C.c_uint64),
        ("true_residual_checks", C.c_uint64),
        ("hierarchy_builds", C.c_uint64),
        ("hierarchy_levels", C.c_uint64),
        ("hierarchy_cells", C.c_uint64),
        ("hierarchy_nonzeros", C.c_uint64),
        ("cycles", C.c_uint64),
        ("smoothing_cell_updates", C.c_uint64),
        ("residual_cell_updates", C.c_uint64),
        ("restriction_cell_updates", C.c_uint64),
        ("prolongation_cell_updates", C.c_uint64),
        ("coarse_solves", C.c_uint64),
        ("refinement_steps", C.c_uint64),
        ("device_seconds", C.c_double),
        ("graph_launches", C.c_uint64),
        ("loop_seconds", C.c_double),
        ("hierarchy_bytes", C.c_uint64),
        ("block_smoothing_cell_updates", C.c_uint64),
        ("block_solves", C.c_uint64),
        ("block_level_cell_visits", C.c_uint64),
        ("factor_setup_seconds", C.c_double),
        ("multigrid_setup_seconds", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class FlowDesc(C.Structure):
    """cfdg_flow_desc: the laminar flow terms of a case (cfdg_grid_set_flow)."""

    _fields_ = [
        ("boundary", C.c_int32 * 3),
        ("size_m", C.c_double * 3),
        ("velocity", C.c_double * 3),
        ("viscosity", C.c_double),
        ("acceleration", C.c_double * 3),
    ]


POLL = C.CFUNCTYPE(C.c_int, C.c_void_p)
_lock = threading.Lock()
_lib = None


def load(path: str = LIB_PATH):
    """Loads libcfdgpu.so and declares its signatures. Raises if it was not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(f"the CUDA engine library is missing ({path}); run __graft_entry__.build()")
        L = C.CDLL(path)
        P = C.c_void_p
        L.cfdg_last_error.restype = C.c_char_p
        L.cfdg_context_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]
        L.cfdg_context_destroy.argtypes = [P]
        L.cfdg_context_destroy.restype = None
        L.cfdg_grid_open.argtypes = [P, C.POINTER(GridDesc), C.POINTER(C.c_void_p)]
        L.cfdg_grid_close.argtypes = [P]
        L.cfdg_grid_close.restype = None
        L.cfdg_grid_update_faces.argtypes = [P, P, P]
        L.cfdg_grid_configure.argtypes = [P, C.c_int32, C.c_int32]
        L.cfdg_project.argtypes = [P, P, P, C.c_double, C.c_double, C.c_uint64, POLL, P, C.POINTER(Info)]
        L.cfdg_project_device.argtypes = [P, P, P, C.c_double, C.c_double, C.c_uint64, POLL, P, C.POINTER(Info)]
        L.cfdg_solve_scaled.argtypes = [P, P, P, C.c_double, C.c_uint64, POLL, P, P, C.POINTER(Info)]
        L.cfdg_apply.argtypes = [P, P, P]
        L.cfdg_center_nullspaces.argtypes = [P, P]
        L.cfdg_multigrid_stats_json.argtypes = [P, C.c_char_p, C.c_size_t]
        L.cfdg_grid_device_bytes.argtypes = [P]
        L.cfdg_grid_device_bytes.restype = C.c_uint64
        L.cfdg_debug_precondition.argtypes = [P, P, P]
        L.cfdg_debug_projection_rhs.argtypes = [P, P, C.c_double, P, P]
        L.cfdg_grid_set_stream.argtypes = [P, P]
        L.cfdg_launch_count.argtypes = []
        L.cfdg_launch_count.restype = C.c_uint64
        L.cfdg_residual_norm_noalloc.argtypes = [P, P, P, P, P]
        L.cfdg_batch_create.argtypes = [P, C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]
        L.cfdg_batch_destroy.argtypes = [P]
        L.cfdg_batch_destroy.restype = None
        L.cfdg_batch_set_stream.argtypes = [P, P]
        L.cfdg_server_create.argtypes = [P, C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]
        L.cfdg_server_destroy.argtypes = [P]
        L.cfdg_server_destroy.restype = None
        L.cfdg_server_set_stream.argtypes = [P, P]
        L.cfdg_server_submit.argtypes = [P, C.c_int32, P, P, C.c_double, C.c_double, C.c_uint64,
                                         C.POINTER(C.c_uint64)]
        L.cfdg_server_progress.argtypes = [P, C.POINTER(C.c_int32)]
        L.cfdg_server_submit_host.argtypes = [P, C.c_int32, P, P, P, P, C.c_double, C.c_double, C.c_uint64,
                                              C.POINTER(C.c_uint64)]
        L.cfdg_server_result.argtypes = [P, C.c_uint64, C.POINTER(Info), C.POINTER(C.c_int32)]
        L.cfdg_server_pending.argtypes = [P]
        L.cfdg_batch_time_kernel.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.cfdg_batch_size.argtypes = [P]
        L.cfdg_batch_debug_rhs.argtypes = [P, C.c_int32, P, P]
        L.cfdg_debug_div_check.argtypes = [C.c_double, C.c_uint64, C.c_int64, C.c_int32, C.POINTER(C.c_uint64)]
        L.cfdg_batch_stats_json.argtypes = [P, C.c_char_p, C.c_int64]
        L.cfdg_batch_stats_json.restype = C.c_int64
        L.cfdg_server_stats_json.argtypes = [P, C.c_char_p, C.c_int64]
        L.cfdg_server_stats_json.restype = C.c_int64
        L.cfdg_server_set_chunk.argtypes = [P, C.c_int32]
        L.cfdg_grid_set_cycle.argtypes = [P, C.c_int32, C.c_int32]
        L.cfdg_grid_set_coarse_scale.argtypes = [P, C.c_double]
        L.cfdg_grid_set_coarse_layout.argtypes = [P, C.c_int32]
        L.cfdg_grid_set_flow.argtypes = [P, C.POINTER(FlowDesc)]
        L.cfdg_step_device.argtypes = [P, P, P, C.c_double, C.c_double, C.c_uint64, POLL, P, C.POINTER(Info)]
        L.cfdg_debug_momentum_update.argtypes = [P, P, P, C.c_double, P]
        L.cfdg_scalar_step_device.argtypes = [P, P, P, P, P, C.c_double]
        L.cfdg_scalar_step_budget.argtypes = [P, P, P, P, P, C.c_double, P]
        L.cfdg_scalar_rates.argtypes = [P, P, P, P, P, C.POINTER(C.c_double)]
        L.cfdg_grid_set_advection.argtypes = [P, C.c_int32]
        L.cfdg_receptors_set.argtypes = [P, C.c_int32, P, P, P]
        L.cfdg_receptors_sample.argtypes = [P, P, P]
        PP = C.POINTER(C.c_void_p)
        L.cfdg_batch_project.argtypes = [P, PP, PP, C.POINTER(C.c_double), C.c_double, C.c_uint64, POLL, P,
                                         C.POINTER(Info), C.POINTER(C.c_int32)]
        L.cfdg_batch_project_device.argtypes = [P, PP, PP, C.POINTER(C.c_double), C.c_double, C.c_uint64, POLL, P,
                                                C.POINTER(Info), C.POINTER(C.c_int32)]
        L.cfdg_debug_time_kernel.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.cfdg_debug_wave_stall.argtypes = [P, C.c_int32, C.c_int64]
        L.cfdg_grid_set_sweep_tile.argtypes = [P, C.c_int32, C.c_int32]
        _lib = L
        return L


def last_error() -> str:
    return load().cfdg_last_error().decode()
