"""ctypes binding of the pdgb C ABI (include/pdgb.h).

The engine lives in ``_lib/libpdgb.so`` next to this file.  There is no
fallback: if the library is missing or cannot load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# PDGB_LIBRARY may name another build of the same library (e.g. a tuning variant).
_LIB_PATH = Path(os.environ.get("PDGB_LIBRARY") or (Path(__file__).resolve().parent / "_lib" / "libpdgb.so"))

PDGB_OK = 0
PDGB_ERR_INVALID_ARGUMENT = 1
PDGB_ERR_BAD_MESH = 2
PDGB_ERR_NOT_SPD = 3
PDGB_ERR_CUDA = 4
PDGB_ERR_OUT_OF_MEMORY = 5
PDGB_ERR_NONFINITE = 6
PDGB_ERR_UNSUPPORTED = 7
PDGB_ERR_TIMEOUT = 8
PDGB_ERR_NOT_FOUND = 9
PDGB_ERR_BUSY = 10

PDGB_MEM_HOST = 0
PDGB_MEM_DEVICE = 1
PDGB_SOLVER_JACOBI = 0
PDGB_SOLVER_CHOLESKY = 1
PDGB_ROTATION_QUAT = 0
PDGB_ROTATION_SVD = 1
PDGB_LOCAL_TILE = 0
PDGB_LOCAL_PIPELINED = 1
PDGB_ORDER_AMD = 0
PDGB_ORDER_ND = 1
PDGB_ORDER_DENSE = 2
PDGB_SOLVE_AUTO = 0
PDGB_SOLVE_CTA = 1
PDGB_SOLVE_CLUSTER = 2
PDGB_SOLVE_LEVELS = 3
PDGB_SOLVE_DSM = 4
PDGB_SOLVE_PERSISTENT = 5
PDGB_FACTOR_GPU = 0
PDGB_FACTOR_HOST = 1
PDGB_TIMING_OFF = 0
PDGB_TIMING_STEPS = 1
PDGB_TIMING_KERNELS = 2
PDGB_FIXED_SPHERE = 0
PDGB_FIXED_PLANE = 1
PDGB_FIXED_CYLINDER = 2


class pdgb_params(C.Structure):
    _fields_ = [
        ("dt", C.c_float),
        ("gravity", C.c_float),
        ("num_iterations", C.c_int),
        ("tol", C.c_float),
        ("rho", C.c_float),
        ("positional_weight", C.c_float),
        ("solver", C.c_int),
        ("refine_steps", C.c_int),
    ]


class pdgb_mesh_desc(C.Structure):
    _fields_ = [
        ("num_verts", C.c_int),
        ("num_tets", C.c_int),
        ("X", C.c_void_p),
        ("V", C.c_void_p),
        ("tets", C.c_void_p),
        ("mass", C.c_void_p),
        ("mu", C.c_void_p),
        ("dbc", C.c_void_p),
        ("memory", C.c_int),
    ]


class pdgb_perf(C.Structure):
    _fields_ = [
        ("prepare_ms", C.c_double),
        ("steps", C.c_double),
        ("iterations", C.c_double),
        ("factor_nnz", C.c_longlong),
        ("tiles", C.c_longlong),
        ("patch_verts", C.c_longlong),
    ]


class pdgb_timing(C.Structure):
    _fields_ = [
        ("step_ms", C.c_double),
        ("steps", C.c_longlong),
        ("local_ms", C.c_double),
        ("local_launches", C.c_longlong),
        ("solve_ms", C.c_double),
        ("solves", C.c_longlong),
    ]


class pdgb_noalloc_mesh(C.Structure):
    _fields_ = [
        ("num_verts", C.c_int),
        ("num_tets", C.c_int),
        ("tets", C.c_void_p),
        ("X0", C.c_void_p),
        ("mass", C.c_void_p),
        ("mu", C.c_void_p),
        ("dbc", C.c_void_p),
    ]


class pdgb_server_config(C.Structure):
    _fields_ = [
        ("params", pdgb_params),
        ("hbm_budget_bytes", C.c_size_t),
        ("max_active", C.c_int),
        ("host_threads", C.c_int),
        ("cache_entries", C.c_int),
        ("reserved", C.c_int),
    ]


class pdgb_server_stats(C.Structure):
    _fields_ = [
        ("completed", C.c_longlong),
        ("failed", C.c_longlong),
        ("active", C.c_int),
        ("waiting", C.c_int),
        ("bytes_in_use", C.c_size_t),
        ("tet_iterations", C.c_double),
        ("busy_ms", C.c_double),
        ("admit_ms", C.c_double),
        ("step_ms", C.c_double),
        ("ticks", C.c_longlong),
        ("ready", C.c_int),
        ("layout_cache_hits", C.c_int),
        ("nonfinite", C.c_longlong),
        ("factors", C.c_longlong),
        ("factor_cache_hits", C.c_longlong),
        ("factor_ms", C.c_double),
        ("finishing", C.c_int),
        ("reserved", C.c_int),
    ]


PDGB_REQ_QUEUED, PDGB_REQ_PREPARING, PDGB_REQ_READY, PDGB_REQ_RUNNING, PDGB_REQ_DONE, PDGB_REQ_FAILED = range(6)


class pdgb_factor_info(C.Structure):
    _fields_ = [
        ("nnz_L", C.c_longlong),
        ("m_entries", C.c_longlong),
        ("num_supernodes", C.c_int),
        ("num_levels", C.c_int),
        ("fwd_items", C.c_int),
        ("bwd_items", C.c_int),
        ("flops", C.c_double),
        ("factor_ms", C.c_double),
        ("solve_launches", C.c_int),
        ("numeric_device", C.c_int),
        ("numeric_ms", C.c_double),
        ("pool_bytes", C.c_longlong),
    ]


class pdgb_layout_info(C.Structure):
    _fields_ = [
        ("num_tiles", C.c_int),
        ("max_patch", C.c_int),
        ("max_tile_tets", C.c_int),
        ("reserved", C.c_int),
        ("patch_verts", C.c_longlong),
    ]


class pdgb_fixed_body(C.Structure):
    _fields_ = [
        ("type", C.c_int),
        ("model", C.c_float * 16),
        ("radius", C.c_float),
        ("up", C.c_float * 3),
    ]


class pdgb_body_file(C.Structure):
    _fields_ = [
        ("node_file", C.c_char_p),
        ("ele_file", C.c_char_p),
        ("face_file", C.c_char_p),
        ("msh_file", C.c_char_p),
        ("pos", C.c_float * 3),
        ("scale", C.c_float * 3),
        ("rot", C.c_float * 3),
        ("centralize", C.c_int),
        ("start_index", C.c_int),
    ]


class pdgb_tet_mesh(C.Structure):
    _fields_ = [
        ("num_verts", C.c_int),
        ("num_tets", C.c_int),
        ("num_tris", C.c_int),
        ("num_edges", C.c_int),
        ("X", C.POINTER(C.c_float)),
        ("tets", C.POINTER(C.c_uint32)),
        ("tris", C.POINTER(C.c_uint32)),
        ("edges", C.POINTER(C.c_uint32)),
    ]


class pdgb_tune_report(C.Structure):
    _fields_ = [
        ("tile_tets", C.c_int),
        ("solve_mode", C.c_int),
        ("candidates", C.c_int),
        ("ordering", C.c_int),
        ("best_ms", C.c_double),
        ("default_ms", C.c_double),
    ]


# name -> (restype, argtypes); every symbol include/pdgb.h declares.
class pdgb_collision_info(C.Structure):
    _fields_ = [
        ("candidate_pairs", C.c_longlong),
        ("vertices_hit", C.c_int),
        ("regrows", C.c_int),
        ("detect_ms", C.c_double),
    ]


SIGNATURES = {
    "pdgb_default_params": (None, [C.POINTER(pdgb_params)]),
    "pdgb_create": (C.c_int, [C.POINTER(pdgb_mesh_desc), C.POINTER(pdgb_params), C.c_void_p, C.POINTER(C.c_void_p)]),
    "pdgb_prepare": (C.c_int, [C.c_void_p]),
    "pdgb_create_batch": (C.c_int, [C.c_int, C.POINTER(pdgb_mesh_desc), C.POINTER(pdgb_params), C.c_void_p,
                                    C.POINTER(C.c_void_p)]),
    "pdgb_num_bodies": (C.c_int, [C.c_void_p]),
    "pdgb_download_body": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_step": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_set_solver": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_set_params": (C.c_int, [C.c_void_p, C.POINTER(pdgb_params)]),
    "pdgb_upload_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_download_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_reset": (C.c_int, [C.c_void_p]),
    "pdgb_get_perf": (C.c_int, [C.c_void_p, C.POINTER(pdgb_perf)]),
    "pdgb_last_step_iterations": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "pdgb_synchronize": (C.c_int, [C.c_void_p]),
    "pdgb_last_step_status": (C.c_int, [C.c_void_p]),
    "pdgb_grid_sync_check": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_longlong]),
    "pdgb_enable_kernel_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_read_timing": (C.c_int, [C.c_void_p, C.POINTER(pdgb_timing)]),
    "pdgb_local_step_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "pdgb_solve_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "pdgb_set_solve_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_set_tile_size": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_time_local": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "pdgb_closest_rotations": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(pdgb_tune_report)]),
    "pdgb_get_solve_mode": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "pdgb_destroy": (C.c_int, [C.c_void_p]),
    "pdgb_stream": (C.c_void_p, [C.c_void_p]),
    "pdgb_status_string": (C.c_char_p, [C.c_int]),
    "pdgb_last_error": (C.c_char_p, []),
    "pdgb_version": (C.c_char_p, []),
    "pdgb_set_ordering": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_get_factor_info": (C.c_int, [C.c_void_p, C.POINTER(pdgb_factor_info)]),
    "pdgb_set_factor_device": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_get_factor_blocks": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "pdgb_set_rotation": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_set_local_kernel": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_bulk_wait_check": (C.c_int, [C.c_int, C.c_longlong]),
    "pdgb_get_local_kernel": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pdgb_host_factor_check": (C.c_int, [C.POINTER(pdgb_mesh_desc), C.POINTER(pdgb_params), C.c_int, C.c_void_p,
                                         C.c_void_p, C.POINTER(pdgb_factor_info)]),
    "pdgb_step_noalloc": (C.c_int, [C.POINTER(pdgb_noalloc_mesh), C.POINTER(pdgb_params), C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_void_p]),
    "pdgb_server_default_config": (None, [C.POINTER(pdgb_server_config)]),
    "pdgb_server_create": (C.c_int, [C.POINTER(pdgb_server_config), C.c_void_p, C.POINTER(C.c_void_p)]),
    "pdgb_server_submit": (C.c_int, [C.c_void_p, C.POINTER(pdgb_mesh_desc), C.c_int, C.POINTER(C.c_longlong)]),
    "pdgb_server_tick": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pdgb_server_poll": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pdgb_server_result": (C.c_int, [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]),
    "pdgb_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(pdgb_server_stats)]),
    "pdgb_server_latencies": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "pdgb_server_destroy": (C.c_int, [C.c_void_p]),
    "pdgb_inspect_layout": (C.c_int, [C.POINTER(pdgb_mesh_desc), C.POINTER(pdgb_layout_info), C.c_void_p,
                                      C.c_void_p]),
    "pdgb_set_drag": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_drag_select": (C.c_int, [C.c_void_p, C.c_int, C.c_float, C.c_double]),
    "pdgb_set_drag_target": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "pdgb_clear_drag": (C.c_int, [C.c_void_p]),
    "pdgb_set_fixed_bodies": (C.c_int, [C.c_void_p, C.POINTER(pdgb_fixed_body), C.c_int, C.c_float, C.c_float]),
    "pdgb_download_xtilde": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_set_collision_surface": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "pdgb_enable_collision": (C.c_int, [C.c_void_p, C.c_int]),
    "pdgb_get_collision": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(pdgb_collision_info)]),
    "pdgb_ccd_detect": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.POINTER(pdgb_collision_info)]),
    "pdgb_load_body_file": (C.c_int, [C.POINTER(pdgb_body_file), C.POINTER(C.POINTER(pdgb_tet_mesh))]),
    "pdgb_free_tet_mesh": (None, [C.POINTER(pdgb_tet_mesh)]),
    "pdgb_surface_triangles": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_int)]),
    "pdgb_render_surface": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
}

_lib = None


class PdgbError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {message} (status {status})")
        self.status = status


def library_path() -> Path:
    return _LIB_PATH


def lib() -> C.CDLL:
    """Loads libpdgb.so (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"pdgb native library not built: {_LIB_PATH} is missing; run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        h = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(status: int, where: str) -> None:
    if status != PDGB_OK:
        msg = lib().pdgb_last_error().decode(errors="replace")
        raise PdgbError(status, where, msg or lib().pdgb_status_string(status).decode())
