"""ctypes view of include/velvet_gb300.h.

`lib()` loads velvet_gb300/libvelvet_gb300.so (built in-tree by velvet_gb300.build) and
declares every entry point's signature.  VT_VARIANT in the environment picks another
build of the same sources: `checked` (bounds-checked; VT_CHECKED=1 means the same) or
`fast` (contracted arithmetic, results within the solver's stated tolerance of the exact
build).  There is no fallback: if the library is missing or fails to load, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# the build variant (see build.py): exact (default), checked or fast
VARIANT = os.environ.get("VT_VARIANT") or ("checked" if os.environ.get("VT_CHECKED") == "1" else "exact")
_LIB_NAMES = {"exact": "libvelvet_gb300.so", "checked": "libvelvet_gb300_checked.so",
              "fast": "libvelvet_gb300_fast.so"}
if VARIANT not in _LIB_NAMES:
    raise ValueError(f"VT_VARIANT={VARIANT!r}: expected one of {sorted(_LIB_NAMES)}")
LIB_PATH = Path(__file__).resolve().parent / _LIB_NAMES[VARIANT]

VT_OK = 0
VT_ERR_INVALID_ARGUMENT = -1
VT_ERR_OUT_OF_MEMORY = -2
VT_ERR_CUDA = -3
VT_ERR_NOT_FOUND = -4
VT_ERR_STATE = -5
VT_ERR_CAPACITY = -6
VT_ERR_NUMERIC = -7
VT_ERR_TIMEOUT = -8

COLLIDER_SPHERE, COLLIDER_PLANE, COLLIDER_CUBE = 0, 1, 2

DEBUG_PARTICLE_HASH, DEBUG_PARTICLE_INDEX, DEBUG_CELL_START, DEBUG_CELL_END = 0, 1, 2, 3
DEBUG_NEIGHBORS, DEBUG_PREDICTED, DEBUG_TABLE_SIZE = 4, 5, 6


class VtParams(C.Structure):
    """vt_params — VtSimParams (Velvet/Common.hpp:19-48)."""

    _fields_ = [
        ("num_substeps", C.c_int32),
        ("num_iterations", C.c_int32),
        ("max_num_neighbors", C.c_int32),
        ("max_speed", C.c_float),
        ("gravity", C.c_float * 3),
        ("bend_compliance", C.c_float),
        ("damping", C.c_float),
        ("relaxation_factor", C.c_float),
        ("long_range_stretchiness", C.c_float),
        ("collision_margin", C.c_float),
        ("friction", C.c_float),
        ("enable_self_collision", C.c_int32),
        ("interleaved_hash", C.c_int32),
        ("num_particles", C.c_uint32),
        ("particle_diameter", C.c_float),
        ("delta_time", C.c_float),
        ("particle_diameter_scalar", C.c_float),
        ("hash_cell_size_scalar", C.c_float),
    ]


class VtSdfCollider(C.Structure):
    """vt_sdf_collider — SDFCollider (Velvet/VtClothSolverGPU.cuh:8-18)."""

    _fields_ = [
        ("type", C.c_int32),
        ("position", C.c_float * 3),
        ("scale", C.c_float * 3),
        ("delta_time", C.c_float),
        ("cur_transform", C.c_float * 9),
        ("inv_cur_transform", C.c_float * 16),
        ("last_transform", C.c_float * 16),
    ]


class VtStageTime(C.Structure):
    """vt_stage_time — one profiler row."""

    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("total_ms", C.c_double)]


class VtServerConfig(C.Structure):
    """vt_server_config."""

    _fields_ = [
        ("hbm_budget_bytes", C.c_uint64),
        ("max_cloths", C.c_uint32),
        ("max_active_particles", C.c_uint32),
        ("frame_dt", C.c_float),
        ("substeps", C.c_int32),
        ("iterations", C.c_int32),
        ("relaxation", C.c_float),
        ("friction", C.c_float),
        ("collision_margin", C.c_float),
    ]


class VtServerTickInfo(C.Structure):
    _fields_ = [
        ("admitted", C.c_int32), ("retired", C.c_int32), ("active", C.c_int32), ("queued", C.c_int32),
        ("active_particles", C.c_uint64), ("frame_ms", C.c_double),
    ]


class VtServerStats(C.Structure):
    _fields_ = [
        ("ticks", C.c_uint64), ("frames_done", C.c_uint64), ("requests_done", C.c_uint64),
        ("particle_iterations", C.c_double), ("gpu_ms", C.c_double),
        ("p50_frame_ms", C.c_double), ("p99_frame_ms", C.c_double),
        ("bytes_in_use", C.c_uint64), ("bytes_budget", C.c_uint64), ("requests_failed", C.c_uint64),
        ("requests_cancelled", C.c_uint64),
    ]


class VtGridCloth(C.Structure):
    """vt_grid_cloth — a grid cloth described for device-side construction."""

    _fields_ = [
        ("resolution", C.c_int32),
        ("cloth_size", C.c_float),
        ("model", C.c_float * 16),
        ("particle_diameter", C.c_float),
        ("attached", C.POINTER(C.c_int32)),
        ("n_attached", C.c_uint32),
    ]


class VtRenderParams(C.Structure):
    """vt_render_params — headless sphere-impostor rendering of the particles."""

    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("view", C.c_float * 16), ("projection", C.c_float * 16),
        ("z_near", C.c_float), ("particle_radius", C.c_float),
        ("light_dir", C.c_float * 3), ("tint", C.c_float * 3), ("ambient", C.c_float),
        ("background", C.c_uint32),
    ]


REQ_QUEUED, REQ_ACTIVE, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, 4


class VtHashParams(C.Structure):
    """vt_hash_params — HashParams (Velvet/SpatialHashGPU.cuh:7-15)."""

    _fields_ = [
        ("num_objects", C.c_uint32),
        ("max_num_neighbors", C.c_uint32),
        ("cell_spacing", C.c_float),
        ("cell_spacing2", C.c_float),
        ("table_size", C.c_int32),
        ("particle_diameter2", C.c_float),
    ]


P = C.c_void_p
I32, U32, U64, F32 = C.c_int32, C.c_uint32, C.c_uint64, C.c_float
PF, PI32, PU32 = C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)

# name -> (restype, argtypes): every function include/velvet_gb300.h declares
SIGNATURES: dict[str, tuple] = {
    "vt_params_default": (None, [C.POINTER(VtParams)]),
    "vt_status_string": (C.c_char_p, [I32]),
    "vt_last_error": (C.c_char_p, []),
    "vt_abi_version": (I32, []),
    "vt_solver_create": (I32, [C.POINTER(VtParams), C.POINTER(P)]),
    "vt_solver_destroy": (I32, [P]),
    "vt_solver_get_params": (I32, [P, C.POINTER(VtParams)]),
    "vt_solver_set_params": (I32, [P, C.POINTER(VtParams)]),
    "vt_cloth_add": (I32, [P, P, U32, P, U32, P, F32, PI32]),
    "vt_stretch_add": (I32, [P, P, P, U32]),
    "vt_attach_slot_add": (I32, [P, P, PI32]),
    "vt_attach_add": (I32, [P, P, P, P, U32]),
    "vt_attach_generate_lra": (I32, [P, I32, U32, I32, U32]),
    "vt_bend_add": (I32, [P, P, P, U32]),
    "vt_cloth_build_grid_constraints": (I32, [P, I32, I32, P, U32]),
    "vt_cloth_build_bending_adjacency": (I32, [P, I32, PU32]),
    "vt_colliders_set": (I32, [P, P, U32]),
    "vt_simulate": (I32, [P, F32, I32, I32, F32, F32, F32, F32, P]),
    "vt_solver_sync": (I32, [P]),
    "vt_solver_num_particles": (I32, [P, PU32]),
    "vt_positions_get": (I32, [P, U32, U32, P, I32, P]),
    "vt_normals_get": (I32, [P, U32, U32, P, I32, P]),
    "vt_velocities_get": (I32, [P, U32, U32, P, I32, P]),
    "vt_positions_set": (I32, [P, U32, U32, P, I32, P]),
    "vt_velocities_set": (I32, [P, U32, U32, P, I32, P]),
    "vt_inv_mass_get": (I32, [P, U32, U32, P]),
    "vt_inv_mass_set": (I32, [P, U32, U32, P]),
    "vt_attach_slot_set": (I32, [P, I32, P]),
    "vt_solver_debug_get": (I32, [P, I32, P, U64]),
    "vt_solver_launch_count": (I32, [P, C.POINTER(C.c_uint64)]),
    "vt_solver_state_size": (I32, [P, C.POINTER(C.c_uint64)]),
    "vt_solver_state_save": (I32, [P, P, U64]),
    "vt_solver_state_load": (I32, [P, P, U64]),
    "vt_solver_use_graphs": (I32, [P, I32]),
    "vt_solver_use_grid_kernel": (I32, [P, I32]),
    "vt_batch_create": (I32, [C.POINTER(P)]),
    "vt_batch_destroy": (I32, [P]),
    "vt_batch_add": (I32, [P, P, PI32]),
    "vt_batch_size": (I32, [P, PI32, C.POINTER(C.c_uint64)]),
    "vt_batch_colliders_set": (I32, [P, I32, P, U32]),
    "vt_batch_attach_slot_set": (I32, [P, I32, I32, P]),
    "vt_batch_simulate": (I32, [P, F32, I32, I32, F32, F32, F32, P, P]),
    "vt_batch_sync": (I32, [P]),
    "vt_batch_positions_get": (I32, [P, I32, P, I32, P]),
    "vt_batch_normals_get": (I32, [P, I32, P, I32, P]),
    "vt_batch_velocities_get": (I32, [P, I32, P, I32, P]),
    "vt_batch_all_get": (I32, [P, I32, P, I32, P]),
    "vt_batch_all_get_async": (I32, [P, I32, P, P]),
    "vt_batch_launch_count": (I32, [P, C.POINTER(C.c_uint64)]),
    "vt_batch_use_graphs": (I32, [P, I32]),
    "vt_server_create": (I32, [C.POINTER(VtServerConfig), C.POINTER(P)]),
    "vt_server_destroy": (I32, [P]),
    "vt_server_submit": (I32, [P, P, I32, C.POINTER(C.c_int64)]),
    "vt_server_submit_grid": (I32, [P, C.POINTER(VtGridCloth), C.POINTER(VtParams), P, U32, I32,
                                    C.POINTER(C.c_int64)]),
    "vt_server_tick": (I32, [P, P, C.POINTER(VtServerTickInfo)]),
    "vt_server_poll": (I32, [P, C.c_int64, PI32, PI32]),
    "vt_server_cancel": (I32, [P, C.c_int64]),
    "vt_server_result": (I32, [P, C.c_int64, P, U32]),
    "vt_server_stats_get": (I32, [P, C.POINTER(VtServerStats)]),
    "vt_tuning_set_grid_tile": (I32, [I32]),
    "vt_tuning_set_tile_loads": (I32, [I32]),
    "vt_tuning_set_substep_clusters": (I32, [I32]),
    "vt_solver_grid_tile": (I32, [P, PI32]),
    "vt_batch_grid_tile": (I32, [P, PI32]),
    "vt_camera_look_at": (I32, [PF, PF, PF, PF]),
    "vt_camera_perspective": (I32, [F32, F32, F32, F32, PF]),
    "vt_solver_render": (I32, [P, C.POINTER(VtRenderParams), P, I32, P]),
    "vt_batch_render": (I32, [P, C.POINTER(VtRenderParams), P, I32, P]),
    "vt_profiler_enable": (I32, [I32]),
    "vt_profiler_reset": (I32, []),
    "vt_profiler_read": (I32, [C.POINTER(VtStageTime), U32, PU32]),
    "vt_hash_objects": (I32, [P, P, P, P, P, P, P, C.POINTER(VtHashParams), P]),
    "vt_hash_objects_noalloc": (I32, [P, P, P, P, P, P, P, C.POINTER(VtHashParams), P]),
}

_LIB: C.CDLL | None = None


class VtError(RuntimeError):
    """A vt_* call returned a non-zero status."""

    def __init__(self, status: int, call: str, message: str):
        self.status = status
        super().__init__(f"{call} failed with {status}: {message}")


def lib() -> C.CDLL:
    """The loaded solver library (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, call: str) -> None:
    if status != VT_OK:
        msg = lib().vt_last_error()
        raise VtError(status, call, msg.decode() if msg else "")


def profiler_enable(on: bool = True) -> None:
    check(lib().vt_profiler_enable(1 if on else 0), "vt_profiler_enable")


def profiler_reset() -> None:
    check(lib().vt_profiler_reset(), "vt_profiler_reset")


def profiler_read() -> dict[str, tuple[int, float]]:
    """{stage: (launches, total_ms)} of everything recorded since the last reset."""
    rows = (VtStageTime * 32)()
    n = C.c_uint32()
    check(lib().vt_profiler_read(rows, 32, C.byref(n)), "vt_profiler_read")
    return {rows[i].name.decode(): (int(rows[i].launches), float(rows[i].total_ms))
            for i in range(min(n.value, 32))}


def default_params() -> VtParams:
    p = VtParams()
    lib().vt_params_default(C.byref(p))
    return p
