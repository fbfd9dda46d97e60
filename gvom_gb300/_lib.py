"""ctypes binding of libgvom_gb300.so (the C ABI in include/gvom_gb300.h).

There is no fallback: if the library is missing or fails to load, `load()`
raises, so nothing silently runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgvom_gb300.so")

GVOM_OK = 0
GVOM_NO_DATA = 1
GVOM_ERR_ARG = 2
GVOM_ERR_OOM = 3
GVOM_ERR_CUDA = 4
GVOM_ERR_TIMEOUT = 5
GVOM_ERR_STATE = 6
GVOM_NONE = -1
GVOM_F32 = 0
GVOM_F64 = 1

# every symbol include/gvom_gb300.h declares
EXPORTS = (
    "gvom_create", "gvom_destroy", "gvom_process", "gvom_process_device", "gvom_process_batch",
    "gvom_combine", "gvom_combine_device", "gvom_debug_voxel_map", "gvom_debug_height_map",
    "gvom_debug_inferred_height_map", "gvom_ring_state", "gvom_slot_count", "gvom_get_slot",
    "gvom_combined_count", "gvom_get_combined", "gvom_get_maps", "gvom_set_stream",
    "gvom_synchronize", "gvom_last_process_stats", "gvom_device_bytes", "gvom_last_error",
    "gvom_version", "gvom_set_stage_timing", "gvom_stage_times", "gvom_stage_name",
    "gvom_debug_voxel_map_noalloc", "gvom_set_graphs", "gvom_set_tuning", "gvom_get_tuning", "gvom_step",
    "gvom_ros_grids", "gvom_process_pointcloud2", "gvom_pose_to_transform", "gvom_reserve",
    "gvom_expand_binary", "gvom_lowpass_binary", "gvom_convolve",
)
GVOM_STAGES = 11


class GvomParams(C.Structure):
    _fields_ = [
        ("xy_resolution", C.c_double), ("z_resolution", C.c_double),
        ("xy_size", C.c_int32), ("z_size", C.c_int32), ("buffer_size", C.c_int32),
        ("min_distance", C.c_double), ("positive_obstacle_threshold", C.c_double),
        ("negative_obstacle_threshold", C.c_double), ("slope_obstacle_threshold", C.c_double),
        ("robot_height", C.c_double), ("robot_radius", C.c_double),
        ("ground_to_lidar_height", C.c_double),
        ("xy_eigen_dist", C.c_int32), ("z_eigen_dist", C.c_int32),
    ]


class GvomScan(C.Structure):
    _fields_ = [
        ("points", C.c_void_p), ("dtype", C.c_int32), ("transform_dtype", C.c_int32),
        ("n", C.c_int64), ("row_stride", C.c_int64), ("ego", C.c_double * 3),
        ("transform", C.c_void_p),
    ]


class GvomTuning(C.Structure):
    _fields_ = [("points_per_block", C.c_int32),
                ("merge_planes_per_thread", C.c_int32), ("stats_blocks_per_sm", C.c_int32),
                ("step_overlap", C.c_int32), ("maps_tile_cells", C.c_int32),
                ("step_pipeline", C.c_int32)]


class GvomRosParams(C.Structure):
    _fields_ = [("density_threshold", C.c_double), ("min_roughness", C.c_double), ("max_roughness", C.c_double)]


class GvomError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def load(path: str | None = None):
    """Load the CUDA library (raises if it is not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                          "or `python gvom_gb300/build.py`")
    lib = C.CDLL(p)
    P = C.c_void_p
    i32, i64 = C.c_int32, C.c_int64
    sig = {
        "gvom_create": ([C.POINTER(GvomParams), C.POINTER(C.c_void_p)], C.c_int),
        "gvom_destroy": ([P], C.c_int),
        "gvom_process": ([P, P, i32, i64, i64, P, P, i32], C.c_int),
        "gvom_process_device": ([P, P, i32, i64, i64, P, P, i32], C.c_int),
        "gvom_process_batch": ([P, C.POINTER(GvomScan), i32, i32], C.c_int),
        "gvom_combine": ([P, P, P, P, P, P], C.c_int),
        "gvom_combine_device": ([P, P, P, P, P, P], C.c_int),
        "gvom_debug_voxel_map": ([P, P, i64, C.POINTER(i64)], C.c_int),
        "gvom_debug_voxel_map_noalloc": ([P, P, i64, C.POINTER(i64)], C.c_int),
        "gvom_set_graphs": ([P, i32], C.c_int),
        "gvom_step": ([P, C.POINTER(GvomScan), i32, i32, P, P, P, P, P, i32], C.c_int),
        "gvom_ros_grids": ([P, C.POINTER(GvomRosParams), P, P, P, P, P, i32], C.c_int),
        "gvom_process_pointcloud2": ([P, P, i64, i32, P, i32, i32, P, P, P], C.c_int),
        "gvom_pose_to_transform": ([P, P, P], C.c_int),
        "gvom_set_tuning": ([P, C.POINTER(GvomTuning)], C.c_int),
        "gvom_get_tuning": ([P, C.POINTER(GvomTuning)], C.c_int),
        "gvom_debug_height_map": ([P, P], C.c_int),
        "gvom_debug_inferred_height_map": ([P, P], C.c_int),
        "gvom_ring_state": ([P, C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "gvom_slot_count": ([P, i32, C.POINTER(i64)], C.c_int),
        "gvom_get_slot": ([P, i32, P, P, P, P, P, P], C.c_int),
        "gvom_combined_count": ([P, C.POINTER(i64)], C.c_int),
        "gvom_get_combined": ([P, P, P, P, P, P, P, P], C.c_int),
        "gvom_get_maps": ([P, P, P, P, P, P, P], C.c_int),
        "gvom_set_stream": ([P, P], C.c_int),
        "gvom_synchronize": ([P], C.c_int),
        "gvom_last_process_stats": ([P, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "gvom_device_bytes": ([P, C.POINTER(i64)], C.c_int),
        "gvom_reserve": ([P, i32, i64, i64], C.c_int),
        "gvom_expand_binary": ([P, P, i32, C.c_double, P], C.c_int),
        "gvom_lowpass_binary": ([P, P, i32, i32, C.c_double, P], C.c_int),
        "gvom_convolve": ([P, P, P, i32, i32, P], C.c_int),
        "gvom_last_error": ([], C.c_char_p),
        "gvom_set_stage_timing": ([P, i32], C.c_int),
        "gvom_stage_times": ([P, C.POINTER(C.c_double), C.POINTER(i64), i32], C.c_int),
        "gvom_stage_name": ([i32], C.c_char_p),
        "gvom_version": ([], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def check(rc: int, allow=(GVOM_OK,)):
    if rc in allow:
        return rc
    lib = load()
    msg = lib.gvom_last_error().decode(errors="replace")
    raise GvomError(rc, msg)
