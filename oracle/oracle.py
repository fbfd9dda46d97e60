"""TEST INFRASTRUCTURE - ctypes front end of the C oracle (oracle/gvom_oracle.c).

`OracleGvom` mirrors the reference mapper's public surface (scripts/gvom.py:21,
105, 222, 395, 412, 428) so parity tests drive the oracle and the GPU library
with the same calls.  Only tests, __graft_entry__.smoke() and bench.py's CPU
baseline use this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import build_oracle

_lib = None


class _Params(C.Structure):
    _fields_ = [
        ("xy_resolution", C.c_double), ("z_resolution", C.c_double),
        ("xy_size", C.c_int32), ("z_size", C.c_int32), ("buffer_size", C.c_int32),
        ("min_distance", C.c_double), ("positive_obstacle_threshold", C.c_double),
        ("negative_obstacle_threshold", C.c_double), ("slope_obstacle_threshold", C.c_double),
        ("robot_height", C.c_double), ("robot_radius", C.c_double),
        ("ground_to_lidar_height", C.c_double),
        ("xy_eigen_dist", C.c_int32), ("z_eigen_dist", C.c_int32),
    ]


def _load():
    global _lib
    if _lib is not None:
        return _lib
    lib = C.CDLL(build_oracle())
    P = C.c_void_p
    i64 = C.c_int64
    lib.gvo_create.restype = P
    lib.gvo_create.argtypes = [C.POINTER(_Params), C.c_int]
    lib.gvo_destroy.argtypes = [P]
    lib.gvo_set_threads.argtypes = [P, C.c_int]
    lib.gvo_process.restype = C.c_int
    lib.gvo_process.argtypes = [P, P, C.c_int, i64, i64, P, P, C.c_int]
    lib.gvo_combine.restype = C.c_int
    lib.gvo_combine.argtypes = [P, P, P, P, P, P]
    lib.gvo_combined_count.restype = i64
    lib.gvo_combined_count.argtypes = [P]
    for name in ("gvo_debug_voxels", "gvo_debug_height_map", "gvo_debug_inferred_height_map"):
        getattr(lib, name).restype = C.c_int
        getattr(lib, name).argtypes = [P, P]
    lib.gvo_get_combined.restype = C.c_int
    lib.gvo_get_combined.argtypes = [P] + [P] * 7
    lib.gvo_get_maps.restype = C.c_int
    lib.gvo_get_maps.argtypes = [P] + [P] * 6
    lib.gvo_slot_count.restype = i64
    lib.gvo_slot_count.argtypes = [P, C.c_int]
    lib.gvo_get_slot.restype = C.c_int
    lib.gvo_get_slot.argtypes = [P, C.c_int] + [P] * 6
    lib.gvo_ring_state.argtypes = [P, P, P]
    lib.gvo_last_process_stats.argtypes = [P, P, P, P]
    lib.gvo_expand_binary.argtypes = [P, P, C.c_int, C.c_double]
    lib.gvo_lowpass_binary.argtypes = [P, P, C.c_int, C.c_int, C.c_double]
    lib.gvo_convolve.argtypes = [P, P, P, C.c_int, C.c_int]
    _lib = lib
    return lib


def expand_binary(img, r):
    """__expand_binary (scripts/gvom.py:807-831) on an (X, X) int32 image."""
    a = np.ascontiguousarray(img, np.int32)
    out = np.empty_like(a)
    _load().gvo_expand_binary(_ptr(a), _ptr(out), a.shape[0], float(r))
    return out


def lowpass_binary(img, filter_size, filter_fraction):
    """__lowpass_binary (scripts/gvom.py:833-861) on an (X, X) int32 image."""
    a = np.ascontiguousarray(img, np.int32)
    out = np.empty_like(a)
    _load().gvo_lowpass_binary(_ptr(a), _ptr(out), a.shape[0], int(filter_size), float(filter_fraction))
    return out


def convolve(img, kernel):
    """__convolve (scripts/gvom.py:863-885) as written, integer radius."""
    a = np.ascontiguousarray(img, np.float64)
    k = np.ascontiguousarray(kernel, np.float64)
    out = np.empty_like(a)
    _load().gvo_convolve(_ptr(a), _ptr(out), _ptr(k), a.shape[0], k.shape[0])
    return out


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class OracleGvom:
    """CPU oracle with the reference `Gvom` constructor and methods."""

    def __init__(self, xy_resolution, z_resolution, xy_size, z_size, buffer_size, min_distance,
                 positive_obstacle_threshold, negative_obstacle_threshold, slope_obsacle_threshold,
                 robot_height, robot_radius, ground_to_lidar_height, xy_eigen_dist=1,
                 z_eigen_dist=1, threads: int = 1):
        lib = _load()
        self.xy_resolution = float(xy_resolution)
        self.z_resolution = float(z_resolution)
        self.xy_size = int(xy_size)
        self.z_size = int(z_size)
        self.buffer_size = int(buffer_size)
        self.voxel_count = self.xy_size * self.xy_size * self.z_size
        p = _Params(float(xy_resolution), float(z_resolution), int(xy_size), int(z_size),
                    int(buffer_size), float(min_distance), float(positive_obstacle_threshold),
                    float(negative_obstacle_threshold), float(slope_obsacle_threshold),
                    float(robot_height), float(robot_radius), float(ground_to_lidar_height),
                    int(xy_eigen_dist), int(z_eigen_dist))
        self._h = lib.gvo_create(C.byref(p), int(threads))
        if not self._h:
            raise ValueError("oracle: invalid parameters")
        self._lib = lib

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.gvo_destroy(h)
            self._h = None

    def set_threads(self, n: int):
        self._lib.gvo_set_threads(self._h, int(n))

    # -- reference API -----------------------------------------------------
    def Process_pointcloud(self, pointcloud, ego_position, transform=None):
        pc = np.asarray(pointcloud)
        if pc.dtype not in (np.float32, np.float64):
            pc = pc.astype(np.float64)
        if pc.ndim != 2 or pc.shape[1] < 3:
            raise ValueError("pointcloud must have shape (N, >=3)")
        pc = np.ascontiguousarray(pc)
        dt = 1 if pc.dtype == np.float64 else 0
        ego = np.ascontiguousarray(np.asarray(ego_position, dtype=np.float64).reshape(3))
        T = None
        tdt = -1
        if transform is not None:
            T = np.asarray(transform)
            if T.dtype not in (np.float32, np.float64):
                T = T.astype(np.float64)
            T = np.ascontiguousarray(T.reshape(4, 4))
            tdt = 1 if T.dtype == np.float64 else 0
        rc = self._lib.gvo_process(self._h, _ptr(pc), dt, pc.shape[0], pc.shape[1], _ptr(ego),
                                   _ptr(T), tdt)
        if rc != 0:
            raise RuntimeError(f"oracle process failed ({rc})")

    process_pointcloud = Process_pointcloud

    def combine_maps(self):
        X = self.xy_size
        origin = np.zeros(3)
        pos = np.zeros((X, X), np.int32)
        neg = np.zeros((X, X), np.int32)
        rough = np.zeros((X, X), np.float64)
        vis = np.zeros((X, X), np.int32)
        rc = self._lib.gvo_combine(self._h, _ptr(origin), _ptr(pos), _ptr(neg), _ptr(rough), _ptr(vis))
        if rc == 1:
            print("ERROR: No data in buffer")
            return None
        if rc != 0:
            raise RuntimeError(f"oracle combine failed ({rc})")
        return origin, pos, neg, rough, vis

    def make_debug_voxel_map(self):
        n = self._lib.gvo_combined_count(self._h)
        if n < 0:
            print("No data")
            return None
        out = np.zeros((n, 8), np.float32)
        self._lib.gvo_debug_voxels(self._h, _ptr(out))
        return out

    def make_debug_height_map(self):
        out = np.zeros((self.xy_size * self.xy_size, 7), np.float32)
        if self._lib.gvo_debug_height_map(self._h, _ptr(out)) != 0:
            print("No data")
            return None
        return out

    def make_debug_inferred_height_map(self):
        out = np.zeros((self.xy_size * self.xy_size, 3), np.float32)
        if self._lib.gvo_debug_inferred_height_map(self._h, _ptr(out)) != 0:
            print("No data")
            return None
        return out

    # -- state access for parity checks -------------------------------------
    def combined_state(self):
        n = self._lib.gvo_combined_count(self._h)
        if n < 0:
            return None
        V = self.voxel_count
        st = dict(index=np.zeros(V, np.int32), hit=np.zeros(n, np.int32), total=np.zeros(n, np.int32),
                  min_h=np.zeros(n, np.float32), metrics=np.zeros((n, 10), np.float32),
                  eigen=np.zeros((n, 3), np.float32), origin=np.zeros(3))
        self._lib.gvo_get_combined(self._h, *[_ptr(st[k]) for k in
                                              ("index", "hit", "total", "min_h", "metrics", "eigen", "origin")])
        return st

    def maps_state(self):
        X = self.xy_size
        keys = ("height", "inferred", "slope_x", "slope_y", "roughness", "guess")
        st = {k: np.zeros((X, X)) for k in keys}
        if self._lib.gvo_get_maps(self._h, *[_ptr(st[k]) for k in keys]) != 0:
            return None
        return st

    def slot_state(self, slot: int):
        n = self._lib.gvo_slot_count(self._h, int(slot))
        if n < 0:
            return None
        st = dict(index=np.zeros(self.voxel_count, np.int32), hit=np.zeros(n, np.int32),
                  total=np.zeros(n, np.int32), min_h=np.zeros(n, np.float32),
                  metrics=np.zeros((n, 10), np.float64), origin=np.zeros(3))
        self._lib.gvo_get_slot(self._h, int(slot), *[_ptr(st[k]) for k in
                                                     ("index", "hit", "total", "min_h", "metrics", "origin")])
        return st

    def ring_state(self):
        a = C.c_int64()
        b = C.c_int64()
        self._lib.gvo_ring_state(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def last_process_stats(self):
        s, h, v = C.c_int64(), C.c_int64(), C.c_int64()
        self._lib.gvo_last_process_stats(self._h, C.byref(s), C.byref(h), C.byref(v))
        return dict(ray_steps=s.value, hits=h.value, valid_points=v.value)
