"""Drop-in `Gvom` mapper on GB300 CUDA kernels (reference: scripts/gvom.py).

Same constructor (14 positional parameters, scripts/gvom.py:21-22), same
methods and return values:

* ``Process_pointcloud(pointcloud, ego_position, transform=None)`` and its
  README spelling ``process_pointcloud`` (scripts/gvom.py:105): voxelises one
  scan into the ring buffer.  ``pointcloud`` is an (N, >=3) float32/float64
  array (NumPy, or a torch tensor on the CPU or on the GPU); ``transform`` an
  optional 4x4 float32/float64 matrix.  The caller's array is never modified.
* ``combine_maps()`` (scripts/gvom.py:222-393) returns ``(origin float64[3],
  positive int32[X,X], negative int32[X,X], roughness float64[X,X],
  visibility int32[X,X])`` as fresh host arrays, or prints
  "ERROR: No data in buffer" and returns None on an empty ring.
* ``make_debug_voxel_map / make_debug_height_map /
  make_debug_inferred_height_map`` (scripts/gvom.py:395-442).  The voxel rows
  come in ascending voxel-id order (the reference's order is that of its
  atomic allocation, which is not reproducible).

Everything runs in libgvom_gb300.so; this module only moves arguments.
Extra (non-reference) methods: ``process_batch`` (several scans in one set of
launches), ``combine_maps_device`` (outputs into device tensors), state
accessors used by the parity tests, ``synchronize``, ``set_stream``.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _lib
from ._lib import GVOM_F32, GVOM_F64, GVOM_NO_DATA, GVOM_NONE, GvomParams, GvomScan, check


def _native_float(dt) -> bool:
    return dt.char in "fd" and dt.isnative


def _as_points(pointcloud):
    """Return (pointer, dtype code, n, row_stride, keepalive, on_device)."""
    if type(pointcloud) is np.ndarray:  # the common case, without conversions
        a = pointcloud
        if a.ndim == 2 and a.shape[1] >= 3 and _native_float(a.dtype) and a.flags.c_contiguous:
            return a.ctypes.data, (GVOM_F64 if a.dtype.char == "d" else GVOM_F32), a.shape[0], a.shape[1], a, False
    try:  # torch tensor?
        import torch  # noqa: F401
        is_tensor = type(pointcloud).__module__.startswith("torch")
    except Exception:  # pragma: no cover - torch missing
        is_tensor = False
    if is_tensor:
        t = pointcloud
        if t.dim() != 2 or t.shape[1] < 3:
            raise ValueError("pointcloud must have shape (N, >=3)")
        import torch
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float64)
        if t.stride(1) != 1 or (t.shape[0] > 1 and t.stride(0) < t.shape[1]):
            t = t.contiguous()
        code = GVOM_F64 if t.dtype == torch.float64 else GVOM_F32
        if t.is_cuda:
            return C.c_void_p(t.data_ptr()), code, t.shape[0], t.stride(0) if t.shape[0] > 1 else t.shape[1], t, True
        t = t.numpy()
        pointcloud = t
    a = np.asarray(pointcloud)
    if a.ndim != 2 or a.shape[1] < 3:
        raise ValueError("pointcloud must have shape (N, >=3)")
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    if not a.flags.c_contiguous:
        a = np.ascontiguousarray(a)
    code = GVOM_F64 if a.dtype == np.float64 else GVOM_F32
    return a.ctypes.data, code, a.shape[0], a.shape[1], a, False


def _as_transform(transform):
    if transform is None:
        return None, GVOM_NONE, None
    if type(transform) is np.ndarray and transform.shape == (4, 4) and _native_float(transform.dtype) \
            and transform.flags.c_contiguous:
        return transform.ctypes.data, (GVOM_F64 if transform.dtype.char == "d" else GVOM_F32), transform
    try:
        import torch
        if isinstance(transform, torch.Tensor):
            transform = transform.detach().cpu().numpy()
    except Exception:  # pragma: no cover
        pass
    T = np.asarray(transform)
    if T.dtype not in (np.float32, np.float64):
        T = T.astype(np.float64)
    T = np.ascontiguousarray(T.reshape(4, 4))
    return T.ctypes.data, (GVOM_F64 if T.dtype == np.float64 else GVOM_F32), T


def _ego3(ego_position):
    return np.array(ego_position, np.float64).reshape(3)  # a fresh C-contiguous copy


_D3 = C.c_double * 3


def _ego_c(ego_position):
    """The ego position as a ctypes double[3] (passed by address without a
    numpy .ctypes lookup): three numbers directly, any other shape that holds
    three values through numpy."""
    try:
        x, y, z = ego_position
        return _D3(float(x), float(y), float(z))
    except (TypeError, ValueError):
        return _D3(*_ego3(ego_position).tolist())


def pose_to_transform(translation, rotation_xyzw) -> np.ndarray:
    """float64 4x4 of tf's fromTranslationRotation (translation, quaternion
    x, y, z, w), as the reference's ROS node builds Process_pointcloud's
    transform (scripts/gvom_ros.py:93-105)."""
    t = np.ascontiguousarray(np.asarray(translation, np.float64).reshape(3))
    q = np.ascontiguousarray(np.asarray(rotation_xyzw, np.float64).reshape(4))
    out = np.empty((4, 4), np.float64)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(_lib.load().gvom_pose_to_transform(P(t), P(q), P(out)))
    return out


class Gvom:
    """GB300 implementation of the reference `Gvom` (scripts/gvom.py:8-442)."""

    def __init__(self, xy_resolution, z_resolution, xy_size, z_size, buffer_size, min_distance,
                 positive_obstacle_threshold, negative_obstacle_threshold, slope_obsacle_threshold,
                 robot_height, robot_radius, ground_to_lidar_height, xy_eigen_dist, z_eigen_dist):
        self._l = _lib.load()
        self.params = (xy_resolution, z_resolution, xy_size, z_size, buffer_size, min_distance,
                       positive_obstacle_threshold, negative_obstacle_threshold, slope_obsacle_threshold,
                       robot_height, robot_radius, ground_to_lidar_height, xy_eigen_dist, z_eigen_dist)
        self.xy_resolution = xy_resolution
        self.z_resolution = z_resolution
        self.xy_size = int(xy_size)
        self.z_size = int(z_size)
        self.buffer_size = int(buffer_size)
        self.min_distance = min_distance
        self.positive_obstacle_threshold = positive_obstacle_threshold
        self.negative_obstacle_threshold = negative_obstacle_threshold
        self.slope_obsacle_threshold = slope_obsacle_threshold
        self.robot_height = robot_height
        self.robot_radius = robot_radius
        self.ground_to_lidar_height = ground_to_lidar_height
        self.xy_eigen_dist = int(xy_eigen_dist)
        self.z_eigen_dist = int(z_eigen_dist)
        self.voxel_count = self.xy_size * self.xy_size * self.z_size
        self.metrics_count = 10
        p = GvomParams(float(xy_resolution), float(z_resolution), self.xy_size, self.z_size, self.buffer_size,
                       float(min_distance), float(positive_obstacle_threshold),
                       float(negative_obstacle_threshold), float(slope_obsacle_threshold),
                       float(robot_height), float(robot_radius), float(ground_to_lidar_height),
                       self.xy_eigen_dist, self.z_eigen_dist)
        h = C.c_void_p()
        check(self._l.gvom_create(C.byref(p), C.byref(h)))
        self._h = h
        self._lock = threading.Lock()

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._l.gvom_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------
    # reference API
    # ------------------------------------------------------------------
    def Process_pointcloud(self, pointcloud, ego_position, transform=None):
        """Voxelise one scan into the ring buffer (scripts/gvom.py:105-217)."""
        ptr, code, n, stride, keep, on_dev = _as_points(pointcloud)
        tptr, tcode, tkeep = _as_transform(transform)
        ego = _ego_c(ego_position)
        fn = self._l.gvom_process_device if on_dev else self._l.gvom_process
        check(fn(self._h, ptr, code, n, stride, ego, tptr, tcode))
        if on_dev:
            # the library runs on its own stream; keep the tensor alive until the scan is consumed
            self.synchronize()
        del keep, tkeep

    process_pointcloud = Process_pointcloud

    def _output_maps(self):
        """combine_maps' four maps (int32, int32, float64, int32; (X, X)) as
        views of one fresh host block laid out as the library's device block
        (roughness, positive, negative, visibility), which it then copies in
        one transfer; the origin (3 doubles) follows at an 8-byte boundary.
        Returns (origin, pos, neg, rough, vis, address of the block)."""
        X2 = self.xy_size * self.xy_size
        oo = (20 * X2 + 7) & ~7
        blk = np.empty(oo + 24, np.uint8)
        sh = (self.xy_size, self.xy_size)
        nd = np.ndarray
        return (nd((3,), np.float64, blk, oo), nd(sh, np.int32, blk, 8 * X2), nd(sh, np.int32, blk, 12 * X2),
                nd(sh, np.float64, blk, 0), nd(sh, np.int32, blk, 16 * X2), blk.ctypes.data)

    def combine_maps(self):
        """Merge the ring and build the 2-D maps (scripts/gvom.py:222-393)."""
        origin, pos, neg, rough, vis, b = self._output_maps()
        X2 = self.xy_size * self.xy_size
        rc = self._l.gvom_combine(self._h, b + ((20 * X2 + 7) & ~7), b + 8 * X2, b + 12 * X2, b, b + 16 * X2)
        if rc == GVOM_NO_DATA:
            print("ERROR: No data in buffer")
            return None
        check(rc)
        return origin, pos, neg, rough, vis

    def process_pointcloud2(self, data, n_points, point_step, xyz_offsets, ego_position, translation,
                            rotation_xyzw, field_dtype=np.float32):
        """Map a PointCloud2 payload as the reference's ROS node does
        (scripts/gvom_ros.py:85-109): x / y / z fields (`field_dtype` float32
        or float64, little-endian) at byte offsets `xyz_offsets` of each
        `point_step`-byte point, widened to float64, non-finite points
        dropped, pose from tf translation + quaternion (x, y, z, w).  `data`:
        bytes / uint8 numpy array, or a CUDA uint8 tensor (read in place)."""
        fd = np.dtype(field_dtype)
        if fd not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise ValueError("x / y / z fields must be float32 or float64")
        fdt = GVOM_F32 if fd == np.float32 else GVOM_F64
        offs = (C.c_int32 * 3)(*[int(v) for v in xyz_offsets])
        ego = _ego3(ego_position)
        t = np.ascontiguousarray(np.asarray(translation, np.float64).reshape(3))
        q = np.ascontiguousarray(np.asarray(rotation_xyzw, np.float64).reshape(4))
        P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        if hasattr(data, "data_ptr") and getattr(data, "is_cuda", False):
            check(self._l.gvom_process_pointcloud2(self._h, C.c_void_p(data.data_ptr()), int(n_points), int(point_step),
                                                   offs, fdt, 1, P(ego), P(t), P(q)))
            self.synchronize()
            return
        buf = np.frombuffer(data, np.uint8) if isinstance(data, (bytes, bytearray, memoryview)) else \
            np.ascontiguousarray(data).view(np.uint8).reshape(-1)
        if buf.size < int(n_points) * int(point_step):
            raise ValueError("data is shorter than n_points * point_step")
        check(self._l.gvom_process_pointcloud2(self._h, P(buf), int(n_points), int(point_step), offs, fdt, 0,
                                               P(ego), P(t), P(q)))

    def ros_grids(self, density_threshold=50, min_roughness=-10, max_roughness=0):
        """The ROS node's OccupancyGrid payloads from the last combine_maps
        (scripts/gvom_ros.py:141-164): {'hard', 'soft', 'certainty',
        'negative', 'roughness'} -> int8[xy_size**2] in column-major order, or
        None before the first combine."""
        X2 = self.xy_size * self.xy_size
        names = ("hard", "soft", "certainty", "negative", "roughness")
        out = {k: np.empty(X2, np.int8) for k in names}
        p = _lib.GvomRosParams(float(density_threshold), float(min_roughness), float(max_roughness))
        rc = self._l.gvom_ros_grids(self._h, C.byref(p), *[out[k].ctypes.data_as(C.c_void_p) for k in names], 0)
        if rc == GVOM_NO_DATA:
            return None
        check(rc)
        return out

    def make_debug_voxel_map(self):
        """[x, y, z, hit/total, hit, l0-l1, l1-l2, l2] per occupied voxel (scripts/gvom.py:395-410)."""
        rows = C.c_int64()
        rc = self._l.gvom_debug_voxel_map(self._h, None, 0, C.byref(rows))
        if rc == GVOM_NO_DATA:
            print("No data")
            return None
        check(rc)
        out = np.zeros((rows.value, 8), np.float32)
        if rows.value:
            check(self._l.gvom_debug_voxel_map(self._h, out.ctypes.data_as(C.c_void_p), rows.value, C.byref(rows)))
        return out

    def make_debug_height_map(self):
        """(X*X, 7) float32 height/roughness/slope cloud (scripts/gvom.py:412-426)."""
        out = np.zeros((self.xy_size * self.xy_size, 7), np.float32)
        rc = self._l.gvom_debug_height_map(self._h, out.ctypes.data_as(C.c_void_p))
        if rc == GVOM_NO_DATA:
            print("No data")
            return None
        check(rc)
        return out

    def make_debug_inferred_height_map(self):
        """(X*X, 3) float32 cloud of the guessed height delta (scripts/gvom.py:428-442)."""
        out = np.zeros((self.xy_size * self.xy_size, 3), np.float32)
        rc = self._l.gvom_debug_inferred_height_map(self._h, out.ctypes.data_as(C.c_void_p))
        if rc == GVOM_NO_DATA:
            print("No data")
            return None
        check(rc)
        return out

    # ------------------------------------------------------------------
    # extensions
    # ------------------------------------------------------------------
    def _scan_array(self, scans):
        arr = (GvomScan * len(scans))()
        keep = []
        on_dev = None
        for i, (pc, ego, T) in enumerate(scans):
            ptr, code, n, stride, k, dev = _as_points(pc)
            if on_dev is None:
                on_dev = dev
            elif on_dev != dev:
                raise ValueError("all scans of a batch must be on the same side (host or device)")
            tptr, tcode, tk = _as_transform(T)
            keep += [k, tk]
            e = _ego3(ego)
            sc = arr[i]
            sc.points = ptr
            sc.dtype = code
            sc.transform_dtype = tcode
            sc.n = n
            sc.row_stride = stride
            sc.ego[:] = e.tolist()
            sc.transform = tptr
        return arr, keep, bool(on_dev)

    def process_batch(self, scans):
        """Process several scans [(pointcloud, ego, transform), ...] in one set of launches;
        equivalent to calling Process_pointcloud on each in order."""
        arr, keep, on_dev = self._scan_array(scans)
        check(self._l.gvom_process_batch(self._h, arr, len(scans), 1 if on_dev else 0))
        if on_dev:
            self.synchronize()
        del keep

    def step(self, scans, device_outputs=None):
        """process_batch(scans) then combine_maps() in one call (the index merge
        overlaps the statistics kernels; one graph in graph mode).  Returns
        combine_maps()'s tuple, or with `device_outputs` = (pos, neg, rough,
        vis) CUDA tensors fills them stream-ordered and returns the origin."""
        arr, keep, on_dev = self._scan_array(scans)
        if device_outputs is not None:
            origin = np.zeros(3, np.float64)
            ptrs = [C.c_void_p(t.data_ptr()) for t in device_outputs]
            check(self._l.gvom_step(self._h, arr, len(scans), 1 if on_dev else 0, origin.ctypes.data, *ptrs, 1))
            del keep
            return origin
        origin, pos, neg, rough, vis, b = self._output_maps()
        X2 = self.xy_size * self.xy_size
        check(self._l.gvom_step(self._h, arr, len(scans), 1 if on_dev else 0, b + ((20 * X2 + 7) & ~7), b + 8 * X2,
                                b + 12 * X2, b, b + 16 * X2, 0))
        del keep
        return origin, pos, neg, rough, vis

    def combine_maps_device(self, pos, neg, rough, vis):
        """combine_maps into preallocated CUDA tensors (int32, int32, float64, int32; (X, X)),
        stream-ordered on the mapper's stream; returns the origin or None."""
        origin = np.zeros(3, np.float64)
        rc = self._l.gvom_combine_device(self._h, origin.ctypes.data_as(C.c_void_p), C.c_void_p(pos.data_ptr()),
                                         C.c_void_p(neg.data_ptr()), C.c_void_p(rough.data_ptr()),
                                         C.c_void_p(vis.data_ptr()))
        if rc == GVOM_NO_DATA:
            return None
        check(rc)
        return origin

    def synchronize(self):
        check(self._l.gvom_synchronize(self._h))

    def set_stream(self, stream_ptr: int | None):
        check(self._l.gvom_set_stream(self._h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def set_tuning(self, tuning: dict):
        """Launch shapes (keys of GvomTuning); speed only, never results."""
        cur = self.get_tuning()
        cur.update(tuning)
        t = _lib.GvomTuning(**{k: int(v) for k, v in cur.items()})
        check(self._l.gvom_set_tuning(self._h, C.byref(t)))

    def get_tuning(self) -> dict:
        t = _lib.GvomTuning()
        check(self._l.gvom_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def set_graphs(self, on: bool):
        """Capture each process / combine launch sequence into a CUDA graph and
        replay it (updated in place while its shape holds)."""
        check(self._l.gvom_set_graphs(self._h, 1 if on else 0))

    def set_stage_timing(self, on: bool):
        """Record CUDA events around every kernel launch (resets the totals)."""
        check(self._l.gvom_set_stage_timing(self._h, 1 if on else 0))

    def stage_times(self):
        """{kernel name: (total ms, launches)} since stage timing was enabled."""
        n = _lib.GVOM_STAGES
        ms = (C.c_double * n)()
        cnt = (C.c_int64 * n)()
        check(self._l.gvom_stage_times(self._h, ms, cnt, n))
        return {self._l.gvom_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(n)}

    def device_bytes(self) -> int:
        b = C.c_int64()
        check(self._l.gvom_device_bytes(self._h, C.byref(b)))
        return b.value

    def reserve(self, max_scans: int, max_points: int, max_row_bytes: int = 12):
        """Allocate now what calls of up to `max_scans` scans and `max_points`
        points in all would allocate on first use (gvom_reserve), so that a
        request loop's latency never includes an allocation."""
        check(self._l.gvom_reserve(self._h, int(max_scans), int(max_points), int(max_row_bytes)))

    # ------------------------------------------------------------------
    # state access (parity checks)
    # ------------------------------------------------------------------
    def ring_state(self):
        a, b = C.c_int64(), C.c_int64()
        check(self._l.gvom_ring_state(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_process_stats(self):
        v, h, s = C.c_int64(), C.c_int64(), C.c_int64()
        check(self._l.gvom_last_process_stats(self._h, C.byref(v), C.byref(h), C.byref(s)))
        return dict(valid_points=v.value, hits=h.value, ray_steps=s.value)

    def slot_state(self, slot: int):
        n = C.c_int64()
        check(self._l.gvom_slot_count(self._h, int(slot), C.byref(n)))
        if n.value < 0:
            return None
        c = n.value
        st = dict(index=np.empty(self.voxel_count, np.int32), hit=np.empty(c, np.int32),
                  total=np.empty(c, np.int32), min_h=np.empty(c, np.float32),
                  metrics=np.empty((c, 10), np.float32), origin=np.zeros(3))
        P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        check(self._l.gvom_get_slot(self._h, int(slot), P(st["index"]), P(st["hit"]), P(st["total"]),
                                    P(st["min_h"]), P(st["metrics"]), P(st["origin"])))
        return st

    def combined_state(self):
        n = C.c_int64()
        check(self._l.gvom_combined_count(self._h, C.byref(n)))
        if n.value < 0:
            return None
        c = n.value
        st = dict(index=np.empty(self.voxel_count, np.int32), hit=np.empty(c, np.int32),
                  total=np.empty(c, np.int32), min_h=np.empty(c, np.float32),
                  metrics=np.empty((c, 10), np.float32), eigen=np.empty((c, 3), np.float32),
                  origin=np.zeros(3))
        P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        check(self._l.gvom_get_combined(self._h, P(st["index"]), P(st["hit"]), P(st["total"]), P(st["min_h"]),
                                        P(st["metrics"]), P(st["eigen"]), P(st["origin"])))
        return st

    def maps_state(self):
        X = self.xy_size
        keys = ("height", "inferred", "slope_x", "slope_y", "roughness", "guess")
        st = {k: np.empty((X, X), np.float64) for k in keys}
        rc = self._l.gvom_get_maps(self._h, *[st[k].ctypes.data_as(C.c_void_p) for k in keys])
        if rc == GVOM_NO_DATA:
            return None
        check(rc)
        return st
