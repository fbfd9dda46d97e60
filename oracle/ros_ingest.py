"""TEST INFRASTRUCTURE - CPU restatement of how the reference's ROS node turns
a lidar message into Process_pointcloud's arguments (scripts/gvom_ros.py:
85-109), the checker for gvom_process_pointcloud2 / gvom_pose_to_transform.

Both steps live in third-party ROS packages that are not part of the
reference tree; their published algorithms are restated here:

- ros_numpy 0.0.5 (eric-wieser/ros_numpy), point_cloud2.pointcloud2_to_xyz_array
  with its default remove_nans=True: the cloud's x / y / z fields read with
  their declared type, rows with a non-finite coordinate removed, the rest
  copied into a float64 (N, 3) array in message order;
- ROS tf 1.13 (tf/listener.py TransformerROS.fromTranslationRotation over
  tf/transformations.py): numpy.dot(translation_matrix(t), quaternion_matrix(q))
  with the quaternion in (x, y, z, w) order.
"""
from __future__ import annotations

import math

import numpy as np

_EPS = np.finfo(float).eps * 4.0


def pointcloud2_to_xyz(data, n_points: int, point_step: int, xyz_offsets, field_dtype=np.float32) -> np.ndarray:
    """float64 (M, 3) points of a little-endian PointCloud2 payload."""
    buf = np.frombuffer(bytes(data) if not isinstance(data, np.ndarray) else data.tobytes(), np.uint8)
    rec = np.dtype({"names": ["x", "y", "z"], "formats": [np.dtype(field_dtype).newbyteorder("<")] * 3,
                    "offsets": [int(o) for o in xyz_offsets], "itemsize": int(point_step)})
    arr = np.frombuffer(buf[:int(n_points) * int(point_step)].tobytes(), rec, count=int(n_points))
    mask = np.isfinite(arr["x"]) & np.isfinite(arr["y"]) & np.isfinite(arr["z"])
    arr = arr[mask]
    out = np.zeros((arr.shape[0], 3), np.float64)
    out[:, 0] = arr["x"]
    out[:, 1] = arr["y"]
    out[:, 2] = arr["z"]
    return out


def quaternion_matrix(q) -> np.ndarray:
    """tf.transformations.quaternion_matrix: 4x4 rotation of (x, y, z, w)."""
    q = np.array(q[:4], dtype=np.float64, copy=True)
    nq = np.dot(q, q)
    if nq < _EPS:
        return np.identity(4)
    q *= math.sqrt(2.0 / nq)
    q = np.outer(q, q)
    return np.array((
        (1.0 - q[1, 1] - q[2, 2], q[0, 1] - q[2, 3], q[0, 2] + q[1, 3], 0.0),
        (q[0, 1] + q[2, 3], 1.0 - q[0, 0] - q[2, 2], q[1, 2] - q[0, 3], 0.0),
        (q[0, 2] - q[1, 3], q[1, 2] + q[0, 3], 1.0 - q[0, 0] - q[1, 1], 0.0),
        (0.0, 0.0, 0.0, 1.0)), dtype=np.float64)


def translation_matrix(t) -> np.ndarray:
    M = np.identity(4)
    M[:3, 3] = np.asarray(t, np.float64)[:3]
    return M


def from_translation_rotation(t, q) -> np.ndarray:
    """tf's TransformerROS.fromTranslationRotation."""
    return np.dot(translation_matrix(t), quaternion_matrix(q))


def make_pointcloud2(points_xyz: np.ndarray, point_step: int = 16, xyz_offsets=(0, 4, 8), field_dtype=np.float32,
                     extra_seed: int = 0) -> bytes:
    """A PointCloud2 payload carrying `points_xyz` in its x / y / z fields;
    the other bytes of each point (intensity, ring, padding) are filled with
    seeded noise so that a reader of the wrong bytes is caught."""
    n = points_xyz.shape[0]
    rng = np.random.default_rng(extra_seed)
    buf = rng.integers(0, 256, n * point_step, dtype=np.uint8)
    rec = np.dtype({"names": ["x", "y", "z"], "formats": [np.dtype(field_dtype).newbyteorder("<")] * 3,
                    "offsets": [int(o) for o in xyz_offsets], "itemsize": int(point_step)})
    arr = np.frombuffer(buf.tobytes(), rec, count=n).copy()
    arr["x"] = points_xyz[:, 0]
    arr["y"] = points_xyz[:, 1]
    arr["z"] = points_xyz[:, 2]
    return arr.tobytes()
