"""Lidar-message ingestion (scripts/gvom_ros.py:85-109): PointCloud2 bytes and
a tf translation + quaternion pose, mapped by gvom_process_pointcloud2.

CPU: the oracle's restatement of tf's quaternion_matrix against tf's own
documented example and scipy; the library's pose -> 4x4 against the oracle,
bit for bit; the PointCloud2 reader on a hand-packed message.
GPU: a message mapped from bytes (host or device, float32 or float64 fields,
non-finite rows, noise in the other fields) gives bit-identical maps to
Process_pointcloud on the oracle-decoded float64 points with the same pose,
and those match the oracle mapper."""
import ctypes
import math
import struct

import numpy as np
import pytest

from oracle.ros_ingest import from_translation_rotation, make_pointcloud2, pointcloud2_to_xyz, quaternion_matrix


def _rotation_x(angle):
    c, s = math.cos(angle), math.sin(angle)
    R = np.identity(4)
    R[1:3, 1:3] = [[c, -s], [s, c]]
    return R


def test_quaternion_matrix_known_answers():
    # tf.transformations' own docstring example: a rotation of 0.123 rad about x
    np.testing.assert_allclose(quaternion_matrix([0.06146124, 0, 0, 0.99810947]), _rotation_x(0.123), atol=1e-7)
    np.testing.assert_array_equal(quaternion_matrix([0, 0, 0, 1]), np.identity(4))
    np.testing.assert_array_equal(quaternion_matrix([1e-9, 0, 0, 0]), np.identity(4))  # below 4 eps: identity
    # 180 degrees about z
    np.testing.assert_allclose(quaternion_matrix([0, 0, 1, 0]), np.diag([-1.0, -1.0, 1.0, 1.0]), atol=1e-15)
    T = from_translation_rotation([1.5, -2.0, 0.25], [0, 0, 0, 1])
    np.testing.assert_array_equal(T[:3, 3], [1.5, -2.0, 0.25])


def test_quaternion_matrix_matches_scipy():
    Rotation = pytest.importorskip("scipy.spatial.transform").Rotation
    rng = np.random.default_rng(11)
    for _ in range(2000):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        np.testing.assert_allclose(quaternion_matrix(q)[:3, :3], Rotation.from_quat(q).as_matrix(), atol=2e-15)


def test_library_pose_matches_oracle_bit_for_bit(gpu_lib):
    from gvom_gb300 import pose_to_transform
    rng = np.random.default_rng(12)
    cases = [([0, 0, 0], [0, 0, 0, 1]), ([1, 2, 3], [0, 0, 0, 0]), ([0, 0, 0], [1e-9, 0, 0, 0]),
             ([-4.5, 1e4, 0.3], [0, 0, 1, 0]), ([0, 0, 0], [0.06146124, 0, 0, 0.99810947])]
    for i in range(20000):
        q = rng.normal(size=4)
        if i % 3:
            q /= np.linalg.norm(q)  # tf lookups are unit quaternions up to rounding
        cases.append((rng.uniform(-1e3, 1e3, 3), q))
    for t, q in cases:
        want = from_translation_rotation(t, q)
        got = pose_to_transform(t, q)
        assert got.tobytes() == want.tobytes() or np.array_equal(got, want), (t, q, got - want)


def test_pose_entry_point_rejects_null(gpu_lib):
    from gvom_gb300._lib import GVOM_ERR_ARG
    out = (ctypes.c_double * 16)()
    assert gpu_lib.gvom_pose_to_transform(None, None, out) == GVOM_ERR_ARG
    assert gpu_lib.gvom_process_pointcloud2(None, None, 0, 16, None, 0, 0, None, None, None) == GVOM_ERR_ARG


def test_pointcloud2_reader_hand_packed():
    # point_step 20: x, y, z float32 at 0, 4, 8; intensity float32 at 12; ring uint16 at 16; 2 pad bytes
    rows = [(1.0, 2.0, 3.0, 9.0, 7), (float("nan"), 0.0, 0.0, 1.0, 1), (-0.5, 1e6, 2.5, 3.0, 2),
            (0.0, float("inf"), 1.0, 0.0, 3), (4.0, 5.0, -6.0, 0.0, 4)]
    data = b"".join(struct.pack("<ffffHxx", *r) for r in rows)
    got = pointcloud2_to_xyz(data, len(rows), 20, (0, 4, 8))
    np.testing.assert_array_equal(got, [[1, 2, 3], [-0.5, 1e6, 2.5], [4, 5, -6]])
    assert got.dtype == np.float64
    # fields in another order (z first), float64
    data = b"".join(struct.pack("<dxxxxxxxxdd", z, x, y) for x, y, z in [(1, 2, 3), (4, 5, 6)])
    got = pointcloud2_to_xyz(data, 2, 32, (16, 24, 0), np.float64)
    np.testing.assert_array_equal(got, [[1, 2, 3], [4, 5, 6]])


def _pose_of(T):
    """(translation, quaternion x, y, z, w) of a rigid 4x4, as a tf lookup gives."""
    Rotation = pytest.importorskip("scipy.spatial.transform").Rotation
    R = np.asarray(T, np.float64)[:3, :3]
    u, _, vt = np.linalg.svd(R)
    return np.asarray(T, np.float64)[:3, 3].copy(), Rotation.from_matrix(u @ vt).as_quat()


def _with_nonfinite(points, rng, frac=0.02):
    p = np.array(points, np.float64)
    idx = rng.choice(p.shape[0], max(1, int(frac * p.shape[0])), replace=False)
    col = rng.integers(0, 3, idx.size)
    p[idx, col] = rng.choice([np.nan, np.inf, -np.inf], idx.size)
    return p


def _same_maps(a, b, what):
    assert (a is None) == (b is None), what
    for x, y, name in zip(a, b, ("origin", "pos", "neg", "rough", "vis")):
        np.testing.assert_array_equal(np.asarray(x), np.asarray(y), f"{what}: {name}")


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [
    dict(point_step=16, offs=(0, 4, 8), ftype=np.float32, device=False),
    dict(point_step=48, offs=(8, 0, 20), ftype=np.float32, device=True),
    dict(point_step=40, offs=(8, 16, 24), ftype=np.float64, device=False),
    dict(point_step=32, offs=(0, 8, 16), ftype=np.float64, device=True),
])
def test_pointcloud2_equals_process_pointcloud(gpu_lib, layout):
    import torch
    from gvom_gb300 import Gvom, pose_to_transform
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    from oracle.canonical import canonical_state
    from oracle.oracle import OracleGvom
    from replay import compare_combine, compare_slot
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 3)
    rng = np.random.default_rng(13)
    params = w.gvom_args()
    g_msg, g_arr, o = Gvom(*params), Gvom(*params), OracleGvom(*params)
    for i, s in enumerate(scans):
        t, q = _pose_of(s.transform)
        pts = _with_nonfinite(s.points, rng)
        data = make_pointcloud2(pts, layout["point_step"], layout["offs"], layout["ftype"], extra_seed=i)
        n = pts.shape[0]
        if layout["device"]:
            dev = torch.frombuffer(bytearray(data), dtype=torch.uint8).cuda()
            g_msg.process_pointcloud2(dev, n, layout["point_step"], layout["offs"], s.ego, t, q, layout["ftype"])
        else:
            g_msg.process_pointcloud2(data, n, layout["point_step"], layout["offs"], s.ego, t, q, layout["ftype"])
        xyz = pointcloud2_to_xyz(data, n, layout["point_step"], layout["offs"], layout["ftype"])
        T = pose_to_transform(t, q)
        np.testing.assert_array_equal(T, from_translation_rotation(t, q))
        g_arr.Process_pointcloud(xyz, s.ego, T)
        o.Process_pointcloud(xyz, s.ego, T)
        _, last = g_msg.ring_state()
        assert g_msg.ring_state() == g_arr.ring_state() == o.ring_state()
        compare_slot(canonical_state(g_msg.slot_state(last)), canonical_state(o.slot_state(last)), f"scan {i}")
        out_msg, out_arr = g_msg.combine_maps(), g_arr.combine_maps()
        _same_maps(out_msg, out_arr, f"scan {i}")
        ref = o.combine_maps()
        refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
        compare_combine(out_msg, refd, g_msg.maps_state(), params, f"combine after scan {i}")
    for g in (g_msg, g_arr):
        g.close()


@pytest.mark.gpu
def test_pointcloud2_argument_checks(gpu_lib):
    from gvom_gb300 import Gvom
    from gvom_gb300._lib import GvomError
    from gvom_gb300.synthetic import WORKLOADS
    g = Gvom(*WORKLOADS["small_32x512"].gvom_args())
    data = make_pointcloud2(np.zeros((4, 3)), 16, (0, 4, 8))
    for step, offs, ft in [(16, (0, 4, 14), np.float32), (16, (0, 4, 16), np.float32), (18, (0, 4, 8), np.float32),
                           (24, (0, 4, 8), np.float64), (0, (0, 4, 8), np.float32)]:
        with pytest.raises((GvomError, ValueError)):
            g.process_pointcloud2(data, 1 if step == 0 else len(data) // step, step, offs, (0, 0, 0),
                                  (0, 0, 0), (0, 0, 0, 1), ft)
    with pytest.raises(ValueError):
        g.process_pointcloud2(data, 4, 16, (0, 4, 8), (0, 0, 0), (0, 0, 0), (0, 0, 0, 1), np.int32)
    assert g.combine_maps() is None  # nothing was enqueued; the instance still answers
    g.close()
