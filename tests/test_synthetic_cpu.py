"""The seeded scene generator behind every benchmark and parity scan
(gvom_gb300/synthetic.py): deterministic, fixed point count, the lidar model's
ranges and angles, a rigid sensor->world transform whose translation is the
ego position, whole-beam dropout and the trajectory's step and yaw limits."""
import math

import numpy as np

from gvom_gb300.synthetic import (Lidar, Terrain, Vegetation, WORKLOADS, make_scan, make_trajectory)


def _scene(**kw):
    t = Terrain.make(0, extent=12.0, path_len=2.0)
    lid = Lidar(beams=16, columns=128)
    pose = make_trajectory(3)[2]
    return t, lid, pose, make_scan(t, lid, pose, 2, **kw)


def test_seeded_and_deterministic():
    _, _, _, a = _scene()
    _, _, _, b = _scene()
    np.testing.assert_array_equal(a.points, b.points)
    np.testing.assert_array_equal(a.transform, b.transform)
    assert a.ego == b.ego


def test_lidar_model_ranges_and_angles():
    t, lid, pose, s = _scene()
    assert s.points.shape == (lid.beams * lid.columns, 3) and s.points.dtype == np.float32
    assert s.n_lidar == lid.n_points and s.n_veg == 0
    r = np.linalg.norm(s.points.astype(np.float64), axis=1)
    assert r.min() >= 0.05                                   # no zero-range point
    assert r.max() <= lid.max_range + 6 * lid.noise_sigma    # misses are emitted at 60 m
    el = np.degrees(np.arcsin(s.points[:, 2] / r))
    assert el.min() >= -22.5 - 1e-3 and el.max() <= 22.5 + 1e-3
    # returns lie on the surface: most on the heightfield within the range
    # noise, the rest on the vertical walls of boxes and ditches, where the
    # heightfield at the return's (x, y) is the top or the floor
    T = s.transform.astype(np.float64)
    w = s.points.astype(np.float64) @ T[:3, :3].T + T[:3, 3]
    hit = r < lid.max_range - 1.0
    import torch
    g = t.height(torch.from_numpy(w[hit, 0]), torch.from_numpy(w[hit, 1])).numpy()
    d = np.abs(w[hit, 2] - g)
    assert np.median(d) < 0.05 and (d < 0.1).mean() > 0.7


def test_transform_is_rigid_and_carries_the_ego():
    _, lid, pose, s = _scene(transform_dtype=np.float64)
    T = s.transform
    assert T.dtype == np.float64
    R = T[:3, :3]
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
    assert abs(np.linalg.det(R) - 1.0) < 1e-12
    np.testing.assert_allclose(T[:3, 3], s.ego, atol=0)
    np.testing.assert_array_equal(T[3], [0, 0, 0, 1])
    assert s.ego[2] > 0.5  # mounted above the ground


def test_whole_beam_dropout():
    _, lid, _, s = _scene(dropout=0.5)
    assert s.points.shape[0] % lid.columns == 0 and 0 < s.points.shape[0] < lid.n_points


def test_trajectory_step_and_yaw():
    p = make_trajectory(30)
    for a, b in zip(p, p[1:]):
        assert abs(math.hypot(b.x - a.x, b.y - a.y) - 0.4) < 1e-12
        assert abs(b.yaw - a.yaw) <= math.radians(3.0) + 1e-12


def test_vegetation_is_appended_inside_the_footprint():
    t = Terrain.make(0, extent=12.0, path_len=2.0)
    veg = Vegetation.make(t, (-10, 10), (-10, 10), density=2.0)
    lid = Lidar(beams=8, columns=64)
    s = make_scan(t, lid, make_trajectory(1)[0], 0, vegetation=veg, footprint=8.0)
    assert s.n_veg > 0 and s.points.shape[0] == lid.n_points + s.n_veg


def test_headline_workload_shape():
    w = WORKLOADS["os1_64_veg"]
    args = w.gvom_args()
    assert args[:5] == (0.15, 0.15, 256, 64, 4)
    assert (w.beams, w.columns) == (64, 1024)
