"""The ROS node's OccupancyGrid payloads (scripts/gvom_ros.py:141-164):
oracle restatement pinned to numpy's own int8 cast on x86; device payloads
(gvom_ros_grids) equal to the oracle's, byte for byte, computed from the
same combine outputs."""
import platform

import numpy as np
import pytest

from oracle.ros_grids import int8_wrap, ros_grids


@pytest.mark.skipif(platform.machine() not in ("x86_64", "AMD64"), reason="numpy's float->int8 cast rule is x86's")
def test_restatement_matches_numpy_astype_on_x86():
    import warnings
    rng = np.random.default_rng(5)
    v = np.concatenate([rng.uniform(-300, 300, 20000), np.arange(-260, 260, 0.25), [-1e10, 1e10, 0.0, -0.0]])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = v.astype(np.int8)
    np.testing.assert_array_equal(int8_wrap(v), ref)
    X = 64
    pos = rng.integers(0, 120, (X, X)).astype(np.int32)
    neg = np.where(rng.uniform(size=(X, X)) < 0.1, 100, 0).astype(np.int32)
    vis = (rng.uniform(size=(X, X)) < 0.7).astype(np.int32)
    rough = np.where(rng.uniform(size=(X, X)) < 0.2, -1.0, rng.uniform(-25, 3, (X, X)))
    got = ros_grids(pos, neg, rough, vis)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        F = lambda a: np.reshape(a, -1, order="F")  # noqa: E731
        want = {"hard": F(np.maximum(100 * (pos > 50), neg)).astype(np.int8),
                "soft": F(100 * (pos <= 50) * (pos > 0)).astype(np.int8),
                "certainty": F(vis * 100).astype(np.int8),
                "negative": F(neg).astype(np.int8),
                "roughness": F(((np.maximum(np.minimum(rough, 0), -10) + -10) / (0 - -10)) * 100).astype(np.int8)}
    for k in want:
        np.testing.assert_array_equal(got[k], want[k], k)


PAYLOAD_OF = {"h_obstacle_map_pub": "hard", "s_obstacle_map_pub": "soft", "g_certainty_pub": "certainty",
              "a_certainty_pub": "certainty", "n_obstacle_map_pub": "negative", "r_map_pub": "roughness"}


def test_restatement_matches_the_reference_callback():
    """Pinned to the reference node itself: tests/golden/ros_epilogue.npz holds what
    VoxelMapper.cb_timer (scripts/gvom_ros.py:113-166), run unchanged on x86 by
    tests/golden/make_ros_golden.py, published for stored combine outputs and edge
    cases (clip bounds, payloads outside int8, NaN, other node parameters)."""
    import os
    from conftest import GOLDEN
    with np.load(os.path.join(GOLDEN, "ros_epilogue.npz")) as z:
        fx = {k: z[k] for k in z.files}
    names = str(fx["cases"]).split(",")
    assert len(names) >= 6
    for n in names:
        thr, lo, hi = fx[f"{n}_params"]
        got = ros_grids(fx[f"{n}_pos"], fx[f"{n}_neg"], fx[f"{n}_rough"], fx[f"{n}_vis"],
                        density_threshold=thr, min_roughness=lo, max_roughness=hi)
        for pub, key in PAYLOAD_OF.items():
            np.testing.assert_array_equal(got[key], fx[f"{n}_{pub}"], f"{n} {pub}")


@pytest.mark.gpu
def test_device_payloads_equal_oracle(gpu_lib):
    from gvom_gb300 import Gvom
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 3)
    g = Gvom(*w.gvom_args())
    assert g.ros_grids() is None
    for s in scans:
        g.Process_pointcloud(s.points, s.ego, s.transform)
        out = g.combine_maps()  # (combine outputs are checked against the oracle elsewhere)
        for kw in ({}, {"density_threshold": 10, "min_roughness": -20, "max_roughness": 5}):
            got = g.ros_grids(**kw)
            want = ros_grids(out[1], out[2], out[3], out[4], **kw)
            for k in want:
                np.testing.assert_array_equal(got[k], want[k], k)
