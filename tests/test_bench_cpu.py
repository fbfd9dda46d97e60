"""bench.py's host-side accounting on CPU: the clock summary, the whole-step roofline follows
the per-unit work of the scan->map accounting, and an auxiliary figure that
fails never breaks the bench line."""
import bench


def test_step_roofline_per_unit_work():
    V, X2, B = 4194304, 65536, 4
    r = bench.step_roofline(n_pts=1000, ns=1, V=V, X2=X2, B=B, C_new=10, C_sum=40, Cc=30, hits=7, steps=500,
                            peak_gbs=1000.0, ms_per_step=1.0)
    process = 12 * 1000 + 64 + 4 * V + 52 * 10
    combine = 4 * V * (B + 1) + 4 * V + 52 * 40 + 2 * 52 * 30 + 20 * X2
    assert r["bytes_per_step"] == process + combine
    assert r["atomics_per_step"] == 2 * 7 + 500
    assert abs(r["hbm_bound_ms"] - (process + combine) / 1e12 * 1e3) < 1e-12
    assert abs(r["frac_of_measured_hbm"] - r["hbm_bound_ms"] / 1.0) < 1e-12
    # the combine's index maps: (B + 2) x 4V, 101 MB at 256 x 256 x 64 with B = 4
    assert abs(4 * V * (B + 2) / 1e6 - 100.7) < 0.1


def test_safe_returns_none_on_failure():
    assert bench._safe(lambda: 1 / 0) is None
    assert bench._safe(lambda: 3) == 3


def test_clock_summary_reads_nvidia_smi_rows():
    rows = ["0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
            "0, 1980, 2070, 1390.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
            "0, 2070, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
            "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",  # unreadable: skipped
            "short row"]
    s = bench.summarize_clocks(rows)
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3, "reasons": ["sw_power_cap"]}
    hot = bench.summarize_clocks(["0, 1500, 2070, 1400, 0x48, Active, Active, Not Active, Not Active"])
    assert hot["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]
    assert bench.summarize_clocks([]) is None


def test_trace_atomic_roofline():
    r = bench.trace_atomic_roofline(hits=95000, steps=6_800_000, ms_per_launch=0.0614)
    assert r["atomics_per_launch"] == 2 * 95000 + 6_800_000
    assert abs(r["achieved_per_s"] - 6_990_000 / 61.4e-6) < 1.0
    assert abs(r["frac"] - r["achieved_per_s"] / bench.RED32_SCATTERED_PER_S) < 1e-12
    assert 0.5 < r["frac"] < 0.6


def test_quaternion_round_trip_and_node_host_work(gpu_lib):
    """bench.py's message builder: the quaternion of a rotation (all four
    branches of Shepperd's method) gives back the rotation through the
    library's tf-style 4x4; the node's host conversions of a message keep the
    finite x, y, z rows as float64 and give five int8 payloads."""
    import numpy as np
    from gvom_gb300 import pose_to_transform
    from scipy.spatial.transform import Rotation
    rng = np.random.default_rng(2)
    Rs = [np.eye(3), np.diag([1.0, -1.0, -1.0]), np.diag([-1.0, 1.0, -1.0]), np.diag([-1.0, -1.0, 1.0])]
    Rs += list(Rotation.random(200, random_state=3).as_matrix())
    for R in Rs:
        q = bench._quat_xyzw(R)
        assert abs(np.linalg.norm(q) - 1.0) < 1e-12
        T = pose_to_transform(np.array([1.0, 2.0, 3.0]), q)
        np.testing.assert_allclose(T[:3, :3], R, atol=1e-12)
    pts = rng.standard_normal((100, 3)).astype(np.float32)
    pts[7, 1] = np.nan
    rows = bench.lidar_message(pts, rng)
    assert rows.shape == (100, 12) and rows.dtype == np.float32
    np.testing.assert_array_equal(rows[:, :3], pts)
    X = 8
    maps = (np.zeros(3), rng.integers(0, 101, (X, X)).astype(np.int32), np.zeros((X, X), np.int32),
            rng.uniform(-12, 1, (X, X)), np.ones((X, X), np.int32))
    xyz, pay = bench.node_host_work(rows, maps)
    assert xyz.shape == (99, 3) and xyz.dtype == np.float64
    assert len(pay) == 5 and all(p.dtype == np.int8 and p.shape == (X * X,) for p in pay)


def test_measure_ros_runs_against_a_stand_in_mapper(monkeypatch):
    """Every line of the ros form on CPU: a stand-in mapper records the
    calls; the form's numbers come out for the given steps."""
    import types

    import numpy as np

    import gvom_gb300
    calls = []

    class FakeGvom:
        def __init__(self, *params):
            self.X = params[2]

        def process_pointcloud2(self, data, n, step, offs, ego, t, q):
            assert np.asarray(data).nbytes >= n * step and tuple(offs) == (0, 4, 8) and len(q) == 4
            calls.append("pc2")

        def combine_maps(self):
            X = self.X
            return (np.zeros(3), np.zeros((X, X), np.int32), np.zeros((X, X), np.int32), np.full((X, X), -1.0),
                    np.ones((X, X), np.int32))

        def ros_grids(self):
            calls.append("grids")

        def make_debug_voxel_map(self):
            calls.append("dbg")

        make_debug_height_map = make_debug_inferred_height_map = make_debug_voxel_map

        def close(self):
            pass

    monkeypatch.setattr(gvom_gb300, "Gvom", FakeGvom)
    torch = types.SimpleNamespace(cuda=types.SimpleNamespace(synchronize=lambda: None))
    rng = np.random.default_rng(0)
    scan = lambda: types.SimpleNamespace(points=rng.standard_normal((50, 3)).astype(np.float32),  # noqa: E731
                                          ego=(0.0, 0.0, 1.0), transform=np.eye(4, dtype=np.float32))
    form = types.SimpleNamespace(name="tiny", steps=[[scan()] for _ in range(3)],
                                 w=types.SimpleNamespace(gvom_args=lambda: (0.2, 0.2, 16, 8, 2, 1.0, 0.5, 0.5, 0.3,
                                                                            2.0, 4.0, 1.0, 1, 1)))
    r = bench.measure_ros(form, torch, n_steps=20, warmup=2)
    assert calls.count("pc2") == 22 and calls.count("grids") == 22 and calls.count("dbg") == 3 * 2
    assert r["steps"] == 20 and r["points_per_s"] > 0 and r["node_host_conversions_us_p50"] > 0
    assert set(r["us_p50"]) == {"process_pointcloud2", "combine_maps", "ros_grids", "debug_exports_all_three"}
