"""GPU parity: libgvom_gb300.so (through the C ABI) against the golden fixtures
and the CPU oracle.

Integer outputs (occupied set in canonical voxel order, hit / pass-through
counts, compact-record hit/total, min height bits, obstacle and visibility
maps) must be bit-exact; float maps within 1e-4 m (heights) or 1e-3 relative
(roughness, slope); statistics within replay.STAT_ATOL.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.canonical import canonical_state
from oracle.oracle import OracleGvom
from replay import compare_combine, compare_slot, load, params_of, replay_and_compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Gvom(gpu_lib):
    from gvom_gb300 import Gvom as G
    return G


@pytest.mark.parametrize("name", golden_files())
def test_golden_replay(Gvom, name):
    fx = load(os.path.join(GOLDEN, name))
    g = Gvom(*params_of(fx))
    replay_and_compare(g, fx)


def _run_both(Gvom, params, scans, combine_every=1):
    g = Gvom(*params)
    o = OracleGvom(*params)
    for i, s in enumerate(scans):
        g.Process_pointcloud(s.points, s.ego, s.transform)
        o.Process_pointcloud(s.points, s.ego, s.transform)
        _, last = g.ring_state()
        assert g.ring_state() == o.ring_state()
        compare_slot(canonical_state(g.slot_state(last)), canonical_state(o.slot_state(last)), f"scan {i}")
        gs, os_ = g.last_process_stats(), o.last_process_stats()
        assert gs == os_, (gs, os_)
        if (i + 1) % combine_every == 0:
            out = g.combine_maps()
            ref = o.combine_maps()
            refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
            compare_combine(out, refd, g.maps_state(), params, f"combine after scan {i}")
            compare_slot(canonical_state(g.combined_state()), canonical_state(o.combined_state()), "combined")
    return g, o


def test_small_32x512_vs_oracle(Gvom):
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 3)
    _run_both(Gvom, w.gvom_args(), scans)


def test_os1_64_vegetation_trajectory_vs_oracle(Gvom):
    """256x256x64 @ 0.15 m, buffer 4, OS1-64 + vegetation, f32 transforms, 6 scans."""
    import torch
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["os1_64_veg"]
    scans = make_workload_scans(w, 6, device="cuda" if torch.cuda.is_available() else "cpu")
    _run_both(Gvom, w.gvom_args(), scans, combine_every=2)


def test_float64_ros_style_inputs(Gvom):
    """float64 transform (ROS tf) and float64 points; strided (N,4) rows."""
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    t = Terrain.make(0, extent=19.2, path_len=2.0)
    lid = Lidar(beams=32, columns=256)
    params = (0.15, 0.15, 128, 32, 3, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    g = Gvom(*params)
    o = OracleGvom(*params)
    for i, p in enumerate(make_trajectory(4)):
        s = make_scan(t, lid, p, i, transform_dtype=np.float64)
        pts = s.points.astype(np.float64) if i % 2 else s.points
        xyzi = np.concatenate([pts, np.ones((pts.shape[0], 1), pts.dtype)], 1)
        g.Process_pointcloud(xyzi, s.ego, s.transform)
        o.Process_pointcloud(xyzi, s.ego, s.transform)
        _, last = g.ring_state()
        compare_slot(canonical_state(g.slot_state(last)), canonical_state(o.slot_state(last)), f"scan {i}")
    out, ref = g.combine_maps(), o.combine_maps()
    refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
    compare_combine(out, refd, g.maps_state(), params, "combine")


def test_eigen_distances_and_far_world_offset(Gvom):
    """eigen distances (2, 0) and a 1e4 m world offset (precision stress)."""
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    t = Terrain.make(0, extent=25.6, path_len=2.0, offset=(1.0e4, 0.0, 0.0))
    lid = Lidar(beams=32, columns=512)
    params = (0.1, 0.1, 256, 48, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 2, 0)
    scans = [make_scan(t, lid, p, i) for i, p in enumerate(make_trajectory(3))]
    _run_both(Gvom, params, scans)


def test_empty_and_out_of_grid_scans(Gvom):
    params = (0.2, 0.2, 64, 16, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    g = Gvom(*params)
    o = OracleGvom(*params)
    assert g.combine_maps() is None
    empty = np.zeros((0, 3), np.float32)
    far = np.array([[500.0, 0.0, 0.0], [0.0, -400.0, 3.0]], np.float32)  # no hit inside the grid
    for pts in (empty, far, empty):
        g.Process_pointcloud(pts, (0.1, 0.2, 1.0))
        o.Process_pointcloud(pts, (0.1, 0.2, 1.0))
        _, last = g.ring_state()
        compare_slot(canonical_state(g.slot_state(last)), canonical_state(o.slot_state(last)), "scan")
        out, ref = g.combine_maps(), o.combine_maps()
        for a, b in zip(out, ref):
            np.testing.assert_array_equal(a, b)


def test_nonfinite_points_dropped_like_oracle(Gvom):
    params = (0.2, 0.2, 64, 16, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    rng = np.random.default_rng(3)
    pts = rng.uniform(-6, 6, (2000, 3)).astype(np.float32)
    pts[::97, 1] = np.nan
    pts[::89, 2] = np.inf
    g, o = Gvom(*params), OracleGvom(*params)
    g.Process_pointcloud(pts, (0.0, 0.0, 0.0))
    o.Process_pointcloud(pts, (0.0, 0.0, 0.0))
    assert g.last_process_stats() == o.last_process_stats()
    compare_slot(canonical_state(g.slot_state(0)), canonical_state(o.slot_state(0)), "scan")


def test_batch_equals_sequential(Gvom):
    """process_batch over uneven scans (dropout) == Process_pointcloud one by one."""
    from gvom_gb300.synthetic import WORKLOADS, Lidar, make_scan, make_trajectory, scene_for
    w = WORKLOADS["small_32x512"]
    t, _ = scene_for(w)
    scans = []
    for i, p in enumerate(make_trajectory(5)):
        lid = Lidar(beams=(16, 32, 64)[i % 3], columns=512)
        scans.append(make_scan(t, lid, p, i, dropout=0.3 * (i % 2)))
    params = w.gvom_args()[:4] + (8,) + w.gvom_args()[5:]
    a, b = Gvom(*params), Gvom(*params)
    for s in scans:
        a.Process_pointcloud(s.points, s.ego, s.transform)
    b.process_batch([(s.points, s.ego, s.transform) for s in scans])
    assert a.ring_state() == b.ring_state()
    for slot in range(5):
        compare_slot(canonical_state(a.slot_state(slot)), canonical_state(b.slot_state(slot)), f"slot {slot}")
    ra, rb = a.combine_maps(), b.combine_maps()
    for x, y in zip(ra, rb):
        np.testing.assert_array_equal(x, y)


def test_batch_longer_than_ring_equals_sequential(Gvom):
    """process_batch of 7 scans into a 3-slot ring keeps the last 3 scans at
    the ring positions one call per scan gives them: the same ring state,
    slots and maps as the scans one by one."""
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 7)
    params = w.gvom_args()[:4] + (3,) + w.gvom_args()[5:]
    a, b = Gvom(*params), Gvom(*params)
    for s in scans[:2]:
        for m in (a, b):
            m.Process_pointcloud(s.points, s.ego, s.transform)
    for s in scans[2:]:
        a.Process_pointcloud(s.points, s.ego, s.transform)
    b.process_batch([(s.points, s.ego, s.transform) for s in scans[2:]])
    assert a.ring_state() == b.ring_state()
    for slot in range(3):
        compare_slot(canonical_state(a.slot_state(slot)), canonical_state(b.slot_state(slot)), f"slot {slot}")
    ra, rb = a.combine_maps(), b.combine_maps()
    for x, y in zip(ra, rb):
        np.testing.assert_array_equal(x, y)


def test_torch_device_input_and_device_outputs(Gvom):
    import torch
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    s = make_workload_scans(w, 1)[0]
    a, b = Gvom(*w.gvom_args()), Gvom(*w.gvom_args())
    a.Process_pointcloud(s.points, s.ego, s.transform)
    b.Process_pointcloud(torch.from_numpy(s.points).cuda(), s.ego, torch.from_numpy(s.transform))
    ra = a.combine_maps()
    X = w.xy_size
    dev = [torch.empty((X, X), dtype=d, device="cuda") for d in (torch.int32, torch.int32, torch.float64, torch.int32)]
    origin = b.combine_maps_device(*dev)
    b.synchronize()
    np.testing.assert_array_equal(origin, ra[0])
    for x, y in zip(ra[1:], dev):
        np.testing.assert_array_equal(x, y.cpu().numpy())


def test_debug_exports_vs_oracle(Gvom):
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    from oracle.canonical import sort_debug_voxels
    from replay import assert_eigen, assert_exact
    w = WORKLOADS["small_32x512"]
    s = make_workload_scans(w, 1)[0]
    g, o = Gvom(*w.gvom_args()), OracleGvom(*w.gvom_args())
    assert g.make_debug_voxel_map() is None
    for m in (g, o):
        m.Process_pointcloud(s.points, s.ego, s.transform)
        m.combine_maps()
    dv = g.make_debug_voxel_map()
    rv = sort_debug_voxels(o.make_debug_voxel_map())
    assert_exact(dv[:, :5], rv[:, :5], "debug voxel rows")
    assert np.all(np.diff(dv[:, 2]) >= 0), "rows not in voxel-id order"
    lmax = np.abs(rv[:, 5:6] + rv[:, 6:7] + rv[:, 7:8])
    assert_eigen(dv[:, 5:], rv[:, 5:], "eigen gaps", scale=np.maximum(lmax, np.abs(rv[:, 5:]).max(axis=1, keepdims=True)))


def test_repeated_combines_accumulate_like_reference(Gvom):
    """combine_maps called repeatedly without new scans re-adds the ring (scripts/gvom.py:242-298)."""
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 2)
    g, o = Gvom(*w.gvom_args()), OracleGvom(*w.gvom_args())
    for m in (g, o):
        for s in scans:
            m.Process_pointcloud(s.points, s.ego, s.transform)
    for k in range(4):
        out, ref = g.combine_maps(), o.combine_maps()
        refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
        compare_combine(out, refd, g.maps_state(), w.gvom_args(), f"combine {k}")
        compare_slot(canonical_state(g.combined_state()), canonical_state(o.combined_state()), f"combined {k}")


def test_graph_mode_equals_direct_launches(Gvom):
    """CUDA-graph replay (captured, updated in place, re-instantiated when the
    batch-size class or the source count changes) == direct launches."""
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 7)
    params = w.gvom_args()[:4] + (4,) + w.gvom_args()[5:]
    a, b = Gvom(*params), Gvom(*params)
    b.set_graphs(True)
    plan = [[0], [1], [2, 3], [4], [5, 6], [0]]  # one scan, then a batch, as the ring fills up
    for k, idx in enumerate(plan):
        batch = [(scans[i].points, scans[i].ego, scans[i].transform) for i in idx]
        for m in (a, b):
            if len(batch) == 1:
                m.Process_pointcloud(*batch[0])
            else:
                m.process_batch(batch)
        ra, rb = a.combine_maps(), b.combine_maps()
        for x, y in zip(ra, rb):
            np.testing.assert_array_equal(x, y)
        assert a.ring_state() == b.ring_state()
        compare_slot(canonical_state(a.combined_state()), canonical_state(b.combined_state()), f"combined {k}")


def test_precision_form_os1_128_far_vs_float64_oracle(Gvom):
    """The precision form at full size: OS1-128x2048 scans (262,144 points),
    512 x 512 x 96 at 0.1 m, buffer 8, world offset 1e4 m.  Integer outputs
    bit-exact; the largest float deviations from the float64 oracle are
    printed and held to the stated tolerances."""
    import json
    import torch
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    from replay import float_errors, stat_errors
    w = WORKLOADS["os1_128_far"]
    scans = make_workload_scans(w, 2, device="cuda" if torch.cuda.is_available() else "cpu")
    g, o = _run_both(Gvom, w.gvom_args(), scans)
    out = g.combine_maps()
    ref = o.combine_maps()
    refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
    compare_combine(out, refd, g.maps_state(), w.gvom_args(), "final combine")
    errs = float_errors(out, refd, g.maps_state())
    print("PRECISION os1_128_far " + json.dumps(errs))
    print("PRECISION os1_128_far stats " + json.dumps(stat_errors(g.combined_state(), o.combined_state())))
    assert errs["height_abs"] <= 1e-4 and errs["inferred_abs"] <= 1e-4
    assert errs["roughness_rel"] <= 1e-3 and errs["slope_x_rel"] <= 1e-3 and errs["slope_y_rel"] <= 1e-3


@pytest.mark.parametrize("graphs", [False, True])
def test_step_equals_process_then_combine(Gvom, graphs):
    """gvom_step (process + combine, index merge forked beside the statistics
    kernels) == process_batch followed by combine_maps."""
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 7)
    params = w.gvom_args()[:4] + (4,) + w.gvom_args()[5:]
    a, b = Gvom(*params), Gvom(*params)
    b.set_graphs(graphs)
    for k, idx in enumerate([[0], [1, 2], [3], [4, 5, 6], [0]]):
        batch = [(scans[i].points, scans[i].ego, scans[i].transform) for i in idx]
        a.process_batch(batch)
        ra = a.combine_maps()
        rb = b.step(batch)
        for x, y in zip(ra, rb):
            np.testing.assert_array_equal(x, y)
        assert a.ring_state() == b.ring_state()
        compare_slot(canonical_state(a.combined_state()), canonical_state(b.combined_state()), f"combined {k}")


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("pipeline", [0, 1, 2])
def test_steps_back_to_back_equal_sequential_calls(Gvom, graphs, pipeline):
    """Steps submitted without a host wait in between (device outputs), so that
    with step_pipeline a step's work overlaps the previous step's, with plain
    process / combine calls in the middle of the sequence and host-input steps
    among them: every step's maps equal those of process_batch + combine_maps."""
    import torch
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["small_32x512"]
    scans = make_workload_scans(w, 7)
    params = w.gvom_args()[:4] + (3,) + w.gvom_args()[5:]
    X = params[2]
    a, b = Gvom(*params), Gvom(*params)
    b.set_graphs(graphs)
    b.set_tuning(dict(b.get_tuning(), step_pipeline=pipeline))
    dev = [torch.from_numpy(np.ascontiguousarray(s.points)).cuda() for s in scans]
    order = [[0], [1, 2], [3], [4], "plain", [5, 6], [0], [2], [1, 3], [4]]
    want, got = [], []
    for k, idx in enumerate(order):
        if idx == "plain":  # the reference-style calls on the same instance, between steps
            s = scans[5]
            a.Process_pointcloud(s.points, s.ego, s.transform)
            b.Process_pointcloud(s.points, s.ego, s.transform)
            want.append(a.combine_maps())
            got.append(b.combine_maps())
            continue
        a.process_batch([(scans[i].points, scans[i].ego, scans[i].transform) for i in idx])
        want.append(a.combine_maps())
        outs = [torch.empty((X, X), dtype=d, device="cuda") for d in (torch.int32, torch.int32, torch.float64,
                                                                        torch.int32)]
        pts = (lambda i: scans[i].points) if k % 3 == 2 else (lambda i: dev[i])  # some steps with host inputs
        origin = b.step([(pts(i), scans[i].ego, scans[i].transform) for i in idx], device_outputs=outs)
        got.append((origin, outs))
    torch.cuda.synchronize()
    for k, (ra, rb) in enumerate(zip(want, got)):
        if isinstance(rb[1], list):
            rb = (rb[0], *[t.cpu().numpy() for t in rb[1]])
        for x, y in zip(ra, rb):
            np.testing.assert_array_equal(x, y, f"step {k}")
    assert a.ring_state() == b.ring_state()
    compare_slot(canonical_state(a.combined_state()), canonical_state(b.combined_state()), "combined")


def _compare_runs(Gvom, params, runs):
    """runs: [(points, ego, T), ...] each followed by a combine."""
    g, o = Gvom(*params), OracleGvom(*params)
    for i, (pts, ego, T) in enumerate(runs):
        g.Process_pointcloud(pts, ego, T)
        o.Process_pointcloud(pts, ego, T)
        assert g.last_process_stats() == o.last_process_stats(), (g.last_process_stats(), o.last_process_stats())
        _, last = g.ring_state()
        compare_slot(canonical_state(g.slot_state(last)), canonical_state(o.slot_state(last)), f"scan {i}")
        out, ref = g.combine_maps(), o.combine_maps()
        refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
        compare_combine(out, refd, g.maps_state(), params, f"combine {i}")


def test_rays_inside_the_sliver_below_zero(Gvom):
    """Ray positions in (-2^-20, 0) voxels with a non-zero grid origin: the one
    range where floor(p) - origin differs from the float64 formula."""
    params = (0.2, 0.2, 64, 16, 2, 0.1, 0.5, 0.5, 0.3, 2.0, 1.0, 1.0, 1, 1)
    rng = np.random.default_rng(11)
    # ego x = -1e-21 m: every position of a ray in the plane x = ego x is
    # -5e-21 voxels, where float64 rounds p - origin back up to -origin while
    # floor(p) - origin is one less
    ex = np.float32(-1.0e-21)
    ego = (float(ex), 0.05, 1.0)
    n = 3000
    pts = np.empty((n, 3), np.float32)
    pts[:, 0] = ex  # rays in the plane x = ego x: x stays inside the sliver for every step
    pts[:, 1] = rng.uniform(-6, 6, n)
    pts[:, 2] = rng.uniform(-1.5, 2.5, n)
    pts[: n // 3, 0] = np.float32(-1e-9) * rng.uniform(0, 1, n // 3).astype(np.float32)  # small negative x ends
    pts2 = pts.copy()
    pts2[:, 0] = np.float32(-4.0e-7)
    _compare_runs(Gvom, params, [(pts, ego, None), (pts2, (-2.0e-7, -0.03, 0.8), None)])


def test_origin_beyond_float32_floor_range(Gvom):
    """A world origin past 2^22 voxels: ray indices take the float64 path."""
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    t = Terrain.make(0, extent=12.8, path_len=2.0, offset=(5.0e5, -2.0e5, 0.0))
    lid = Lidar(beams=16, columns=256)
    params = (0.1, 0.1, 128, 32, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)  # 5e5 m / 0.1 m = 5e6 voxels
    runs = []
    for i, p in enumerate(make_trajectory(2)):
        s = make_scan(t, lid, p, i, transform_dtype=np.float64)
        runs.append((s.points, s.ego, s.transform))
    _compare_runs(Gvom, params, runs)


def test_odd_grid_and_row_length(Gvom):
    """xy_size 63 (extended rows of 65 cells) and eigen distances (1, 2)."""
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    t = Terrain.make(0, extent=12.6, path_len=2.0)
    lid = Lidar(beams=16, columns=512)
    params = (0.2, 0.2, 63, 21, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 2)
    runs = [(s.points, s.ego, s.transform) for s in
            (make_scan(t, lid, p, i) for i, p in enumerate(make_trajectory(2)))]
    _compare_runs(Gvom, params, runs)


@pytest.mark.parametrize("B", [1, 2, 4, 8, 12, 16])
def test_ring_sizes_every_source_class_vs_oracle(Gvom, B):
    """Rings of 1 to 16 slots, a combine after every scan: the merge runs with
    every source count from 1 to B + 1, so every source-count class of the
    index, count and statistics merges (2, 3, 5, 9 and 17 sources) is compared
    with the oracle, including the 17-source class with the ring full and
    after it wraps (scripts/gvom.py:242-298)."""
    import torch
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    n = B + 3
    t = Terrain.make(0, extent=12.8, path_len=n * 0.4)
    lid = Lidar(beams=16, columns=256)
    params = (0.2, 0.2, 64, 16, B, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    scans = [make_scan(t, lid, p, i, dropout=0.25, device=dev) for i, p in enumerate(make_trajectory(n))]
    _run_both(Gvom, params, scans)


def test_batched_8_shape_vs_oracle(Gvom):
    """The batched form's measured shape: 8 sensors of 16,384-262,144 points
    with 0-60 % whole-beam dropout on 4 mountings, 256 x 256 x 64 at 0.15 m,
    buffer 16.  Three steps of one process_batch each (one launch per kernel
    over the 8 scans), a combine after each (17 sources from the second step
    on): every written slot and every combine equal the oracle's run of the
    same scans one by one."""
    import torch
    from gvom_gb300.synthetic import BATCHED, make_batched_steps
    w = BATCHED["batched_8"]
    steps = make_batched_steps(w, 3, device="cuda" if torch.cuda.is_available() else "cpu")
    params = w.gvom_args()
    g = Gvom(*params)
    o = OracleGvom(*params, threads=os.cpu_count() or 1)
    for k, scans in enumerate(steps):
        g.process_batch([(s.points, s.ego, s.transform) for s in scans])
        for s in scans:
            o.Process_pointcloud(s.points, s.ego, s.transform)
        assert g.ring_state() == o.ring_state()
        bi, _ = g.ring_state()
        for j in range(len(scans)):
            slot = (bi - len(scans) + j) % w.buffer_size
            compare_slot(canonical_state(g.slot_state(slot)), canonical_state(o.slot_state(slot)),
                         f"step {k} slot {slot}")
        out, ref = g.combine_maps(), o.combine_maps()
        refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
        compare_combine(out, refd, g.maps_state(), params, f"step {k} combine")
        compare_slot(canonical_state(g.combined_state()), canonical_state(o.combined_state()), f"step {k} combined")


def test_os1_64_veg_30_scans_combine_each_vs_oracle(Gvom):
    """The headline workload's first 30 scans (256 x 256 x 64 at 0.15 m,
    buffer 4, OS1-64 + vegetation, float32 transforms) with a combine after
    every scan, so the previous combined map is carried through 30 merges."""
    import torch
    from gvom_gb300.synthetic import WORKLOADS, make_workload_scans
    w = WORKLOADS["os1_64_veg"]
    scans = make_workload_scans(w, 30, device="cuda" if torch.cuda.is_available() else "cpu")
    g = Gvom(*w.gvom_args())
    o = OracleGvom(*w.gvom_args(), threads=os.cpu_count() or 1)
    params = w.gvom_args()
    for i, s in enumerate(scans):
        g.Process_pointcloud(s.points, s.ego, s.transform)
        o.Process_pointcloud(s.points, s.ego, s.transform)
        _, last = g.ring_state()
        compare_slot(canonical_state(g.slot_state(last)), canonical_state(o.slot_state(last)), f"scan {i}")
        out, ref = g.combine_maps(), o.combine_maps()
        refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
        compare_combine(out, refd, g.maps_state(), params, f"combine after scan {i}")
    compare_slot(canonical_state(g.combined_state()), canonical_state(o.combined_state()), "combined")


@pytest.mark.parametrize("form", ["os1_64_veg", "batched_8"])
def test_pipelined_full_size_steps_equal_one_at_a_time(Gvom, form):
    """The measured forms at full size, steps submitted back to back from
    device memory with graphs on and the step pipeline at its deepest level,
    so that every overlap the pipeline allows happens (the device is held back
    until all steps are queued): every step's maps equal, and the combined
    map's statistics and debug voxel rows stay within tolerance of, the same
    steps run one call at a time with a wait after each (process_batch +
    combine_maps)."""
    import torch
    from gvom_gb300.synthetic import BATCHED, WORKLOADS, make_batched_steps, make_workload_scans
    from oracle.canonical import sort_debug_voxels
    from replay import assert_eigen, assert_exact
    if form in WORKLOADS:
        w = WORKLOADS[form]
        steps = [[s] for s in make_workload_scans(w, 12, device="cuda")]
    else:
        w = BATCHED[form]
        steps = make_batched_steps(w, 6, device="cuda")
    params = w.gvom_args()
    X = params[2]
    a, b = Gvom(*params), Gvom(*params)
    b.set_graphs(True)
    b.set_tuning(dict(b.get_tuning(), step_pipeline=2))
    dev = [[torch.from_numpy(np.ascontiguousarray(s.points)).cuda() for s in st] for st in steps]
    torch.cuda.synchronize()
    want = []
    for st in steps:
        a.process_batch([(s.points, s.ego, s.transform) for s in st])
        want.append(a.combine_maps())
    got = []
    outs_all = [[torch.empty((X, X), dtype=d, device="cuda") for d in (torch.int32, torch.int32, torch.float64,
                                                                        torch.int32)] for _ in steps]
    # hold the device back while every step is submitted: the mapper's stream
    # sleeps first, and the pipeline's streams start after it, so that all
    # the steps' work is queued before any of it runs
    hold = torch.cuda.Stream()
    b.set_stream(hold.cuda_stream)
    with torch.cuda.stream(hold):
        torch.cuda._sleep(200_000_000)
    for k, st in enumerate(steps):
        origin = b.step([(dev[k][j], s.ego, s.transform) for j, s in enumerate(st)], device_outputs=outs_all[k])
        got.append((origin, outs_all[k]))
    b.synchronize()
    b.set_stream(None)
    for k, (ra, (origin, outs)) in enumerate(zip(want, got)):
        rb = (origin, *[t.cpu().numpy() for t in outs])
        for x, y in zip(ra, rb):
            np.testing.assert_array_equal(x, y, f"step {k}")
    compare_slot(canonical_state(a.combined_state()), canonical_state(b.combined_state()), "combined")
    da, db = sort_debug_voxels(a.make_debug_voxel_map()), sort_debug_voxels(b.make_debug_voxel_map())
    assert_exact(db[:, :5], da[:, :5], "debug voxel rows")
    lmax = np.abs(da[:, 5:6] + da[:, 6:7] + da[:, 7:8])
    assert_eigen(db[:, 5:], da[:, 5:], "debug voxel eigen gaps",
                 scale=np.maximum(lmax, np.abs(da[:, 5:]).max(axis=1, keepdims=True)))
