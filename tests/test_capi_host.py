"""The library's C ABI on the CPU: gvom_capi.cu compiled for the host over a
stand-in of the CUDA runtime calls it makes (tests/cpp/host_cuda/
host_runtime.h: device memory is tracked host memory, launches complete when
issued, graph capture is refused), with every kernel file compiled unchanged
and run block by block under tests/cpp/host_cuda/block_threads.h, loaded
through the package's own binding (gvom_gb300.Gvom over gvom_gb300/_lib.py).
So the host code the GPU tests run -- the ring of physical slots and its
spares, the scan tables, batches, the step pipeline at every level, the
device-output path, the free-memory admission, the debug exports -- runs here
against the golden fixtures and the oracle.  Every device allocation sits
between guard zones; after each test no write may have landed in one."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.canonical import canonical_state
from oracle.oracle import OracleGvom
from replay import compare_combine, compare_slot, load, ops_of, params_of, replay_and_compare

CAPI_PRELUDE = r"""
#define __CUDACC__ 1
#include <algorithm>
#include <cmath>
#include "cuda_runtime.h"
#include "host_runtime.h"
"""

# settable device memory of the stand-in runtime, for the admission tests
CAPI_TAIL = r"""
extern "C" void host_runtime_set_total(unsigned long long bytes) { host_runtime::total = bytes; }
extern "C" unsigned long long host_runtime_used() { return host_runtime::used; }
// guard zones overwritten so far (freed allocations, and live ones now)
extern "C" unsigned long long host_runtime_guard_faults() {
    host_runtime::check_live();
    return host_runtime::guard_faults;
}
extern "C" void host_runtime_set_junk(unsigned char v) { host_runtime::junk = v; }
extern "C" void block_threads_shuffle(unsigned long long seed) {
    block_threads::shuffle_seed = seed;
    block_threads::shuffle_state = seed;
}
"""


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from hostbuild import CSRC, PRELUDE, compile_units, host_source
    read = lambda f: open(os.path.join(CSRC, f)).read()  # noqa: E731
    capi = read("gvom_capi.cu").replace('#include "../../include/gvom_gb300.h"', '#include "gvom_gb300.h"')
    units = {"proc.cpp": PRELUDE + '#include "k_process.cu"\n',
             "comb.cpp": PRELUDE + host_source(read("k_combine.cu")),
             "morph.cpp": PRELUDE + host_source(read("k_morph.cu")),
             "dbg.cpp": PRELUDE + host_source(read("k_debug_static.cu")),
             "capi.cpp": CAPI_PRELUDE + capi + CAPI_TAIL}
    so = compile_units(units, tmp_path_factory.mktemp("capi"), "libgvom_host.so")
    from gvom_gb300 import _lib
    saved = _lib._lib
    lib = _lib.load(str(so))
    raw = C.CDLL(str(so))
    raw.host_runtime_set_total.argtypes = [C.c_ulonglong]
    raw.host_runtime_used.restype = C.c_ulonglong
    raw.block_threads_shuffle.argtypes = [C.c_ulonglong]
    raw.host_runtime_guard_faults.restype = C.c_ulonglong
    raw.host_runtime_set_junk.argtypes = [C.c_ubyte]
    _lib._lib = lib
    # GVOM_HOST_SHUFFLE=<seed>: every test of the module under a shuffled schedule
    raw.block_threads_shuffle(int(os.environ.get("GVOM_HOST_SHUFFLE", "0")))
    try:
        yield lib, raw
    finally:
        _lib._lib = saved


@pytest.fixture(autouse=True)
def _no_write_out_of_bounds(host_lib):
    """After every test, with its instances freed: no guard zone around any
    device allocation was overwritten (a write past either end of a buffer,
    by a kernel or by the host code)."""
    yield
    import gc
    gc.collect()
    assert host_lib[1].host_runtime_guard_faults() == 0


def _gvom(params):
    from gvom_gb300 import Gvom
    return Gvom(*params)


@pytest.mark.parametrize("name", golden_files())
def test_c_abi_replays_every_fixture(host_lib, name):
    """gvom_gb300.Gvom over the host-built library through every fixture:
    slots, combined maps, maps and debug exports against the reference."""
    fx = load(os.path.join(GOLDEN, name))
    replay_and_compare(_gvom(params_of(fx)), fx)


def _scans_of(fx):
    return [(op[2], op[3], op[4]) for op in ops_of(fx) if op[0] == "P"]


def _compare_ring(g, o, what):
    assert g.ring_state() == o.ring_state(), what
    B = int(g.params[4])
    for s in range(B):
        a, b = g.slot_state(s), o.slot_state(s)
        assert (a is None) == (b is None), (what, s)
        if a is not None:
            compare_slot(canonical_state(a), canonical_state(b), f"{what} slot {s}")


def _compare_combine(out, o, g, params, what):
    ref = o.combine_maps()
    refd = dict(origin=ref[0], pos=ref[1], neg=ref[2], rough=ref[3], vis=ref[4], **o.maps_state())
    compare_combine(out, refd, g.maps_state(), params, what)
    compare_slot(canonical_state(g.combined_state()), canonical_state(o.combined_state()), f"{what} combined")


@pytest.mark.parametrize("name,k", [("synth_ring16.npz", 16), ("synth_ring16.npz", 5), ("synth_longrun.npz", 3)])
def test_process_batch_equals_oracle(host_lib, name, k):
    """gvom_process_batch: the fixture's scans k at a time (the ring wraps
    inside a batch for the 16-slot ring), each batch then combined; every
    ring slot and every combine equal the oracle's sequential calls."""
    fx = load(os.path.join(GOLDEN, name))
    params = params_of(fx)
    g, o = _gvom(params), OracleGvom(*params)
    scans = _scans_of(fx)
    for b0 in range(0, len(scans), k):
        batch = scans[b0:b0 + k]
        g.process_batch(batch)
        for pts, ego, T in batch:
            o.Process_pointcloud(pts, ego, T)
        _compare_ring(g, o, f"batch at {b0}")
        _compare_combine(g.combine_maps(), o, g, params, f"combine after batch at {b0}")


class _HostTensor:
    """A buffer of the stand-in runtime's "device" (host memory) with the one
    method the binding reads from a device tensor."""

    def __init__(self, shape, dtype):
        self.a = np.zeros(shape, dtype)

    def data_ptr(self):
        return self.a.ctypes.data


@pytest.mark.parametrize("pipeline", [0, 1, 2])
def test_steps_at_every_pipeline_level_equal_oracle(host_lib, pipeline):
    """gvom_step back to back with device outputs, at step-pipeline levels 0,
    1 and 2 (the trace of a step beside the previous step's combine, the
    process and merges beside its maps; spare slots taken and released), and
    with host outputs: every step's maps equal the oracle's process +
    combine."""
    fx = load(os.path.join(GOLDEN, "synth_ring16.npz"))
    params = params_of(fx)
    g, o = _gvom(params), OracleGvom(*params)
    g.set_tuning({"step_pipeline": pipeline})
    X = int(params[2])
    scans = _scans_of(fx)
    for i in range(0, len(scans), 2):
        batch = scans[i:i + 2]
        for pts, ego, T in batch:
            o.Process_pointcloud(pts, ego, T)
        if i % 4 == 0:
            outs = [_HostTensor((X, X), d) for d in (np.int32, np.int32, np.float64, np.int32)]
            origin = g.step(batch, device_outputs=outs)
            g.synchronize()
            out = (origin, outs[0].a, outs[1].a, outs[2].a, outs[3].a)
        else:
            out = g.step(batch)
        _compare_combine(out, o, g, params, f"step {i // 2} (level {pipeline})")
    _compare_ring(g, o, "after the steps")


def test_admission_refuses_what_does_not_fit(host_lib):
    """The free-memory admission: an instance larger than the device is
    refused with GVOM_ERR_OOM before it allocates; a scan whose scratch does
    not fit is refused with GVOM_ERR_OOM and leaves the instance usable."""
    from gvom_gb300._lib import GVOM_ERR_OOM, GvomError
    _, raw = host_lib
    fx = load(os.path.join(GOLDEN, "synth_f32.npz"))
    params = params_of(fx)
    raw.host_runtime_set_total(256 << 20)
    try:
        big = (0.1, 0.1, 512, 96) + tuple(params[4:])
        used = raw.host_runtime_used()
        with pytest.raises(GvomError) as e:
            _gvom(big)
        assert e.value.code == GVOM_ERR_OOM and raw.host_runtime_used() == used
        g, o = _gvom(params), OracleGvom(*params)
        scans = _scans_of(fx)
        pts, ego, T = scans[0]
        g.Process_pointcloud(pts, ego, T)
        o.Process_pointcloud(pts, ego, T)
        huge = np.zeros((8_000_000, 3), np.float32)
        with pytest.raises(GvomError) as e:
            g.Process_pointcloud(huge, ego, T)
        assert e.value.code == GVOM_ERR_OOM
        pts, ego, T = scans[1]
        g.Process_pointcloud(pts, ego, T)
        o.Process_pointcloud(pts, ego, T)
        _compare_ring(g, o, "after the refusal")
        _compare_combine(g.combine_maps(), o, g, params, "combine after the refusal")
    finally:
        raw.host_runtime_set_total(8 << 30)


def test_allocation_free_debug_export_and_reserve(host_lib):
    """gvom_reserve allocates up front; the allocation-free voxel export
    (file-scope scratch, caller-owned output) gives the regular export's
    rows; neither allocates during the calls."""
    lib, raw = host_lib
    fx = load(os.path.join(GOLDEN, "synth_f64T_veg.npz"))
    params = params_of(fx)
    g = _gvom(params)
    scans = _scans_of(fx)
    g.reserve(2, max(s[0].shape[0] for s in scans) * 2)
    before = raw.host_runtime_used()
    for pts, ego, T in scans:
        g.Process_pointcloud(pts, ego, T)
    assert raw.host_runtime_used() == before  # nothing allocated after the reservation
    g.combine_maps()
    rows = g.make_debug_voxel_map()
    out = np.zeros((rows.shape[0] + 5, 8), np.float32)
    n = C.c_int64()
    assert lib.gvom_debug_voxel_map_noalloc(g._h, out.ctypes.data_as(C.c_void_p), out.shape[0], C.byref(n)) == 0
    assert n.value == rows.shape[0]
    np.testing.assert_array_equal(out[:n.value], rows)


def test_error_codes(host_lib):
    """The C ABI's argument and state errors, on the host build."""
    from gvom_gb300._lib import GVOM_ERR_ARG, GVOM_NO_DATA
    lib, _ = host_lib
    fx = load(os.path.join(GOLDEN, "kat_shift.npz"))
    g = _gvom(params_of(fx))
    assert g.combine_maps() is None  # an empty ring: the reference's None
    origin = np.zeros(3)
    assert lib.gvom_combine(g._h, origin.ctypes.data_as(C.c_void_p), None, None, None, None) == GVOM_NO_DATA
    assert lib.gvom_process(None, None, 0, 0, 3, None, None, -1) == GVOM_ERR_ARG
    bad = np.zeros((4, 3), np.float32)
    ego = (C.c_double * 3)(0, 0, 0)
    assert lib.gvom_process(g._h, bad.ctypes.data_as(C.c_void_p), 7, 4, 3, ego, None, -1) == GVOM_ERR_ARG


# the GPU parity tests whose inputs are host arrays, at their own sizes,
# against the host build (the others need CUDA tensors, graph capture, or
# grids of millions of voxels per step)
GPU_TESTS_ON_HOST = ["test_small_32x512_vs_oracle", "test_float64_ros_style_inputs",
                     "test_empty_and_out_of_grid_scans", "test_nonfinite_points_dropped_like_oracle",
                     "test_batch_equals_sequential", "test_batch_longer_than_ring_equals_sequential",
                     "test_debug_exports_vs_oracle",
                     "test_repeated_combines_accumulate_like_reference", "test_rays_inside_the_sliver_below_zero",
                     "test_origin_beyond_float32_floor_range", "test_odd_grid_and_row_length"]


@pytest.mark.parametrize("name", GPU_TESTS_ON_HOST)
def test_gpu_parity_tests_on_the_host_build(host_lib, name):
    import test_parity_gpu
    from gvom_gb300 import Gvom
    getattr(test_parity_gpu, name)(Gvom)


@pytest.mark.parametrize("B", [1, 16])
def test_gpu_ring_size_test_on_the_host_build(host_lib, B):
    import test_parity_gpu
    from gvom_gb300 import Gvom
    test_parity_gpu.test_ring_sizes_every_source_class_vs_oracle(Gvom, B)


@pytest.mark.parametrize("layout", [0, 2])
def test_gpu_pointcloud2_tests_on_the_host_build(host_lib, layout):
    """The ROS ingestion test's host-memory layouts (float32 x, y, z at 0, 4,
    8 of 16-byte points; float64 at 8, 16, 24 of 40-byte points, widened as
    the node does) and its argument checks, against the host build."""
    import test_ros_ingest
    marks = test_ros_ingest.test_pointcloud2_equals_process_pointcloud.pytestmark
    layouts = next(m.args[1] for m in marks if m.name == "parametrize")
    assert not layouts[layout]["device"]
    test_ros_ingest.test_pointcloud2_equals_process_pointcloud(host_lib[0], layouts[layout])
    test_ros_ingest.test_pointcloud2_argument_checks(host_lib[0])


def test_gpu_ros_grids_test_on_the_host_build(host_lib):
    import test_ros_grids
    test_ros_grids.test_device_payloads_equal_oracle(host_lib[0])


@pytest.mark.parametrize("seed", range(16))
def test_random_call_sequences_equal_oracle(host_lib, seed):
    """Seeded random sequences of the library's calls on a small map -- single
    scans, batches of 1 to 20 scans (longer than the ring too), steps at a
    random pipeline level with host or device outputs, combines, debug
    exports, empty and out-of-grid scans -- against the oracle's sequential
    calls, compared after every call: ring state, every slot, every combine's
    maps and combined map."""
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    rng = np.random.default_rng(1000 + seed)
    B = int(rng.integers(1, 7))
    X, Z = int(rng.choice([20, 24, 31])), int(rng.choice([8, 12]))
    exy, ez = [(1, 1), (2, 0), (0, 1), (1, 2)][int(rng.integers(4))]
    params = (0.3, 0.25, X, Z, B, 0.8, 0.5, 0.5, 0.3, 2.0, 1.5, 1.0, exy, ez)
    t = Terrain.make(seed, extent=X * 0.3, path_len=12.0)
    lid = Lidar(beams=8, columns=128)
    poses = make_trajectory(40)
    pool = []
    for i, p in enumerate(poses):
        s = make_scan(t, lid, p, i, dropout=float(rng.uniform(0, 0.5)),
                      transform_dtype=np.float64 if i % 3 == 0 else np.float32)
        pts = s.points if i % 4 else s.points.astype(np.float64)
        pool.append((pts, s.ego, s.transform))
    pool.append((np.zeros((0, 3), np.float32), poses[0].ego if hasattr(poses[0], "ego") else pool[0][1], None))
    pool.append((np.array([[500.0, 0.0, 0.0]], np.float32), pool[1][1], None))
    g, o = _gvom(params), OracleGvom(*params)
    nxt = 0

    def take(n):
        nonlocal nxt
        out = []
        for _ in range(n):
            out.append(pool[nxt % len(pool)] if rng.random() > 0.08 else pool[-1 - int(rng.integers(2))])
            nxt += 1
        return out

    combined = False
    for step in range(20):
        what = f"seed {seed} call {step}"
        op = rng.choice(["scan", "batch", "step", "combine", "debug"], p=[0.3, 0.25, 0.25, 0.15, 0.05])
        if op == "scan":
            (pts, ego, T), = take(1)
            g.Process_pointcloud(pts, ego, T)
            o.Process_pointcloud(pts, ego, T)
        elif op == "batch":
            batch = take(int(rng.integers(1, 21)))
            if len({b[0].dtype for b in batch}) > 1:
                batch = [(b[0].astype(np.float32), b[1], b[2]) for b in batch]
            g.process_batch(batch)
            for pts, ego, T in batch:
                o.Process_pointcloud(pts, ego, T)
        elif op == "step":
            batch = take(int(rng.integers(1, 5)))
            if len({b[0].dtype for b in batch}) > 1:
                batch = [(b[0].astype(np.float32), b[1], b[2]) for b in batch]
            g.set_tuning({"step_pipeline": int(rng.integers(0, 3))})
            for pts, ego, T in batch:
                o.Process_pointcloud(pts, ego, T)
            if rng.random() < 0.5:
                outs = [_HostTensor((X, X), d) for d in (np.int32, np.int32, np.float64, np.int32)]
                origin = g.step(batch, device_outputs=outs)
                g.synchronize()
                out = (origin, outs[0].a, outs[1].a, outs[2].a, outs[3].a)
            else:
                out = g.step(batch)
            _compare_combine(out, o, g, params, what)
            combined = True
        elif op == "combine":
            out = g.combine_maps()
            if out is None:
                assert o.combine_maps() is None, what
            else:
                _compare_combine(out, o, g, params, what)
                combined = True
        elif op == "debug" and combined:
            from oracle.canonical import sort_debug_voxels
            from replay import assert_exact
            dv, rv = sort_debug_voxels(g.make_debug_voxel_map()), sort_debug_voxels(o.make_debug_voxel_map())
            assert_exact(dv[:, :5], rv[:, :5], what)
        _compare_ring(g, o, what)


def _adversarial_scan(rng, params, ego):
    """Points on voxel boundaries and corners, piles of hundreds to
    thousands in one voxel, points inside the minimum distance, outside the
    grid and non-finite, around `ego`."""
    xy, zr, X, Z = params[0], params[1], params[2], params[3]
    n = int(rng.integers(200, 3000))
    half = np.array([X * xy / 2, X * xy / 2, Z * zr / 2])
    p = ego + rng.uniform(-1.2, 1.2, (n, 3)) * half
    k = rng.random(n)
    snap = k < 0.3  # onto voxel faces / corners
    p[snap] = np.round(p[snap] / [xy, xy, zr]) * [xy, xy, zr]
    pile = (k >= 0.3) & (k < 0.45)  # one voxel, many points
    c = ego + rng.uniform(-0.4, 0.4, 3) * half
    p[pile] = c + rng.uniform(0, 1, (int(pile.sum()), 3)) * [xy, xy, zr] * 0.999
    near = (k >= 0.45) & (k < 0.5)  # inside the minimum distance
    p[near] = ego + rng.normal(size=(int(near.sum()), 3)) * params[5] * 0.3
    far = (k >= 0.5) & (k < 0.55)
    p[far] = ego + rng.uniform(-1, 1, (int(far.sum()), 3)) * half * 20
    bad = rng.random(n) < 0.01
    p[bad, int(rng.integers(3))] = np.nan
    return p.astype(np.float64 if rng.random() < 0.4 else np.float32)


@pytest.mark.parametrize("seed", range(8))
def test_adversarial_scans_equal_oracle(host_lib, seed):
    """Adversarial scans (voxel boundaries, piles in one voxel, minimum
    distance, outside the grid, non-finite) through process and combine on
    small maps, against the oracle after every call."""
    rng = np.random.default_rng(2000 + seed)
    B = int(rng.integers(1, 5))
    X, Z = int(rng.choice([16, 21, 32])), int(rng.choice([8, 10]))
    exy, ez = [(1, 1), (2, 1), (0, 0), (1, 2)][seed % 4]
    params = (float(rng.choice([0.2, 0.25, 0.3])), float(rng.choice([0.2, 0.4])), X, Z, B, 0.5, 0.5, 0.5, 0.3,
              2.0, 1.0, 1.0, exy, ez)
    g, o = _gvom(params), OracleGvom(*params)
    ego = np.array([0.05, -0.1, 0.9])
    for i in range(6):
        ego = ego + rng.uniform(-0.5, 0.5, 3) * [1, 1, 0.1]
        pts = _adversarial_scan(rng, params, ego)
        T = None
        if i % 2:
            a = rng.uniform(-0.3, 0.3)
            T = np.array([[np.cos(a), -np.sin(a), 0, 0.1], [np.sin(a), np.cos(a), 0, -0.2], [0, 0, 1, 0.05],
                          [0, 0, 0, 1]], np.float64 if i % 4 == 1 else np.float32)
        g.Process_pointcloud(pts, tuple(ego), T)
        o.Process_pointcloud(pts, tuple(ego), T)
        assert g.last_process_stats() == o.last_process_stats(), f"seed {seed} scan {i}"
        _compare_ring(g, o, f"seed {seed} scan {i}")
        _compare_combine(g.combine_maps(), o, g, params, f"seed {seed} combine {i}")


@pytest.mark.parametrize("seed", [1, 2])
@pytest.mark.parametrize("name", ["kat_boundaries.npz", "kat_guess.npz", "kat_eigen.npz", "synth_f64T_veg.npz",
                                  "synth_ring16.npz", "small_32x512.npz"])
def test_shuffled_schedules_replay_fixtures(host_lib, name, seed):
    """Fixture replays with a shuffled schedule: blocks in a random order and
    a random ready thread resumed at every barrier phase, so a read that only
    a missing barrier separates from its write, or code that counts on block
    order, would change the results.  Integer outputs stay exact, statistics
    within the parity tolerance."""
    _, raw = host_lib
    raw.block_threads_shuffle(seed)
    try:
        fx = load(os.path.join(GOLDEN, name))
        replay_and_compare(_gvom(params_of(fx)), fx)
    finally:
        raw.block_threads_shuffle(int(os.environ.get("GVOM_HOST_SHUFFLE", "0")))


def test_gpu_step_test_on_the_host_build(host_lib):
    """The GPU test that gvom_step equals process_batch + combine_maps, with
    graphs off (the host runtime refuses capture), against the host build."""
    import test_parity_gpu
    from gvom_gb300 import Gvom
    test_parity_gpu.test_step_equals_process_then_combine(Gvom, False)


def test_headline_workload_on_the_host_build(host_lib):
    """The GPU test of the headline workload's trajectory (os1_64_veg: 256 x
    256 x 64 voxels at 0.15 m, six OS1-64 scans with vegetation, about 95K
    points each, a combine after each) against the host build: the grid
    sizes, block counts, hash table and large-cell paths of the measured
    configuration."""
    import test_parity_gpu
    from gvom_gb300 import Gvom
    test_parity_gpu.test_os1_64_vegetation_trajectory_vs_oracle(Gvom)


@pytest.mark.skipif(os.environ.get("GVOM_HOST_FULL_SIZE") != "1",
                    reason="full-size forms on the host take minutes (GVOM_HOST_FULL_SIZE=1 runs them)")
@pytest.mark.parametrize("name", ["test_batched_8_shape_vs_oracle",
                                  "test_precision_form_os1_128_far_vs_float64_oracle"])
def test_full_size_gpu_tests_on_the_host_build(host_lib, name):
    """The batched_8 shape (8 sensors, 16 slots) and the precision form
    (512 x 512 x 96, two OS1-128 scans, 1e4 m offset) against the host
    build."""
    import test_parity_gpu
    from gvom_gb300 import Gvom
    getattr(test_parity_gpu, name)(Gvom)


def test_gpu_far_world_offset_test_on_the_host_build(host_lib):
    """Eigen distances (2, 0) at a 1e4 m world offset on 256 x 256 x 48."""
    import test_parity_gpu
    from gvom_gb300 import Gvom
    test_parity_gpu.test_eigen_distances_and_far_world_offset(Gvom)


def test_gpu_launch_shape_test_on_the_host_build(host_lib):
    """The autotuner's test that every launch shape (points per block,
    merge planes, statistics blocks, index-merge overlap, maps tile, step
    pipeline) gives identical maps, against the host build."""
    import test_autotune
    test_autotune.test_every_launch_shape_gives_identical_maps(host_lib[0])


@pytest.mark.parametrize("junk", [0x00, 0xff])
@pytest.mark.parametrize("name", ["kat_guess.npz", "synth_ring16.npz", "synth_f64T_veg.npz"])
def test_results_do_not_depend_on_fresh_memory(host_lib, name, junk):
    """Fixture replays with fresh device allocations holding 0x00 or 0xff
    instead of the usual pattern: a result that read memory before it was
    written would change with what fresh memory holds."""
    _, raw = host_lib
    raw.host_runtime_set_junk(junk)
    try:
        fx = load(os.path.join(GOLDEN, name))
        replay_and_compare(_gvom(params_of(fx)), fx)
    finally:
        raw.host_runtime_set_junk(0xa5)


def test_image_kernel_entry_points_on_the_host_build(host_lib):
    """gvom_expand_binary / gvom_lowpass_binary / gvom_convolve through the C
    ABI of the host build (buffers are the host runtime's device memory):
    the reference's own outputs on the fixture cases, the oracle on staged
    and unstaged sizes, and the argument refusals."""
    from oracle.oracle import convolve, expand_binary, lowpass_binary
    from gvom_gb300._lib import GVOM_ERR_ARG
    lib, _ = host_lib
    P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    with np.load(os.path.join(GOLDEN, "morph_binary.npz")) as z:
        fx = {k: z[k] for k in z.files}
    n = 0
    while f"expand{n}_img" in fx:
        img = np.ascontiguousarray(fx[f"expand{n}_img"], np.int32)
        out = np.full_like(img, -7)
        assert lib.gvom_expand_binary(P(img), P(out), img.shape[0], float(fx[f"expand{n}_r"]), None) == 0
        np.testing.assert_array_equal(out, fx[f"expand{n}_out"])
        n += 1
    n = 0
    while f"lowpass{n}_img" in fx:
        img = np.ascontiguousarray(fx[f"lowpass{n}_img"], np.int32)
        out = np.full_like(img, -7)
        assert lib.gvom_lowpass_binary(P(img), P(out), img.shape[0], int(fx[f"lowpass{n}_fs"]),
                                       float(fx[f"lowpass{n}_frac"]), None) == 0
        np.testing.assert_array_equal(out, fx[f"lowpass{n}_out"])
        n += 1
    rng = np.random.default_rng(9)
    a = (rng.uniform(size=(100, 100)) < 0.003).astype(np.int32)
    out = np.full_like(a, -7)
    assert lib.gvom_expand_binary(P(a), P(out), 100, 60.0, None) == 0  # beyond the shared staging
    np.testing.assert_array_equal(out, expand_binary(a, 60.0))
    d = rng.normal(size=(33, 33))
    k = rng.normal(size=(4, 4))
    outd = np.full_like(d, np.nan)
    assert lib.gvom_convolve(P(d), P(outd), P(k), 33, 4, None) == 0
    np.testing.assert_array_equal(outd, convolve(d, k))
    b = np.zeros((8, 8), np.int32)
    assert lib.gvom_expand_binary(None, None, 8, 1.0, None) == GVOM_ERR_ARG
    assert lib.gvom_lowpass_binary(P(b), P(b), 8, -1, 0.5, None) == GVOM_ERR_ARG
    assert lib.gvom_convolve(P(d), P(outd), P(k), 8, 0, None) == GVOM_ERR_ARG
