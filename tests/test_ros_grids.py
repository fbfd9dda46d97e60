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
    v = np.concatenate([rng.uniform(-300, 300, 20000), np.arange(-260, 260, 0.25), rng.uniform(-1e12, 1e12, 2000),
                        [-1e10, 1e10, 0.0, -0.0, 2.0 ** 31 - 0.5, 2.0 ** 31, 2.0 ** 31 + 255, -2.0 ** 31,
                         -2.0 ** 31 - 0.5, -2.0 ** 31 - 1, 3e9 + 7, 1e19, -1e19, np.nan, np.inf, -np.inf]])
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


def test_kernel_int8_cast_equals_numpy_on_x86(tmp_path):
    """k_ros_grids' int8 cast (`int8_wrap` in gvom_gb300/csrc/k_combine.cu),
    compiled for the host from the kernel source, equals numpy's
    float64 -> int8 astype on x86 (the node's host) and the oracle's."""
    import ctypes as C
    import os
    import shutil
    import subprocess
    import warnings
    if shutil.which("g++") is None or platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("needs g++ on x86")
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "gvom_gb300", "csrc", "k_combine.cu")).read()
    a = src.index("__device__ __forceinline__ signed char int8_wrap(")
    b = src.index("\n}\n", a) + 3
    cpp = tmp_path / "int8.cpp"
    cpp.write_text("#include <cmath>\nusing std::fabs;\n#define __device__\n#define __forceinline__ inline\n" + src[a:b] +
                   'extern "C" void wrap_all(const double *v, long long n, signed char *o) '
                   "{ for (long long i = 0; i < n; i++) o[i] = int8_wrap(v[i]); }\n")
    so = tmp_path / "libint8.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    lib.wrap_all.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p]
    rng = np.random.default_rng(9)
    v = np.concatenate([rng.uniform(-300, 300, 50000), np.arange(-260, 260, 0.125), rng.uniform(-1e12, 1e12, 1000),
                        [np.nan, np.inf, -np.inf, 1e19, -1e19, 0.0, -0.0, 127.9, 128.0, -128.9, -129.0]])
    got = np.empty(v.size, np.int8)
    lib.wrap_all(v.ctypes.data, v.size, got.ctypes.data)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        want = v.astype(np.int8)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got, int8_wrap(v))


def test_kernel_payloads_equal_the_reference_callback(tmp_path):
    """k_ros_grids (gvom_gb300/csrc/k_combine.cu), compiled for the host from
    the kernel source through the host stand-in header and run cell by cell,
    on the maps of tests/golden/ros_epilogue.npz: its five payloads equal
    what the reference node's callback published for them, byte for byte."""
    import ctypes as C
    import os
    import shutil
    import subprocess
    from conftest import GOLDEN
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "gvom_gb300", "csrc")
    src = open(os.path.join(csrc, "k_combine.cu")).read()
    a = src.index("__device__ __forceinline__ signed char int8_wrap(")
    k = src.index("__global__ void __launch_bounds__(256) k_ros_grids(")
    b = src.index("\n}\n", k) + 3
    cpp = tmp_path / "ros_host.cpp"
    cpp.write_text('#include <cmath>\nusing std::fabs; using std::isnan;\n#include "gvom_internal.cuh"\n'
                   "namespace gvom {\n" + src[a:b] + "}\nusing namespace gvom;\n"
                   'extern "C" void grids(const RosGridParams *p) {\n'
                   "    for (int i = 0; i < p->X * p->X; i++) { blockIdx.x = i; threadIdx.x = 0; blockDim.x = 1; k_ros_grids(*p); }\n"
                   "}\n")
    so = tmp_path / "libros.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(here, "cpp", "host_cuda"), "-I", csrc, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))

    class Params(C.Structure):
        _fields_ = [("X", C.c_int), ("pos", C.c_void_p), ("neg", C.c_void_p), ("vis", C.c_void_p),
                    ("rough", C.c_void_p), ("density_thr", C.c_double), ("min_r", C.c_double), ("max_r", C.c_double),
                    ("hard", C.c_void_p), ("soft", C.c_void_p), ("certainty", C.c_void_p), ("negative", C.c_void_p),
                    ("roughness", C.c_void_p)]
    lib.grids.argtypes = [C.POINTER(Params)]
    with np.load(os.path.join(GOLDEN, "ros_epilogue.npz")) as z:
        fx = {k: z[k] for k in z.files}
    for n in str(fx["cases"]).split(","):
        pos, neg, vis = (np.ascontiguousarray(fx[f"{n}_{k}"], np.int32) for k in ("pos", "neg", "vis"))
        rough = np.ascontiguousarray(fx[f"{n}_rough"], np.float64)
        X = pos.shape[0]
        out = {k: np.zeros(X * X, np.int8) for k in ("hard", "soft", "certainty", "negative", "roughness")}
        thr, lo, hi = fx[f"{n}_params"]
        prm = Params(X, pos.ctypes.data, neg.ctypes.data, vis.ctypes.data, rough.ctypes.data, thr, lo, hi,
                     *[out[k].ctypes.data for k in ("hard", "soft", "certainty", "negative", "roughness")])
        lib.grids(C.byref(prm))
        for pub, key in PAYLOAD_OF.items():
            np.testing.assert_array_equal(out[key], fx[f"{n}_{pub}"], f"{n} {pub}")
