"""k_columns (gvom_gb300/csrc/k_combine.cu: height of the lowest occupied
voxel or the robot disc, inferred height of the lowest free voxel, and the
positive-obstacle band density), compiled for the host from the kernel
source and run column by column on the oracle's combined map of every golden
fixture, with the column parameters filled as the library's host code fills
them: heights and inferred heights bit for bit, band densities equal to the
oracle's obstacle map wherever the slope does not decide it."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.oracle import OracleGvom
from replay import load, ops_of, params_of

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc")
PLANES = 16  # z planes per column-summary chunk (the merge's default)

DRIVER = r"""
using namespace gvom;
extern "C" int columns_all(const int *idx, const int *hit, const int *total, const float *minh, int X, int Z,
                           const double *co, const double *ego, double xy_res, double z_res, double robot_r,
                           double lidar_h, double pos_thr, double robot_h, double *height, double *inferred,
                           int *pos_density) {
    const long long V = (long long)X * X * Z;
    const int planes = %(planes)d, nch = (Z + planes - 1) / planes;
    VoxelRec *rec = new VoxelRec[V]();
    int2 *colinfo = new int2[(long long)nch * X * X];
    for (long long v = 0; v < V; v++)
        if (idx[v] >= 0) { rec[v].hit = hit[v]; rec[v].total = total[v]; rec[v].min_h = minh[v]; }
    for (int ch = 0; ch < nch; ch++)
        for (int y = 0; y < X; y++)
            for (int x = 0; x < X; x++) {
                int occ_z = Z, free_z = Z;
                for (int z = ch * planes; z < std::min(Z, (ch + 1) * planes); z++) {
                    const int c = idx[x + y * X + (long long)z * X * X];
                    if (c >= 0 && occ_z == Z) occ_z = z;
                    if (c < -1 && free_z == Z) free_z = z;
                }
                colinfo[(long long)ch * X * X + y * X + x] = int2{occ_z, free_z};
            }
    ColumnParams cp;
    std::memset(&cp, 0, sizeof cp);
    cp.X = X; cp.Z = Z; cp.planes = planes; cp.idx = idx; cp.rec = rec; cp.colinfo = colinfo;
    for (int a = 0; a < 3; a++) { cp.co[a] = co[a]; cp.ego[a] = ego[a]; }
    cp.xy_res = xy_res; cp.z_res = z_res;
    cp.robot_r2 = robot_r * robot_r;
    cp.disc_h = ego[2] - lidar_h;
    cp.pos_thr = pos_thr; cp.robot_h = robot_h;
    cp.pthr_v = (float)(pos_thr / z_res);
    cp.robh_v = (float)(robot_h / z_res);
    cp.base_xf = (float)(co[0] * xy_res - ego[0]);
    cp.base_yf = (float)(co[1] * xy_res - ego[1]);
    cp.res_f = (float)xy_res;
    cp.r2_f = (float)cp.robot_r2;
    int *zlow = new int[(long long)X * X];
    float *mlow = new float[(long long)X * X];
    cp.height = height; cp.inferred = inferred; cp.pos_density = pos_density; cp.zlow = zlow; cp.mlow = mlow;
    for (int by = 0; by * 8 < X; by++)
        for (int bx = 0; bx * 32 < X; bx++)
            for (int ty = 0; ty < 8; ty++)
                for (int tx = 0; tx < 32; tx++) {
                    blockIdx.x = bx; blockIdx.y = by; threadIdx.x = tx; threadIdx.y = ty;
                    k_columns(cp);
                }
    delete[] rec; delete[] colinfo; delete[] zlow; delete[] mlow;
    return 0;
}
"""


@pytest.fixture(scope="module")
def columns_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(os.path.join(CSRC, "k_combine.cu")).read()
    h0 = src.index("// Doubles compared and widened on their bit patterns")
    h1 = src.index("\n}\n", src.index("__device__ __forceinline__ double widen(float f) {", h0)) + 3
    a = src.index("__device__ __forceinline__ bool near_integer(")
    k = src.index("__global__ void __launch_bounds__(256) k_columns(")
    b = src.index("\n}\n", k) + 3
    d = tmp_path_factory.mktemp("columns")
    cpp = d / "columns_host.cpp"
    cpp.write_text("#include <algorithm>\n#include <cmath>\nusing std::floor; using std::fabs;\n"
                   '#include "gvom_internal.cuh"\nnamespace gvom {\n' + src[h0:h1] + src[a:b] + "}\n" +
                   DRIVER % {"planes": PLANES})
    so = d / "libcolumns.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(HERE, "cpp", "host_cuda"), "-I", CSRC, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.columns_all.argtypes = [P, P, P, P, C.c_int, C.c_int, P, P] + [C.c_double] * 6 + [P, P, P]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_columns_equal_oracle(columns_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    xy, zr, X, Z = p[0], p[1], p[2], p[3]
    V = X * X * Z
    o = OracleGvom(*p)
    ego = None
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            ego = np.asarray(op[3], np.float64)
            continue
        out = o.combine_maps()
        m = o.maps_state()
        cs = o.combined_state()
        idx = np.asarray(cs["index"], np.int32).reshape(-1)
        occ = idx >= 0
        full = lambda a, dt: np.ascontiguousarray(  # noqa: E731
            np.where(occ, np.asarray(a)[np.where(occ, idx, 0)], 0).astype(dt))
        vidx = np.ascontiguousarray(np.where(occ, np.arange(V), idx).astype(np.int32))
        co = np.ascontiguousarray(np.round(np.asarray(out[0]) / np.array([xy, xy, zr])))
        e = np.ascontiguousarray(ego)
        h, inf = np.empty((X, X)), np.empty((X, X))
        pd = np.empty((X, X), np.int32)
        hit, total, minh = full(cs["hit"], np.int32), full(cs["total"], np.int32), full(cs["min_h"], np.float32)
        columns_lib.columns_all(vidx.ctypes.data, hit.ctypes.data, total.ctypes.data, minh.ctypes.data,
                                X, Z, co.ctypes.data, e.ctypes.data, xy, zr, p[10], p[11], p[6], p[9],
                                h.ctypes.data, inf.ctypes.data, pd.ctypes.data)
        np.testing.assert_array_equal(h, m["height"], f"{name} height")
        np.testing.assert_array_equal(inf, m["inferred"], f"{name} inferred")
        steep = np.hypot(m["slope_x"], m["slope_y"]) >= p[8]
        np.testing.assert_array_equal(pd[~steep], out[1][~steep], f"{name} band density")


def _reference_columns(idx, hit, total, minh, X, Z, co, ego, xy_res, z_res, robot_r, lidar_h, pos_thr, robot_h):
    """__make_height_map, __make_inferred_height_map and the band density of
    __make_positive_obstacle_map (scripts/gvom.py:515-590) restated in Python
    floats per column, the voxel's record fields given per voxel: (height,
    inferred height, band density)."""
    import math
    H = np.full((X, X), -1000.0)
    INF = np.full((X, X), -1000.0)
    PD = np.zeros((X, X), np.int64)
    for x in range(X):
        for y in range(X):
            xp = ((co[0] + x) * xy_res) - ego[0]
            yp = ((co[1] + y) * xy_res) - ego[1]
            if xp * xp + yp * yp <= robot_r * robot_r:
                H[x, y] = ego[2] - lidar_h
            for z in range(Z):
                v = x + y * X + z * X * X
                if idx[v] >= 0:
                    H[x, y] = (float(minh[v]) + z + co[2]) * z_res
                    break
            for z in range(Z):
                if idx[x + y * X + z * X * X] < -1:
                    INF[x, y] = (z + co[2]) * z_res
                    break
            lo = int(math.floor(((H[x, y] + pos_thr) / z_res) - co[2])) + 1
            hi = int(math.floor(((H[x, y] + robot_h) / z_res) - co[2]))
            if not (0 <= lo < Z and 0 <= hi < Z):
                continue
            dens = n = 0.0
            for z in range(lo, hi + 1):
                v = x + y * X + z * X * X
                if idx[v] >= 0 and hit[v] > 10:
                    n += float(total[v])
                    dens += float(hit[v])
            if n > 0.0:
                dens /= n
            PD[x, y] = int(dens * 100)
    return H, INF, PD


@pytest.mark.parametrize("seed", range(4))
def test_kernel_columns_on_random_maps(columns_lib, seed):
    """Random combined maps (occupied voxels with hit / total counts and
    in-voxel heights, some placed so that the band limits fall within 1e-6
    of a voxel boundary; free and unknown voxels; a robot disc; varied
    origins and resolutions): heights, inferred heights and band densities
    equal to the Python restatement, the heights bit for bit."""
    rng = np.random.default_rng(50 + seed)
    X, Z = 14, 24
    V = X * X * Z
    for trial in range(3):
        z_res = (0.1, 0.15, 0.2)[trial]
        xy_res, pos_thr, robot_h = 0.2, (0.3, 0.25, 0.5)[seed % 3], 2.0
        co = np.ascontiguousarray(np.array([rng.integers(-40, 40), rng.integers(-40, 40), rng.integers(-10, 10)],
                                           np.float64))
        ego = np.ascontiguousarray(np.array([(co[0] + X / 2) * xy_res, (co[1] + X / 2) * xy_res, 1.0]))
        u = rng.random(V)
        idx = np.where(u < 0.2, 0, np.where(u < 0.6, -1, -2 - rng.integers(0, 5, V))).astype(np.int32)
        # make most columns have their lowest occupied voxel in the lower half
        hit = rng.integers(0, 40, V).astype(np.int32)
        total = (hit + rng.integers(0, 40, V)).astype(np.int32)
        minh = rng.random(V).astype(np.float32)
        # in-voxel heights that put minh + pos_thr / z_res within 1e-6 of an integer
        near = rng.random(V) < 0.3
        frac = np.float32(pos_thr / z_res - np.floor(pos_thr / z_res))
        minh[near] = np.clip(np.float32(1.0) - frac + rng.normal(0, 1e-6, near.sum()).astype(np.float32), 0, 0.9999)
        vidx = np.ascontiguousarray(np.where(idx >= 0, np.arange(V), idx).astype(np.int32))
        h, inf = np.empty((X, X)), np.empty((X, X))
        pd = np.empty((X, X), np.int32)
        robot_r, lidar_h = 0.6, 0.8
        columns_lib.columns_all(vidx.ctypes.data, hit.ctypes.data, total.ctypes.data, minh.ctypes.data, X, Z,
                                co.ctypes.data, ego.ctypes.data, xy_res, z_res, robot_r, lidar_h, pos_thr, robot_h,
                                h.ctypes.data, inf.ctypes.data, pd.ctypes.data)
        H, INF, PD = _reference_columns(idx, hit, total, minh, X, Z, co, ego, xy_res, z_res, robot_r, lidar_h,
                                        pos_thr, robot_h)
        np.testing.assert_array_equal(h.view(np.uint64), H.view(np.uint64))
        np.testing.assert_array_equal(inf.view(np.uint64), INF.view(np.uint64))
        np.testing.assert_array_equal(pd, PD)
        assert (PD > 0).any()
