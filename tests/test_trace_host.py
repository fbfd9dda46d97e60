"""The ray-trace kernel's per-point code (k_voxelize_trace in
gvom_gb300/csrc/k_process.cu: transform, min-distance filter, exact hit
voxel, float32 march with the fast floor, the sliver, the shared cube and
hash table and their flush), compiled for the host from the kernel source
and run thread by thread, against the oracle on every scan of every golden
fixture: the per-voxel hit counts (the cell words) and totals (the index map
counted down from -1) of each slot must be equal.
The scan descriptor is filled the way the library's host code does
(prepare_scans in gvom_gb300/csrc/gvom_capi.cu)."""
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


def _matching_block(src, start):
    """src[start:] begins a line ending in '{': return through its matching '}'."""
    i = src.index("{", start)
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[start:j + 1]
    raise AssertionError("unbalanced braces")


def _kernel_parts():
    src = open(os.path.join(CSRC, "k_process.cu")).read()
    a = src.index("#ifndef GVOM_TRACE_HASH_BITS")
    b = src.index("constexpr unsigned kHashEmpty = 0xffffffffu;") + len("constexpr unsigned kHashEmpty = 0xffffffffu;")
    hashc = src[a:b]
    a = src.index("template <typename PT>\n__device__ __forceinline__ void load_point(")
    b = src.index("__device__ __forceinline__ void warp_add_u64(")
    helpers = src[a:b]
    k = src.index("__global__ void __launch_bounds__(256) k_voxelize_trace(")
    point = _matching_block(src, src.index("    if (active) {", k))
    f = src.index("    if (kHash)\n        for (int k = threadIdx.x; k < (1 << kHashBits); k += blockDim.x) {\n"
                  "            const unsigned t = htag[k];", k)
    flush_hash = _matching_block(src, f)
    c = src.index("    if (!sd.cube_on) return;", f)
    flush_cube = "    if (sd.cube_on)\n" + _matching_block(src, src.index("    for (int k = threadIdx.x; k < kCubeCells;", c))
    return hashc, helpers, point, flush_hash, flush_cube


DRIVER = r"""
namespace gvom {
template <typename PT>
static void trace_block(const ProcessConst &pc, const ScanDesc &sd, long long first, float4 *prec, int *prank) {
    static unsigned cube[kCubeCells];
    static unsigned htag[1 << kHashBits], hcnt[1 << kHashBits];
    for (int k = 0; k < kCubeCells; k++) cube[k] = 0u;
    for (int k = 0; k < (1 << kHashBits); k++) { htag[k] = kHashEmpty; hcnt[k] = 0u; }
    const Geom g = pc.g;
    const int ffloor = sd.fast_floor;
    const int Xe = g.Xe, XeXe = g.Xe * g.Xe;
    const int XX = g.X * g.X;
    for (int t = 0; t < 256; t++) {
        const long long i = first + t;
        const bool active = i < sd.n;
        unsigned long long n_valid = 0, n_hit = 0, n_steps = 0;
%(point)s
        (void)n_valid; (void)n_hit; (void)n_steps;
    }
%(flush_hash)s
%(flush_cube)s
}
}  // namespace gvom

using namespace gvom;

static ExactRes exact_res(double r) {
    int e;
    const double f = std::frexp(r, &e);
    ExactRes R;
    R.mr = (unsigned long long)std::ldexp(f, 53);
    R.er = e - 53;
    unsigned __int128 w = ((unsigned __int128)1 << 116) / R.mr;
    if (w >> 64) w = ~0ull;
    R.W = (unsigned long long)w;
    R.pad = 0;
    return R;
}

// prepare_scans (gvom_capi.cu) for one scan; counts of the grid's voxels out
extern "C" int trace_scan(const void *pts, int dtype, long long n, long long stride, const double *ego,
                          const double *T, int tmode, double xy_res, double z_res, int X, int Z, int exy, int ez,
                          double min_distance, int *hit, int *total, int pc2, const int *off, float *minh) {
    ProcessConst pc;
    std::memset(&pc, 0, sizeof pc);
    Geom &g = pc.g;
    g.X = X; g.Z = Z; g.exy = exy; g.ez = ez; g.Xe = X + 2 * exy; g.Ze = Z + 2 * ez;
    g.V = (long long)X * X * Z; g.Vext = (long long)g.Xe * g.Xe * g.Ze;
    pc.xy_res = xy_res; pc.z_res = z_res;
    pc.md2 = min_distance * min_distance;
    float f = (float)pc.md2;
    if ((double)f < pc.md2) f = std::nextafter(f, INFINITY);
    while ((double)std::nextafter(f, -INFINITY) >= pc.md2) f = std::nextafter(f, -INFINITY);
    pc.md2_f32 = f;
    pc.rxy = exact_res(xy_res);
    pc.rz = exact_res(z_res);
    pc.step_cap = 2 * std::max(X, Z) + 8;
    pc.nscans = 1;
    ScanDesc d;
    std::memset(&d, 0, sizeof d);
    d.pts = pts; d.n = n; d.stride = stride; d.tmode = tmode;
    d.pc2 = pc2;
    for (int a = 0; a < 3; a++) d.off[a] = off ? off[a] : 0;
    for (int r = 0; r < 12; r++) { d.T[r] = T ? T[r] : 0.0; d.Tf[r] = (float)d.T[r]; }
    d.od[0] = std::floor((ego[0] / xy_res) - (double)X / 2.0);
    d.od[1] = std::floor((ego[1] / xy_res) - (double)X / 2.0);
    d.od[2] = std::floor((ego[2] / z_res) - (double)Z / 2.0);
    bool fast = true, exact = true;
    const double lim = 4194304.0 - (double)std::max(X, Z) - 2.0;
    for (int a = 0; a < 3; a++) {
        if (!(std::fabs(d.od[a]) < 2147483648.0)) exact = false;
        if (!(std::fabs(d.od[a]) < lim)) fast = false;
    }
    for (int a = 0; a < 3; a++) d.oi[a] = exact ? (int)d.od[a] : 0;
    d.fast_floor = fast; d.exact_ok = exact;
    d.pt0[0] = (float)(ego[0] / xy_res); d.pt0[1] = (float)(ego[1] / xy_res); d.pt0[2] = (float)(ego[2] / z_res);
    d.cube_on = (fast && X >= kCube && Z >= kCube) ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        const int dim = a < 2 ? X : Z;
        int c = 0;
        if (d.cube_on) {
            const double ev = std::floor((double)d.pt0[a] - d.od[a]);
            c = (int)std::min(std::max(ev - kCube / 2, 0.0), (double)(dim - kCube));
        }
        d.cube0[a] = c;
    }
    unsigned long long *cnt = new unsigned long long[g.Vext]();
    int *vmap = new int[g.V];
    for (long long v = 0; v < g.V; v++) vmap[v] = -1;  // the slot's index map before the scan
    float4 *prec = new float4[n > 0 ? n : 1];
    int *prank = new int[n > 0 ? n : 1];
    d.cnt = cnt;
    d.idx = vmap;
    for (long long b = 0; b < n; b += 256) {
        if (dtype == 0) trace_block<float>(pc, d, b, prec, prank);
        else trace_block<double>(pc, d, b, prec, prank);
    }
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < X; y++)
            for (int x = 0; x < X; x++) {
                const unsigned long long w = cnt[(x + exy) + (long long)(y + exy) * g.Xe + (long long)(z + ez) * g.Xe * g.Xe];
                const long long v = x + (long long)y * X + (long long)z * X * X;
                hit[v] = (int)(w & 0xffffffffu);
                total[v] = -1 - vmap[v];
            }
    // lowest in-voxel height fraction per voxel from the points' records (cell, fractions)
    if (minh) {
        for (long long v = 0; v < g.V; v++) minh[v] = 1.0f;
        for (long long i = 0; i < n; i++) {
            const int cell = __float_as_int(prec[i].w);
            if (cell < 0) continue;
            const int ex = cell %% g.Xe, ey = (cell / g.Xe) %% g.Xe, ez2 = cell / (g.Xe * g.Xe);
            const int x = ex - exy, y = ey - exy, z = ez2 - ez;
            if (x < 0 || x >= X || y < 0 || y >= X || z < 0 || z >= Z) continue;
            const long long v = x + (long long)y * X + (long long)z * X * X;
            minh[v] = std::min(minh[v], prec[i].z);
        }
    }
    delete[] cnt; delete[] vmap; delete[] prec; delete[] prank;
    return 0;
}
"""


@pytest.fixture(scope="module")
def trace_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    hashc, helpers, point, flush_hash, flush_cube = _kernel_parts()
    d = tmp_path_factory.mktemp("trace")
    cpp = d / "trace_host.cpp"
    cpp.write_text("#include <algorithm>\n#include <cmath>\nusing std::isfinite;\n"
                   '#include "gvom_internal.cuh"\nnamespace gvom {\n' + hashc + "\n" + helpers + "\n}\n" +
                   DRIVER % {"point": point, "flush_hash": flush_hash, "flush_cube": flush_cube})
    so = d / "libtrace.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-frounding-math", "-fPIC", "-shared",
                    "-I", os.path.join(HERE, "cpp", "host_cuda"), "-I", CSRC, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.trace_scan.argtypes = [P, C.c_int, C.c_longlong, C.c_longlong, P, P, C.c_int, C.c_double, C.c_double,
                               C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, P, P, C.c_int, P, P]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_trace_counts_equal_oracle(trace_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    xy, zr, X, Z = p[0], p[1], p[2], p[3]
    o = OracleGvom(*p)
    V = X * X * Z
    for op in ops_of(fx):
        if op[0] != "P":
            continue
        _, pi, pts, ego, T = op
        pts = np.ascontiguousarray(pts)
        o.Process_pointcloud(pts, ego, T)
        _, last = o.ring_state()
        st = o.slot_state(last)
        idx = np.asarray(st["index"]).reshape(-1)
        ref_hit = np.zeros(V, np.int64)
        ref_total = np.zeros(V, np.int64)
        occ = idx >= 0
        ref_hit[occ] = np.asarray(st["hit"])[idx[occ]]
        ref_total[occ] = np.asarray(st["total"])[idx[occ]]
        ref_total[~occ] = -idx[~occ].astype(np.int64) - 1
        Td = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(4, 4))
        tmode = 0 if T is None else (1 if np.asarray(T).dtype == np.float32 else 2)
        e = np.ascontiguousarray(np.asarray(ego, np.float64))
        hit = np.empty(V, np.int32)
        total = np.empty(V, np.int32)
        minh = np.empty(V, np.float32)
        rc = trace_lib.trace_scan(pts.ctypes.data, 0 if pts.dtype == np.float32 else 1, pts.shape[0], pts.shape[1],
                                  e.ctypes.data, None if Td is None else Td.ctypes.data, tmode, xy, zr, X, Z,
                                  int(p[12]), int(p[13]), p[5], hit.ctypes.data, total.ctypes.data, 0, None,
                                  minh.ctypes.data)
        assert rc == 0
        np.testing.assert_array_equal(hit, ref_hit, f"{name} scan {pi} hits")
        np.testing.assert_array_equal(total, ref_total, f"{name} scan {pi} totals")
        # the points' z fractions (the exact hit-voxel arithmetic): their minimum per voxel is the slot's min height
        ref_minh = np.asarray(st["min_h"], np.float32)[idx[occ]]
        np.testing.assert_array_equal(minh[occ], ref_minh, f"{name} scan {pi} min height")


@pytest.mark.parametrize("name", ["synth_f32.npz", "kat_boundaries.npz", "synth_aniso_z.npz"])
def test_kernel_trace_reads_pointcloud2_bytes(trace_lib, name):
    """The same per-point code on PointCloud2-style bytes (float32 x, y, z at
    byte offsets 8, 0, 20 of 28-byte points, widened to float64 as the
    reference's ROS node does) against the oracle on the float64 points."""
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    xy, zr, X, Z = p[0], p[1], p[2], p[3]
    V = X * X * Z
    o = OracleGvom(*p)
    for op in ops_of(fx):
        if op[0] != "P":
            continue
        _, pi, pts, ego, T = op
        if pts.dtype != np.float32:
            continue
        n = pts.shape[0]
        rows = np.random.default_rng(pi).random((n, 7), dtype=np.float32)
        rows[:, 2], rows[:, 0], rows[:, 5] = pts[:, 0], pts[:, 1], pts[:, 2]
        rows = np.ascontiguousarray(rows)
        xyz = np.ascontiguousarray(pts.astype(np.float64))
        o.Process_pointcloud(xyz, ego, T)
        _, last = o.ring_state()
        st = o.slot_state(last)
        idx = np.asarray(st["index"]).reshape(-1)
        occ = idx >= 0
        ref_hit = np.zeros(V, np.int64)
        ref_total = np.where(occ, 0, -idx.astype(np.int64) - 1)
        ref_hit[occ] = np.asarray(st["hit"])[idx[occ]]
        ref_total[occ] = np.asarray(st["total"])[idx[occ]]
        Td = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(4, 4))
        e = np.ascontiguousarray(np.asarray(ego, np.float64))
        off = np.array([8, 0, 20], np.int32)
        hit = np.empty(V, np.int32)
        total = np.empty(V, np.int32)
        assert trace_lib.trace_scan(rows.ctypes.data, 1, n, 28, e.ctypes.data, None if Td is None else Td.ctypes.data,
                                    0 if T is None else 2, xy, zr, X, Z, int(p[12]), int(p[13]), p[5],
                                    hit.ctypes.data, total.ctypes.data, 1, off.ctypes.data, None) == 0
        np.testing.assert_array_equal(hit, ref_hit, f"{name} scan {pi} hits")
        np.testing.assert_array_equal(total, ref_total, f"{name} scan {pi} totals")


def _adversarial_scan(rng, res, zres, X, Z, ego, n):
    """Points around `ego`: uniform in and beyond the map, on voxel
    boundaries, in the float sliver just below zero, inside the minimum
    distance, and non-finite."""
    half = X * res / 2
    p = [ego + rng.uniform(-1.3 * half, 1.3 * half, (n, 3)) * [1, 1, 0.2]]
    k = rng.integers(-X, X, (n // 4, 3)).astype(np.float64)
    p.append(np.floor(ego / [res, res, zres]) * [res, res, zres] + k * [res, res, zres])  # on boundaries
    s = ego + rng.uniform(-half, half, (n // 8, 3)) * [1, 1, 0.2]
    s[:, rng.integers(0, 3)] = -rng.choice([1e-7, 2.0 ** -21, 2.0 ** -24, 1e-30, 0.0], n // 8)  # the sliver
    p.append(s)
    p.append(ego + rng.normal(0, 0.3, (n // 16, 3)))  # within the minimum distance
    bad = ego + rng.uniform(-1, 1, (8, 3))
    bad[:3, 0] = [np.nan, np.inf, -np.inf]
    p.append(bad)
    return np.concatenate(p)


@pytest.mark.parametrize("seed", range(6))
def test_kernel_trace_counts_on_adversarial_scans(trace_lib, seed):
    """Random scans built to reach the exact paths of the per-point code --
    points on voxel boundaries, coordinates in (-2^-20, 0), rays leaving the
    grid, points inside the minimum distance, non-finite points; float32 and
    float64 points and transforms; maps near the world origin and 1e4 m away;
    rays whose every step lies in the sliver -- against the oracle: hits,
    totals and min heights equal."""
    rng = np.random.default_rng(900 + seed)
    res, zres = (0.2, 0.15)[seed % 2], (0.2, 0.1, 0.15)[seed % 3]
    X, Z = int(rng.integers(20, 34)), int(rng.integers(10, 18))
    p = (res, zres, X, Z, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    far = 1e4 if seed >= 4 else 0.0
    ego = np.array([far + rng.uniform(-3, 3), far / 2 + rng.uniform(-3, 3), rng.uniform(-1, 1)])
    V = X * X * Z
    o = OracleGvom(*p)
    for scan in range(3 if far == 0.0 else 2):
        pts = _adversarial_scan(rng, res, zres, X, Z, ego, 3000)
        dt = np.float32 if (seed + scan) % 2 == 0 else np.float64
        if scan == 2:
            # rays in the plane x = ego x, ego x just below zero: every step of
            # them lies in the sliver (-2^-20, 0) voxels
            ego = np.array([float(np.float32(-1e-21)), rng.uniform(-1, 1), 1.0])
            pts = np.empty((3000, 3))
            pts[:, 0] = ego[0]
            pts[:, 1] = ego[1] + rng.uniform(-X * res / 2, X * res / 2, 3000)
            pts[:, 2] = rng.uniform(-1.5, 2.5, 3000)
            pts[:1000, 0] = -1e-9 * rng.random(1000)  # small negative x ends
            dt, T = np.float32, None
        elif scan == 0:
            T = None
        else:  # a sensor pose: rotation about z, translation to the ego; points in the sensor frame
            a = rng.uniform(-0.2, 0.2)
            R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
            T = np.eye(4)
            T[:3, :3] = R
            T[:3, 3] = ego
            T = T.astype(dt)
            with np.errstate(invalid="ignore"):  # the non-finite rows stay non-finite
                pts = (pts - ego) @ R  # R^T (w - ego), row by row
        pts = np.ascontiguousarray(pts.astype(dt))
        o.Process_pointcloud(pts, ego, T)
        _, last = o.ring_state()
        st = o.slot_state(last)
        idx = np.asarray(st["index"]).reshape(-1)
        ref_hit = np.zeros(V, np.int64)
        ref_total = np.zeros(V, np.int64)
        occ = idx >= 0
        ref_hit[occ] = np.asarray(st["hit"])[idx[occ]]
        ref_total[occ] = np.asarray(st["total"])[idx[occ]]
        ref_total[~occ] = -idx[~occ].astype(np.int64) - 1
        Td = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(4, 4))
        tmode = 0 if T is None else (1 if T.dtype == np.float32 else 2)
        e = np.ascontiguousarray(ego)
        hit = np.empty(V, np.int32)
        total = np.empty(V, np.int32)
        minh = np.empty(V, np.float32)
        rc = trace_lib.trace_scan(pts.ctypes.data, 0 if pts.dtype == np.float32 else 1, pts.shape[0], pts.shape[1],
                                  e.ctypes.data, None if Td is None else Td.ctypes.data, tmode, res, zres, X, Z,
                                  1, 1, p[5], hit.ctypes.data, total.ctypes.data, 0, None, minh.ctypes.data)
        assert rc == 0
        np.testing.assert_array_equal(hit, ref_hit, f"seed {seed} scan {scan} hits")
        np.testing.assert_array_equal(total, ref_total, f"seed {seed} scan {scan} totals")
        np.testing.assert_array_equal(minh[occ], np.asarray(st["min_h"], np.float32)[idx[occ]],
                                      f"seed {seed} scan {scan} min height")
        assert occ.sum() > 50
