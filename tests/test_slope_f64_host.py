"""The float64 plane-fit sequence of k_maps2d (`slope_f64_group` in
gvom_gb300/csrc/k_combine.cu, the path of the cells whose float32 fit cannot
be trusted; eight lanes per cell), compiled for the host from the kernel
source with its eight lanes emulated (tests/cpp/host_cuda/group_lanes.h),
and run on every cell of every golden fixture's height maps: its roughness
and slopes must equal the oracle's __calculate_slope (scripts/gvom.py:
717-805) bit for bit.  The device code uses only correctly rounded float64
operations (no contraction), so the host build performs the same
arithmetic; only the final log / atan2 is taken from the host's libm here,
as the oracle does."""
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
KERNEL = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc", "k_combine.cu")

PRELUDE = r"""
#include <algorithm>
#include <cmath>
#include "group_lanes.h"
using std::max; using std::min; using std::sqrt;
#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long b; std::memcpy(&b, &d, 8); return b; }
static inline double __longlong_as_double(long long b) { double d; std::memcpy(&d, &b, 8); return d; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
#define __dadd_rn(a, b) ((double)(a) + (double)(b))
#define __dsub_rn(a, b) ((double)(a) - (double)(b))
#define __dmul_rn(a, b) ((double)(a) * (double)(b))
#define __ddiv_rn(a, b) ((double)(a) / (double)(b))
constexpr int kHalo = %(halo)d;
static inline double rough_of(double err) { return err > 0.0 ? std::log(err) : err; }
static inline double slope_angle(double a, double m, double im) { (void)m; return std::atan2(a, im); }
"""

DRIVER = r"""
constexpr int kS = 600;
static double sh[kS][kS];
static unsigned char kn[kS][kS];
extern "C" int slope_all(const double *H, int X, double res, double *rough, double *sx, double *sy) {
    if (X + 2 * kHalo > kS) return 1;
    for (int i = 0; i < kS; i++)
        for (int j = 0; j < kS; j++) { sh[i][j] = -1000.0; kn[i][j] = 0; }
    for (int x = 0; x < X; x++)
        for (int y = 0; y < X; y++) {
            sh[x + kHalo][y + kHalo] = H[x * X + y];
            kn[x + kHalo][y + kHalo] = H[x * X + y] > -1000.0;
        }
    for (int x0 = 0; x0 < X; x0++)
        for (int y0 = 0; y0 < X; y0++) {
            double r = -1.0, a = 0.0, b = 0.0;
            int n = 0;
            for (int x = std::max(0, x0 - 1); x < std::min(X, x0 + 2); x++)
                for (int y = std::max(0, y0 - 1); y < std::min(X, y0 + 2); y++) n += kn[x + kHalo][y + kHalo];
            if (n >= 3) {
                double out[8];
                if (!run_group([&](int g) { return slope_f64_group<kS>(sh, kn, 0, 0, x0, y0, true, X, res, g); }, out))
                    return 2;
                r = out[0];
                a = out[1];
                b = out[2];
            }
            rough[x0 * X + y0] = r;
            sx[x0 * X + y0] = a;
            sy[x0 * X + y0] = b;
        }
    return 0;
}
"""


def _kernel_slope_source():
    """The kernel's widen helper and its eight-lane float64 sequence."""
    src = open(KERNEL).read()
    w = src.index("__device__ __forceinline__ double widen(float f) {")
    w_end = src.index("\n}\n", w) + 3
    a = src.index("template <int kSY>\n__device__ __forceinline__ double slope_f64_group")
    b = src.index("template <int kTX, int kTY>", a)
    return src[w:w_end] + src[a:b]


def _halo():
    import re
    for f in os.listdir(os.path.dirname(KERNEL)):
        m = re.search(r"constexpr int kHalo = (\d+);", open(os.path.join(os.path.dirname(KERNEL), f)).read())
        if m:
            return int(m.group(1))
    raise AssertionError("kHalo not found")


@pytest.fixture(scope="module")
def slope_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("slope")
    cpp = d / "slope_f64_host.cpp"
    cpp.write_text(PRELUDE % {"halo": _halo()} + _kernel_slope_source() + DRIVER)
    so = d / "libslope.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                    "-I", os.path.join(HERE, "cpp", "host_cuda"), "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.slope_all.argtypes = [P, C.c_int, C.c_double, P, P, P]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_float64_sequence_equals_oracle(slope_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    o = OracleGvom(*p)
    X, res = p[2], p[0]
    checked = 0
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        out = o.combine_maps()
        m = o.maps_state()
        H = np.ascontiguousarray(m["height"], np.float64)
        r, sx, sy = (np.empty((X, X)) for _ in range(3))
        assert slope_lib.slope_all(H.ctypes.data, X, res, r.ctypes.data, sx.ctypes.data, sy.ctypes.data) == 0
        np.testing.assert_array_equal(r, out[3])
        np.testing.assert_array_equal(sx, m["slope_x"])
        np.testing.assert_array_equal(sy, m["slope_y"])
        checked += int((r != -1.0).sum())
    # scenes without three known heights around any cell have no plane fit at all
    assert checked > 0 or name.split(".")[0] in ("kat_clear10", "kat_clear11", "kat_rays", "kat_eigen")


def _reference_slope(H, X, res, x0, y0):
    """__calculate_slope (scripts/gvom.py:717-805) for one cell, restated in
    Python floats (IEEE double, operations in the reference's order):
    (roughness, slope x, slope y), or None where the reference leaves the
    cell alone (fewer than three known neighbours, or det == 0)."""
    import math
    pts = [(x * res, y * res, H[x][y])
           for x in range(max(0, x0 - 1), min(X, x0 + 2))
           for y in range(max(0, y0 - 1), min(X, y0 + 2)) if H[x][y] > -1000]
    n = len(pts)
    if n < 3:
        return None
    mx = my = mz = 0.0
    for px, py, pz in pts:
        mx += px
        my += py
        mz += pz
    mx /= float(n)
    my /= float(n)
    mz /= float(n)
    xx = xy = xz = yy = yz = 0.0
    for px, py, pz in pts:
        xx += (px - mx) * (px - mx)
        xy += (px - mx) * (py - my)
        xz += (px - mx) * (pz - mz)
        yy += (py - my) * (py - my)
        yz += (py - my) * (pz - mz)
    det = xx * yy - xy * xy
    if det == 0.0:
        return None
    a0 = (yy * xz - xy * yz) / det
    a1 = (xx * yz - xy * xz) / det
    m = math.sqrt(a0 * a0 + a1 * a1 + 1)
    a0 /= m
    a1 /= m
    err = 0.0
    for px, py, pz in pts:
        e = (pz - mz) - (a0 * (px - mx) + a1 * (py - my))
        err += e * e
    err /= float(n)
    if err > 0:
        err = math.log(err)
    return err, math.atan2(a0, 1.0 / m), math.atan2(a1, 1.0 / m)


def test_kernel_float64_sequence_on_random_neighbourhoods(slope_lib):
    """Random height maps -- noise, voxel-quantised heights, flat patches,
    single known rows and columns, sparse known cells, map edges -- through
    the kernel's eight-lane sequence and the Python restatement: equal bit
    for bit on every cell with a plane fit."""
    rng = np.random.default_rng(17)
    X, checked = 24, 0
    for trial in range(24):
        res = (0.15, 0.2, 0.1, 0.25)[trial % 4]
        kind = trial % 6
        if kind == 0:
            H = rng.normal(0.0, 1.0, (X, X))
        elif kind == 1:  # voxel-quantised: integer z times a resolution plus a fraction
            H = rng.integers(-5, 20, (X, X)) * 0.15 + rng.random((X, X)) * 0.15
        elif kind == 2:  # flat patches
            H = np.repeat(np.repeat(rng.integers(0, 3, (X // 4, X // 4)) * 0.3, 4, 0), 4, 1).astype(np.float64)
        elif kind == 3:  # a gentle plane with tiny noise (near-cancellations)
            xs, ys = np.meshgrid(np.arange(X), np.arange(X), indexing="ij")
            H = 0.01 * xs + 0.02 * ys + rng.normal(0.0, 1e-9, (X, X))
        elif kind == 4:  # only some rows known (collinear neighbourhoods)
            H = rng.normal(0.0, 1.0, (X, X))
            H[rng.random(X) < 0.6, :] = -1000.0
        else:  # only some columns known
            H = rng.normal(0.0, 1.0, (X, X))
            H[:, rng.random(X) < 0.6] = -1000.0
        H[rng.random((X, X)) < 0.25] = -1000.0  # unknown cells
        H = np.ascontiguousarray(H, np.float64)
        r, sx, sy = (np.empty((X, X)) for _ in range(3))
        assert slope_lib.slope_all(H.ctypes.data, X, res, r.ctypes.data, sx.ctypes.data, sy.ctypes.data) == 0
        Hl = H.tolist()
        for x0 in range(X):
            for y0 in range(X):
                ref = _reference_slope(Hl, X, res, x0, y0)
                if ref is None:
                    # the kernel leaves the defaults (roughness -1, slopes 0)
                    n = sum(1 for x in range(max(0, x0 - 1), min(X, x0 + 2))
                            for y in range(max(0, y0 - 1), min(X, y0 + 2)) if Hl[x][y] > -1000)
                    if n >= 3:
                        assert (r[x0, y0], sx[x0, y0], sy[x0, y0]) == (-1.0, 0.0, 0.0), (trial, x0, y0)
                    continue
                got = (r[x0, y0], sx[x0, y0], sy[x0, y0])
                assert np.array(got).view(np.uint64).tolist() == np.array(ref).view(np.uint64).tolist(), \
                    (trial, x0, y0, got, ref)
                checked += 1
    assert checked > 5000
