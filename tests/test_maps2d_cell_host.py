"""k_maps2d's slope and roughness path for every cell (gvom_gb300/csrc/
k_combine.cu: the float32 plane fit with its rules, the two closed forms,
and the float64 sequence for the cells the rules queue (its eight lanes
emulated), with the kernel's
float32 log / atan2), compiled for the host from the kernel source with the
whole map as one tile, against the oracle's float64 maps on every golden
fixture, at the parity tolerance (1e-3 relative)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.oracle import OracleGvom
from replay import assert_rel, load, ops_of, params_of, SLOPE_ATOL

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc")


def _kernel_parts():
    src = open(os.path.join(CSRC, "k_combine.cu")).read()
    h0 = src.index("// Doubles compared and widened on their bit patterns")
    h1 = src.index("\n}\n", src.index("__device__ __forceinline__ double widen(float f) {", h0)) + 3
    a = src.index("constexpr int kHalo = ")
    b = src.index("template <int kTX, int kTY>", a)
    helpers = src[h0:h1] + src[a:b]
    c = src.index("    double rough = -1.0, slx = 0.0, sly = 0.0;\n")
    d = src.index("    // cells that need the float64 sequence are compacted", c)
    return helpers, src[c:d]


DRIVER = r"""
constexpr int kS = 250;  // the whole map as one tile: X + 2 kHalo <= kS
static double sh[kS][kS];
static unsigned char kn[kS][kS];
static int szl[kS][kS];
static float sml[kS][kS];
struct { double xy_res, z_res; } mp;
extern "C" int cells_all(const double *H, const int *zlow, const float *mlow, int X, double xy_res, double z_res,
                         double *rough_out, double *sx_out, double *sy_out, int *queued) {
    if (X + 2 * kHalo > kS) return 1;
    for (int i = 0; i < kS; i++)
        for (int j = 0; j < kS; j++) { sh[i][j] = -1000.0; kn[i][j] = 0; szl[i][j] = -1; sml[i][j] = 0.f; }
    for (int x = 0; x < X; x++)
        for (int y = 0; y < X; y++) {
            const int c = x * X + y;
            sh[x + kHalo][y + kHalo] = H[c];
            kn[x + kHalo][y + kHalo] = height_known(H[c]) ? 1 : 0;
            szl[x + kHalo][y + kHalo] = zlow[c];
            sml[x + kHalo][y + kHalo] = mlow[c];
        }
    mp.xy_res = xy_res;
    mp.z_res = z_res;
    const int x0t = 0, y0t = 0;
    *queued = 0;
    for (int x0 = 0; x0 < X; x0++)
        for (int y0 = 0; y0 < X; y0++) {
            const bool valid = true;
            const int tid = 0;
            int qcell[1];
            int qn = 0;
%(cell)s
            if (need_exact) {
                double out[8];
                if (!run_group([&](int g) { return slope_f64_group<kS>(sh, kn, x0t, y0t, x0, y0, true, X, mp.xy_res, g); },
                               out))
                    return 2;
                rough = out[0];
                slx = out[1];
                sly = out[2];
                ++*queued;
            }
            (void)qcell;
            rough_out[x0 * X + y0] = rough;
            sx_out[x0 * X + y0] = slx;
            sy_out[x0 * X + y0] = sly;
        }
    return 0;
}
"""


@pytest.fixture(scope="module")
def cell_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    helpers, cell = _kernel_parts()
    d = tmp_path_factory.mktemp("cells")
    cpp = d / "cells_host.cpp"
    cpp.write_text("#include <algorithm>\n#include <cmath>\nusing std::max; using std::min;\n"
                   '#include "cuda_runtime.h"\n#include "group_lanes.h"\n' + helpers + DRIVER % {"cell": cell})
    so = d / "libcells.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                    "-I", os.path.join(HERE, "cpp", "host_cuda"), "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.cells_all.argtypes = [P, P, P, C.c_int, C.c_double, C.c_double, P, P, P, P]
    return lib


def _lowest(o, X, Z):
    cs = o.combined_state()
    idx = np.asarray(cs["index"]).reshape(Z, X, X)  # [z][y][x]
    occ = idx >= 0
    zl = np.where(occ.any(axis=0), occ.argmax(axis=0), -1).T.astype(np.int32)  # [x][y]
    ml = np.zeros((X, X), np.float32)
    xs, ys = np.nonzero(zl >= 0)
    ml[xs, ys] = np.asarray(cs["min_h"])[idx[zl[xs, ys], ys, xs]]
    return np.ascontiguousarray(zl), np.ascontiguousarray(ml)


@pytest.mark.parametrize("name", golden_files())
def test_kernel_cell_path_within_tolerance(cell_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    X, Z = p[2], p[3]
    o = OracleGvom(*p)
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        out = o.combine_maps()
        m = o.maps_state()
        H = np.ascontiguousarray(m["height"], np.float64)
        zl, ml = _lowest(o, X, Z)
        r, sx, sy = (np.empty((X, X)) for _ in range(3))
        q = C.c_int()
        assert cell_lib.cells_all(H.ctypes.data, zl.ctypes.data, ml.ctypes.data, X, p[0], p[1], r.ctypes.data,
                                  sx.ctypes.data, sy.ctypes.data, C.byref(q)) == 0
        assert_rel(r, out[3], f"{name} roughness", atol=1e-9)
        assert_rel(sx, m["slope_x"], f"{name} slope x", atol=SLOPE_ATOL)
        assert_rel(sy, m["slope_y"], f"{name} slope y", atol=SLOPE_ATOL)
