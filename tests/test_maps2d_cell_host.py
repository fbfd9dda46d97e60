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


@pytest.mark.parametrize("seed", range(4))
def test_kernel_cell_path_on_random_terrain(cell_lib, seed):
    """Random voxel-quantised terrains -- each height built as the columns
    pass builds it, (in-voxel fraction + lowest occupied z + origin z) times
    z_res, from random slopes, steps, noise and flat stretches -- with a
    robot-disc patch and unknown cells, through the kernel's whole per-cell
    path (float32 fit, its rules, the closed forms, the queued float64
    sequence), against a plain-Python restatement of __calculate_slope at the
    parity tolerance."""
    from test_slope_f64_host import _reference_slope
    rng = np.random.default_rng(300 + seed)
    X = 40
    for trial in range(3):
        xy_res, z_res = (0.15, 0.2, 0.1)[trial], (0.15, 0.1, 0.2)[(trial + seed) % 3]
        oz = int(rng.integers(-30, 30))
        xs, ys = np.meshgrid(np.arange(X), np.arange(X), indexing="ij")
        kind = (trial + seed) % 4
        if kind == 0:  # plane with noise
            h = 0.05 * xs * xy_res + 0.12 * ys * xy_res + rng.normal(0, 0.02, (X, X))
        elif kind == 1:  # steps and flat stretches
            h = np.where(xs < X // 2, 0.0, 0.6) + np.where(ys % 9 < 4, 0.0, 0.3)
        elif kind == 2:  # rough ground
            h = rng.normal(0, 0.3, (X, X))
        else:  # a gentle ramp (small slopes, near-cancelling residuals)
            h = 0.002 * xs + 0.001 * ys + rng.normal(0, 1e-4, (X, X))
        w = h / z_res - oz  # in voxel units above the origin
        zl = np.floor(w).astype(np.int32)
        ml = (w - zl).astype(np.float32)
        H = (ml.astype(np.float64) + zl + oz) * z_res  # the columns pass's height
        disc = (xs - X // 3) ** 2 + (ys - X // 3) ** 2 <= 9  # robot disc: one float64 height, no voxel
        H[disc] = 0.7
        zl[disc] = -1
        ml[disc] = 0.0
        unknown = rng.random((X, X)) < 0.15
        H[unknown] = -1000.0
        zl[unknown] = -1
        ml[unknown] = 0.0
        H, zl, ml = (np.ascontiguousarray(a) for a in (H, zl, ml))
        r, sx, sy = (np.empty((X, X)) for _ in range(3))
        q = C.c_int()
        assert cell_lib.cells_all(H.ctypes.data, zl.ctypes.data, ml.ctypes.data, X, xy_res, z_res, r.ctypes.data,
                                  sx.ctypes.data, sy.ctypes.data, C.byref(q)) == 0
        Hl = H.tolist()
        rr, rx, ry = np.full((X, X), -1.0), np.zeros((X, X)), np.zeros((X, X))
        for x0 in range(X):
            for y0 in range(X):
                ref = _reference_slope(Hl, X, xy_res, x0, y0)
                if ref is not None:
                    rr[x0, y0], rx[x0, y0], ry[x0, y0] = ref
        assert_rel(r, rr, f"seed {seed} trial {trial} roughness", atol=1e-9)
        assert_rel(sx, rx, f"seed {seed} trial {trial} slope x", atol=SLOPE_ATOL)
        assert_rel(sy, ry, f"seed {seed} trial {trial} slope y", atol=SLOPE_ATOL)
