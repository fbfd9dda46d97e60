"""The per-voxel neighbourhood statistics (__calculate_mean,
__normalize_mean, __calculate_covariance, __normalize_covariance,
__calculate_min_height: scripts/gvom.py:1249-1421) as the kernels compute
them, compiled for the host from gvom_gb300/csrc/k_process.cu: k_cell_moments'
one-thread and one-warp cell sums (the warp run lane by lane with its
shuffles emulated), then k_voxel_stats' four-lane (eigen distances 1, 1) and
one-thread (any distances) Chan combinations of the neighbour cells.  Inputs
are adversarial cells -- up to 20,000 points in a cell, points piled on one
spot, on the cell's faces, on a plane or a line, two far clusters -- in and
around a small grid.  Counts and minimum heights must equal the float64
truth; means and covariances must lie within the parity tolerance the GPU
tests apply against the oracle's float64 sums."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from replay import STAT_ATOL, STAT_RTOL

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc")

PRELUDE = r"""
#include <algorithm>
#include <cmath>
#include <cstdlib>
using std::max; using std::min;
template <class T> static inline T __ldg(const T *p) { return *p; }
#include "gvom_internal.cuh"

// Lane-by-lane emulation of a warp (or of one four-lane group of it) whose
// shuffles all lie outside divergent branches: each lane runs alone; a
// shuffle records the caller's value and returns its source lane's value at
// the same call in the previous pass; passes repeat until nothing changes
// (a fixpoint), which is lockstep execution's result.
namespace lanes {
constexpr int kMax = 32, kCalls = 4096;
inline int n = 32, lane = 0, call = 0;
inline float rec[kMax][kCalls], prev[kMax][kCalls];
}  // namespace lanes
static inline float lane_shfl(float v, int src) {
    using namespace lanes;
    const int k = call++;
    if (k >= kCalls) std::abort();
    rec[lane][k] = v;
    return (src >= 0 && src < n) ? prev[src][k] : v;
}
static inline float __shfl_xor_sync(unsigned, float v, int o) { return lane_shfl(v, lanes::lane ^ o); }
static inline float __shfl_down_sync(unsigned, float v, int d) { return lane_shfl(v, lanes::lane + d); }
template <class F>
static bool run_lanes(int nl, F f, int max_passes = 64) {
    using namespace lanes;
    n = nl;
    std::memset(prev, 0, sizeof prev);
    for (int p = 0; p < max_passes; p++) {
        int calls = -1;
        for (int g = 0; g < nl; g++) {
            lane = g;
            call = 0;
            f(g);
            if (calls >= 0 && call != calls) return false;
            calls = call;
        }
        bool fixed = true;
        for (int g = 0; g < nl && fixed; g++) fixed = std::memcmp(rec[g], prev[g], sizeof(float) * calls) == 0;
        if (fixed) return true;
        for (int g = 0; g < nl; g++) std::memcpy(prev[g], rec[g], sizeof(float) * calls);
    }
    return false;
}
#define store_min_h(...) ((void)0)
namespace gvom {
"""

DRIVER = r"""
struct FakeScan {
    VoxelRec *rec;
    const unsigned long long *cnt;
    long long pt_base;
};

// one cell's moments by the one-thread body (warp = 0) or the one-warp body
// (warp = 1) of k_cell_moments, written to mom[off]
extern "C" int cell_moments(const float4 *sorted, int off, int n, int warp, CellMom *mom) {
    FakeScan sd{nullptr, nullptr, 0};
    if (!warp) {
        bool mine = true;
        const int ci = -1;
        (void)ci;
SMALL_BODY
        return 0;
    }
    const int hq_off[1] = {off}, hq_n[1] = {n}, hq_rec[1] = {-1};
    (void)hq_rec;
    const int q = 0;
    return run_lanes(32, [&](int lane_) {
        const int lane = lane_;
WARP_BODY
    }) ? 0 : 1;
}

extern "C" int small_cell_limit() { return kSmallCell; }

// k_voxel_stats for records 0..C-1: e3 = 1 the four-lane body (eigen
// distances 1, 1), e3 = 0 the one-thread body
extern "C" int voxel_stats(const unsigned long long *cnt, const CellMom *M, VoxelRec *rec, int C, int X, int Z,
                           int exy, int ez, int e3) {
    FakeScan sd{rec, cnt, 0};
    Geom g;
    std::memset(&g, 0, sizeof g);
    g.X = X; g.Z = Z; g.exy = exy; g.ez = ez; g.Xe = X + 2 * exy; g.Ze = Z + 2 * ez;
    for (int c = 0; c < C; c++) {
        if (e3) {
            const int XeXe = g.Xe * g.Xe;
            NbAcc res;
            if (!run_lanes(4, [&](int sub) {
E3_BODY
                if (sub == 0) res = a;
            }))
                return 1;
            res.store(&rec[c]);
        } else {
GENERIC_BODY
        }
    }
    return 0;
}
}  // namespace gvom
"""


def _between(src, start, end, include_end=True, after=None):
    a = src.index(start, src.index(after) if after else 0)
    b = src.index(end, a)
    return src[a:b + (len(end) if include_end else 0)]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(os.path.join(CSRC, "k_process.cu")).read()
    head = _between(src, "struct __align__(16) CellMom {", "// the record of an in-grid cell's voxel", False)
    nbacc = _between(src, "struct NbAcc {", "\n};\n")
    small = _between(src, "    if (mine) {\n", "        store_min_h(sd, ci, mh);\n    }\n")
    warp = _between(src, "        const int qo = hq_off[q], qn = hq_n[q];\n",
                    "            store_min_h(sd, hq_rec[q], mh);\n        }\n")
    e3 = _between(src, "            NbAcc a;\n            a.init();\n            if (c < C) {\n",
                  "            if (sub == 0) a.merge(o);\n", after="k_voxel_stats(const ProcessConst pc")
    gen = _between(src, "            VoxelRec *r = &sd.rec[c];\n", "            a.store(r);\n",
                   after="k_voxel_stats(const ProcessConst pc")
    driver = (DRIVER.replace("SMALL_BODY", small).replace("WARP_BODY", warp)
              .replace("E3_BODY", e3).replace("GENERIC_BODY", gen))
    d = tmp_path_factory.mktemp("moments")
    cpp = d / "moments_host.cpp"
    cpp.write_text(PRELUDE + head + nbacc + driver)
    so = d / "libmoments.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(HERE, "cpp", "host_cuda"), "-I", CSRC, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.cell_moments.argtypes = [P, C.c_int, C.c_int, C.c_int, P]
    lib.voxel_stats.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    return lib


MOM = np.dtype([("m", "<f4", 3), ("n", "<f4"), ("c", "<f4", 6), ("min_h", "<f4"), ("pad", "<f4")])
REC = np.dtype([("mean", "<f4", 3), ("cov", "<f4", 6), ("count", "<f4"), ("hit", "<i4"), ("total", "<i4"),
                ("min_h", "<f4"), ("aux", "<i4", 3)])
assert MOM.itemsize == 48 and REC.itemsize == 64
BELOW_ONE = np.float32(np.nextafter(np.float32(1), np.float32(0)))


def _cell_points(rng, kind, n):
    """n in-cell fractions (float32, each in [0, 1)) of the named shape."""
    if kind == "uniform":
        f = rng.random((n, 3))
    elif kind == "spot":  # a tight cluster anywhere in the cell, spread 1e-2 .. 1e-7
        f = rng.random(3) + rng.normal(size=(n, 3)) * 10.0 ** rng.uniform(-7, -2)
    elif kind == "same":  # every point on one spot
        f = np.repeat(rng.random((1, 3)), n, axis=0)
    elif kind == "faces":  # on the cell's faces: 0 or just below 1 in each coordinate
        f = np.where(rng.random((n, 3)) < 0.5, 0.0, BELOW_ONE)
    elif kind == "plane":  # a level plane, as ground returns
        f = rng.random((n, 3))
        f[:, 2] = rng.random()
    elif kind == "line":  # a vertical line, as a pole
        f = np.repeat(rng.random((1, 3)), n, axis=0)
        f[:, 2] = rng.random(n)
    elif kind == "two":  # two far clusters
        f = np.where(rng.random((n, 1)) < 0.5, 0.02, 0.97) + rng.normal(size=(n, 3)) * 1e-3
    else:
        raise ValueError(kind)
    return np.clip(f, 0.0, BELOW_ONE).astype(np.float32)


KINDS = ("uniform", "spot", "same", "faces", "plane", "line", "two")


def _scene(rng, X, Z, exy, ez):
    """Points of every cell of the grid extended by the eigen distances:
    per cell a count (empty, small, warp-sized, up to 20,000) and a shape."""
    Xe, Ze = X + 2 * exy, Z + 2 * ez
    cells = []
    for e in range(Xe * Xe * Ze):
        u = rng.random()
        if u < 0.45:
            n = 0
        elif u < 0.75:
            n = int(rng.integers(1, 17))
        elif u < 0.95:
            n = int(rng.integers(17, 2000))
        else:
            n = int(rng.integers(5000, 20001))
        cells.append(_cell_points(rng, KINDS[int(rng.integers(len(KINDS)))], n) if n else np.zeros((0, 3), np.float32))
    return cells


def _layout(cells):
    """The kernels' inputs: points sorted by cell, the dense count words
    (group offset << 32 | points) over the extended grid."""
    counts = np.array([len(c) for c in cells], np.int64)
    off = np.concatenate([[0], np.cumsum(counts)[:-1]])
    sorted_pts = np.zeros((max(int(counts.sum()), 1), 4), np.float32)
    for c, o in zip(cells, off):
        sorted_pts[o:o + len(c), :3] = c
    cnt = ((off.astype(np.uint64) << np.uint64(32)) | counts.astype(np.uint64)).astype(np.uint64)
    return sorted_pts, cnt, off, counts


def _truth(cells, X, Z, exy, ez, x, y, z):
    """float64 mean, covariance (divided by the count, as __normalize_covariance)
    and count of the points in the voxel's neighbourhood, in voxel units from
    the voxel's corner, and its own cell's lowest height fraction."""
    Xe = X + 2 * exy
    ls = []
    for dz in range(-ez, ez + 1):
        for dy in range(-exy, exy + 1):
            for dx in range(-exy, exy + 1):
                e = (x + exy + dx) + (y + exy + dy) * Xe + (z + ez + dz) * Xe * Xe
                if len(cells[e]):
                    ls.append(cells[e].astype(np.float64) + np.array([dx, dy, dz], np.float64))
    L = np.concatenate(ls)
    m = L.mean(axis=0)
    d = L - m
    cov = np.array([np.mean(d[:, i] * d[:, j]) for i, j in ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))])
    own = cells[(x + exy) + (y + exy) * Xe + (z + ez) * Xe * Xe]
    return m, cov, len(L), float(own[:, 2].min())


def _close(a, b):
    return np.abs(np.asarray(a, np.float64) - b) <= STAT_ATOL + STAT_RTOL * np.abs(b)


def _moments(lib, sorted_pts, off, counts, warp_all=None):
    mom = np.zeros(sorted_pts.shape[0], MOM)
    limit = lib.small_cell_limit()
    for o, n in zip(off, counts):
        if n == 0:
            continue
        warp = int(n > limit) if warp_all is None else warp_all
        assert lib.cell_moments(sorted_pts.ctypes.data, int(o), int(n), warp, mom.ctypes.data) == 0
    return mom


@pytest.mark.parametrize("warp", [0, 1])
def test_cell_moments_both_forms(lib, warp):
    """Every cell through the one-thread body and through the one-warp body:
    count, lowest height exact; mean and second moments against float64."""
    rng = np.random.default_rng(51 + warp)
    cells = _scene(rng, 4, 3, 1, 1)
    sorted_pts, cnt, off, counts = _layout(cells)
    mom = _moments(lib, sorted_pts, off, counts, warp_all=warp)
    checked = 0
    for c, o, n in zip(cells, off, counts):
        if n == 0:
            continue
        r = mom[o]
        f = c.astype(np.float64)
        m = f.mean(axis=0)
        d = f - m
        c2 = np.array([np.mean(d[:, i] * d[:, j]) for i, j in ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))])
        assert r["n"] == n and r["min_h"] == np.float32(c[:, 2].min())
        assert _close(r["m"] + 0.5, m).all(), (n, r["m"] + 0.5, m)
        assert _close(r["c"] / np.float64(n), c2).all(), (n, r["c"] / n, c2)
        checked += 1
    assert checked > 50


@pytest.mark.parametrize("exy,ez,e3", [(1, 1, 1), (1, 1, 0), (2, 1, 0), (1, 2, 0), (0, 0, 0)])
def test_voxel_stats_against_float64(lib, exy, ez, e3):
    """Neighbourhood mean, covariance and count of every occupied voxel from
    the kernel's cell moments (one-thread or one-warp by the cell's size) and
    its neighbourhood body, against float64 over the same points."""
    X, Z = 5, 4
    rng = np.random.default_rng(100 * exy + 10 * ez + e3)
    cells = _scene(rng, X, Z, exy, ez)
    sorted_pts, cnt, off, counts = _layout(cells)
    mom = _moments(lib, sorted_pts, off, counts)
    Xe = X + 2 * exy
    vox = [(x, y, z) for z in range(Z) for y in range(X) for x in range(X)
           if counts[(x + exy) + (y + exy) * Xe + (z + ez) * Xe * Xe]]
    rec = np.zeros(len(vox), REC)
    for i, (x, y, z) in enumerate(vox):
        rec[i]["aux"][0] = x + y * X + z * X * X
    assert lib.voxel_stats(cnt.ctypes.data, mom.ctypes.data, rec.ctypes.data, len(vox), X, Z, exy, ez, e3) == 0
    worst = 0.0
    for i, (x, y, z) in enumerate(vox):
        m, cov, n, _ = _truth(cells, X, Z, exy, ez, x, y, z)
        r = rec[i]
        assert r["count"] == n
        assert _close(r["mean"], m).all(), ((x, y, z), r["mean"], m)
        assert _close(r["cov"], cov).all(), ((x, y, z), r["cov"], cov)
        worst = max(worst, float(np.max(np.abs(r["cov"] - cov) / (STAT_ATOL + STAT_RTOL * np.abs(cov)))))
    assert len(vox) > 20 and worst <= 1.0


def test_four_lane_and_one_thread_bodies_agree(lib):
    """The four-lane order ((0 + 1) + (2 + 3) of seven-cell runs) and the
    one-thread cell-by-cell order give the same counts and statistics within
    float32 rounding of each other."""
    X, Z = 5, 4
    rng = np.random.default_rng(7)
    cells = _scene(rng, X, Z, 1, 1)
    sorted_pts, cnt, off, counts = _layout(cells)
    mom = _moments(lib, sorted_pts, off, counts)
    vox = [(x, y, z) for z in range(Z) for y in range(X) for x in range(X)
           if counts[(x + 1) + (y + 1) * (X + 2) + (z + 1) * (X + 2) ** 2]]
    out = []
    for e3 in (1, 0):
        rec = np.zeros(len(vox), REC)
        for i, (x, y, z) in enumerate(vox):
            rec[i]["aux"][0] = x + y * X + z * X * X
        assert lib.voxel_stats(cnt.ctypes.data, mom.ctypes.data, rec.ctypes.data, len(vox), X, Z, 1, 1, e3) == 0
        out.append(rec)
    a, b = out
    assert np.array_equal(a["count"], b["count"])
    np.testing.assert_allclose(a["mean"], b["mean"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(a["cov"], b["cov"], rtol=1e-4, atol=1e-6)
