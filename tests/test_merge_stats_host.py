"""The statistics merge (merge_counts and merge_voxel in
gvom_gb300/csrc/k_combine.cu: hit / total sums, minimum height, the float32
Chan merge of mean, covariance and count in source order, and the
eigen-solve), compiled for the host from the kernel source and run for every
occupied combined voxel of every golden fixture on the oracle's slot and
previous combined records: counts and minimum heights equal the oracle's,
statistics and eigenvalues within the parity tolerance -- including the
long run, where the float32 merge is applied again at every combine."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from oracle.canonical import canonical_state
from oracle.oracle import OracleGvom
from replay import assert_eigen, assert_exact, assert_stats, load, ops_of, params_of

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc")

PRELUDE = r"""
#include <algorithm>
#include <cmath>
using std::max; using std::min; using std::copysign;
template <class T> static inline T __ldg(const T *p) { return *p; }
static inline float __frcp_rn(float x) { return 1.0f / x; }
#include "gvom_internal.cuh"
static inline float __fdividef(float a, float b) { return a / b; }
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
namespace gvom {
"""

DRIVER = r"""
}  // namespace gvom
using namespace gvom;
extern "C" int merge_voxels(const int *const *idx, const VoxelRec *const *rec, const int *dx, const int *dy,
                            const int *dz, const int *is_last, int nsrc, int X, int Z, const int *vids, int nv,
                            VoxelRec *out) {
    if (nsrc > kMaxSources) return 1;
    MergeParams mp;
    std::memset(&mp, 0, sizeof mp);
    mp.g.X = X; mp.g.Z = Z; mp.nsrc = nsrc;
    for (int s = 0; s < nsrc; s++) {
        mp.src[s].idx = idx[s]; mp.src[s].rec = rec[s];
        mp.src[s].dx = dx[s]; mp.src[s].dy = dy[s]; mp.src[s].dz = dz[s]; mp.src[s].is_last = is_last[s];
    }
    mp.out_rec = out;
    for (int i = 0; i < nv; i++) {
        merge_counts<kMaxSources>(mp, vids[i]);
        merge_voxel<kMaxSources>(mp, vids[i]);
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def stats_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = open(os.path.join(CSRC, "k_combine.cu")).read()
    a = src.index("__device__ __forceinline__ void jacobi_rot(")
    b = src.index("// k_merge: every thread decides")
    d = tmp_path_factory.mktemp("mstats")
    cpp = d / "merge_stats_host.cpp"
    cpp.write_text(PRELUDE + src[a:b] + DRIVER)
    so = d / "libmstats.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(HERE, "cpp", "host_cuda"), "-I", CSRC, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.merge_voxels.argtypes = [P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, P, C.c_int, P]
    return lib


def _records(st):
    """VoxelRec rows (16 float32: mean 3, cov 6, count, hit, total as int bits, min_h, aux 3) of a state."""
    m = np.asarray(st["metrics"], np.float64)
    n = m.shape[0]
    rec = np.zeros((max(n, 1), 16), np.float32)
    rec[:n, :10] = m[:, :10].astype(np.float32)
    rec[:n, 10] = np.asarray(st["hit"], np.int32).view(np.float32)
    rec[:n, 11] = np.asarray(st["total"], np.int32).view(np.float32)
    rec[:n, 12] = np.asarray(st["min_h"], np.float32)[:n]
    return np.ascontiguousarray(rec)


@pytest.mark.parametrize("name", golden_files())
def test_kernel_statistics_merge_within_tolerance(stats_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    xy, zr, X, Z, B = p[0], p[1], p[2], p[3], p[4]
    V = X * X * Z
    o = OracleGvom(*p)
    prev = None
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        out = o.combine_maps()
        co = np.round(np.asarray(out[0]) / np.array([xy, xy, zr])).astype(np.int64)
        srcs = []
        for s in range(B):
            st = o.slot_state(s)
            if st is None:
                continue
            od = np.round(np.asarray(st["origin"], np.float64)).astype(np.int64)
            srcs.append((np.ascontiguousarray(np.asarray(st["index"], np.int32).reshape(-1)), _records(st), co - od, 0))
        if prev is not None:
            srcs.append((prev[0], prev[1], co - prev[2], 1))
        cst = o.combined_state()
        cidx = np.asarray(cst["index"], np.int32).reshape(-1)
        vids = np.ascontiguousarray(np.flatnonzero(cidx >= 0).astype(np.int32))
        got = np.zeros((V, 16), np.float32)
        ar = lambda v: np.ascontiguousarray(np.array(v, np.int32))  # noqa: E731
        iptr = (C.c_void_p * len(srcs))(*[s[0].ctypes.data for s in srcs])
        rptr = (C.c_void_p * len(srcs))(*[s[1].ctypes.data for s in srcs])
        dx, dy, dz = ar([s[2][0] for s in srcs]), ar([s[2][1] for s in srcs]), ar([s[2][2] for s in srcs])
        last = ar([s[3] for s in srcs])
        assert stats_lib.merge_voxels(iptr, rptr, dx.ctypes.data, dy.ctypes.data, dz.ctypes.data, last.ctypes.data,
                                      len(srcs), X, Z, vids.ctypes.data, len(vids), got.ctypes.data) == 0
        can = canonical_state(cst)  # canonical order = ascending voxel id = vids
        g = got[vids]
        assert_exact(g[:, 10].view(np.int32), can["hit"], f"{name} hit")
        assert_exact(g[:, 11].view(np.int32), can["total"], f"{name} total")
        assert_exact(g[:, 12], np.asarray(can["min_h"], np.float32), f"{name} min height")
        assert_exact(g[:, 9], np.asarray(can["metrics"])[:, 9].astype(np.float32), f"{name} count")
        assert_stats(g[:, :9], np.asarray(can["metrics"])[:, :9], f"{name} mean / covariance")
        assert_eigen(g[:, 13:16], can["eigen"], f"{name} eigenvalues")
        prev = (np.ascontiguousarray(cidx.copy()), _records(cst), co)
