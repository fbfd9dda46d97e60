"""The index merge of k_merge (gvom_gb300/csrc/k_combine.cu: ring slots in
slot order, then the previous combined map with the clearing rule; pass
counts added), compiled for the host from the kernel source and run column
by column, against the oracle's combined index map after every combine of
every golden fixture (scripts/gvom.py:242-298, 1009-1063): equal."""
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
KZC = 16  # z planes per thread


def _kernel_merge_block():
    src = open(os.path.join(CSRC, "k_combine.cu")).read()
    k = src.index("__global__ void __launch_bounds__(256) k_merge(")
    a = src.index("    int occ[kZC], cnt[kZC];", k)
    end = "    for (int k = 0; k < kZC; k++) cmb[k] = occ[k] >= 0 ? kOcc : cnt[k];\n"
    return src[a:src.index(end, a) + len(end)]


DRIVER = r"""
using namespace gvom;
constexpr int kOccHost = 0x7fffffff;
extern "C" int merge_all(const int *const *idx, const int *dx, const int *dy, const int *dz, const int *is_last,
                         int nsrc, int X, int Z, int *out) {
    constexpr int NSRC = kMaxSources;
    constexpr int kZC = %(kzc)d;
    constexpr int kOcc = kOccHost;
    if (nsrc > NSRC) return 1;
    MergeParams mp;
    std::memset(&mp, 0, sizeof mp);
    mp.g.X = X; mp.g.Z = Z; mp.nsrc = nsrc;
    for (int s = 0; s < nsrc; s++) {
        mp.src[s].idx = idx[s]; mp.src[s].dx = dx[s]; mp.src[s].dy = dy[s]; mp.src[s].dz = dz[s];
        mp.src[s].is_last = is_last[s];
    }
    const int plane = X * X;
    for (int z0 = 0; z0 < Z; z0 += kZC)
        for (int y = 0; y < X; y++)
            for (int x = 0; x < X; x++) {
                const bool col = true;
%(block)s
                for (int k = 0; k < kZC && z0 + k < Z; k++) {
                    const int vid = x + y * X + (z0 + k) * plane;
                    out[vid] = cmb[k] == kOcc ? vid : cmb[k];
                }
            }
    return 0;
}
"""


@pytest.fixture(scope="module")
def merge_lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("merge")
    cpp = d / "merge_host.cpp"
    cpp.write_text("#include <algorithm>\nusing std::max; using std::min;\n"
                   "#define __ldg(p) (*(p))\n"
                   '#include "gvom_internal.cuh"\n' + DRIVER % {"kzc": KZC, "block": _kernel_merge_block()})
    so = d / "libmerge.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(HERE, "cpp", "host_cuda"),
                    "-I", CSRC, "-o", str(so), str(cpp)], check=True)
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.merge_all.argtypes = [P, P, P, P, P, C.c_int, C.c_int, C.c_int, P]
    return lib


@pytest.mark.parametrize("name", golden_files())
def test_kernel_index_merge_equals_oracle(merge_lib, name):
    fx = load(os.path.join(GOLDEN, name))
    p = params_of(fx)
    xy, zr, X, Z, B = p[0], p[1], p[2], p[3], p[4]
    o = OracleGvom(*p)
    prev = None  # (index map, origin) of the previous combined map
    for op in ops_of(fx):
        if op[0] == "P":
            o.Process_pointcloud(*op[2:])
            continue
        out = o.combine_maps()
        co = np.round(np.asarray(out[0]) / np.array([xy, xy, zr])).astype(np.int64)
        srcs = []
        for s in range(B):
            st = o.slot_state(s)
            if st is None:  # never written: contributes nothing
                continue
            od = np.round(np.asarray(st["origin"], np.float64)).astype(np.int64)
            srcs.append((np.ascontiguousarray(np.asarray(st["index"], np.int32).reshape(-1)), co - od, 0))
        if prev is not None:
            srcs.append((prev[0], co - prev[1], 1))
        keep = [s[0] for s in srcs]
        ptrs = (C.c_void_p * len(srcs))(*[s[0].ctypes.data for s in srcs])
        ar = lambda v: np.ascontiguousarray(np.array(v, np.int32))  # noqa: E731
        dx, dy, dz = ar([s[1][0] for s in srcs]), ar([s[1][1] for s in srcs]), ar([s[1][2] for s in srcs])
        last = ar([s[2] for s in srcs])
        got = np.empty(X * X * Z, np.int32)
        assert merge_lib.merge_all(ptrs, dx.ctypes.data, dy.ctypes.data, dz.ctypes.data, last.ctypes.data,
                                   len(srcs), X, Z, got.ctypes.data) == 0
        ref = np.asarray(o.combined_state()["index"], np.int32).reshape(-1)
        np.testing.assert_array_equal(got >= 0, ref >= 0, f"{name} occupied set")
        np.testing.assert_array_equal(np.where(ref >= 0, 0, got), np.where(ref >= 0, 0, ref), f"{name} free map")
        prev = (ref.copy(), co)
        del keep


def _reference_merge(srcs, X, Z):
    """__combine_indices / __combine_old_indices (scripts/gvom.py:1009-1063)
    restated in numpy, source after source: a voxel becomes occupied (True)
    where a source holds an occupied entry and the combined value is not
    occupied yet (the previous combined map only while that value is
    >= -11); a free entry o <= -2 adds o + 1 while the value is not
    occupied.  Returns (occupied mask, combined values)."""
    V = X * X * Z
    c = np.full(V, -1, np.int64)
    occ = np.zeros(V, bool)
    z, y, x = np.meshgrid(np.arange(Z), np.arange(X), np.arange(X), indexing="ij")
    x, y, z = x.reshape(-1), y.reshape(-1), z.reshape(-1)
    for idx, (dx, dy, dz), last in srcs:
        xs, ys, zs = x + dx, y + dy, z + dz
        inb = (xs >= 0) & (xs < X) & (ys >= 0) & (ys < X) & (zs >= 0) & (zs < Z)
        o = np.full(V, -1, np.int64)
        o[inb] = idx[(xs + ys * X + zs * X * X)[inb]]
        free = ~occ
        take = free & (o >= 0) & ((c >= -11) if last else True)
        add = free & ~take & (o < -1)
        occ |= take
        c[add] += o[add] + 1
    return occ, c


@pytest.mark.parametrize("seed", range(6))
def test_kernel_index_merge_random_rings(merge_lib, seed):
    """Random rings of 1-16 slot index maps (occupied entries, unknown ones
    and free counts around the -11 return threshold) plus, half the time, a
    previous combined map, with random ego shifts: the kernel's merge block
    (AND for occupancy, clamped sum for the pass count) against the
    reference's rule restated source by source."""
    rng = np.random.default_rng(100 + seed)
    for _ in range(4):
        X, Z = int(rng.integers(5, 13)), int(rng.integers(KZC // 2, 2 * KZC + 3))
        V = X * X * Z
        nsl = int(rng.integers(1, 17))
        srcs = []
        for s in range(nsl + int(rng.integers(0, 2))):
            u = rng.random(V)
            idx = np.where(u < 0.15, rng.integers(0, 1000, V),
                           np.where(u < 0.55, -1, -rng.integers(2, 9, V))).astype(np.int32)
            shift = tuple(int(v) for v in rng.integers(-3, 4, 3))
            srcs.append((np.ascontiguousarray(idx), shift, 1 if s == nsl else 0))
        ptrs = (C.c_void_p * len(srcs))(*[s[0].ctypes.data for s in srcs])
        ar = lambda v: np.ascontiguousarray(np.array(v, np.int32))  # noqa: E731
        dx, dy, dz = (ar([s[1][a] for s in srcs]) for a in range(3))
        last = ar([s[2] for s in srcs])
        got = np.empty(V, np.int32)
        assert merge_lib.merge_all(ptrs, dx.ctypes.data, dy.ctypes.data, dz.ctypes.data, last.ctypes.data,
                                   len(srcs), X, Z, got.ctypes.data) == 0
        occ, c = _reference_merge([(s[0].astype(np.int64), s[1], s[2]) for s in srcs], X, Z)
        np.testing.assert_array_equal(got >= 0, occ)
        np.testing.assert_array_equal(got[~occ], c[~occ])
        assert occ.any() and (c[~occ] < -11).any()  # both branches of the return rule reached
