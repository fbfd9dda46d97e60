"""The whole process launch sequence (launch_process in
gvom_gb300/csrc/k_process.cu: k_voxelize_trace, k_assign, k_scatter,
k_cell_moments, k_voxel_stats, k_cleanup, with the launcher's own grids),
compiled unchanged for the host and run block by block with one fiber per
CUDA thread (tests/cpp/host_cuda/block_threads.h: block barriers, warp
shuffles, shared memory, atomics).  Scan descriptors are filled the way the
library's host code fills them (prepare_scans in
gvom_gb300/csrc/gvom_capi.cu).  On every scan of every golden fixture the
slot equals the oracle's: occupied set, pass-through counts, hit, total and
minimum height exactly, the scan counters exactly, mean / covariance /
count within the parity tolerance; and the cell words are back to zero.
Batches of scans (one launch set for up to 16 scans) give the same slots as
the scans one at a time."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN
from hostbuild import PRELUDE, compile_units
from oracle.canonical import canonical_state
from oracle.oracle import OracleGvom
from replay import compare_slot, load, ops_of, params_of

SOURCE = r"""
#include "k_process.cu"
#include "host_scan.h"

using namespace gvom;

struct HostScan {
    const void *pts;
    long long n, stride;
    int tmode;         // 0 none, 1 float32, 2 float64 transform
    double ego[3];
    double T[12];      // rows 0..2 of the 4x4
};

// One process call over k scans (prepare_scans + launch_scans of the
// library): idx[i] (V ints) and rec[i] (rec_cap records) are scan i's slot,
// ctr[i] its counters.  Returns the number of cell words left non-zero.
extern "C" long long process_scans(const HostScan *scans, int k, int dtype, double xy_res, double z_res, int X,
                                   int Z, int exy, int ez, double min_distance, int num_sms, int pts_block,
                                   int *const *idx, VoxelRec *const *rec, long long rec_cap, ScanCounters *ctr) {
    const ProcessConst pc = host_scan::process_const(X, Z, exy, ez, xy_res, z_res, min_distance, k, num_sms);
    const Geom &g = pc.g;
    std::vector<ScanDesc> table(k);
    std::vector<std::vector<unsigned long long>> cnt(k, std::vector<unsigned long long>(g.Vext, 0ull));
    long long base = 0, max_n = 0;
    int block = 0;
    for (int i = 0; i < k; i++) {
        const HostScan &s = scans[i];
        ScanDesc &d = table[i];
        host_scan::scan_desc(d, pc, s.pts, s.n, s.stride, s.tmode, s.ego, s.T);
        d.block_begin = block;
        d.nblocks = (int)((s.n + pts_block - 1) / pts_block);
        block += d.nblocks;
        d.pt_base = base;
        base += s.n;
        max_n = std::max(max_n, s.n);
        d.cnt = cnt[i].data();
        d.idx = idx[i];
        d.rec = rec[i];
        d.rec_cap = rec_cap;
        d.ctr = &ctr[i];
        std::memset(&ctr[i], 0, sizeof(ScanCounters));
        for (long long v = 0; v < g.V; v++) idx[i][v] = -1;  // the slot's index map before the scan
    }
    const long long np = std::max<long long>(base, 1);
    std::vector<float4> prec(np), sorted(np);
    std::vector<int> prank(np);
    std::vector<unsigned char> mom((size_t)np * kCellMomBytes);
    const cudaError_t e = launch_process(pc, table.data(), k, std::max(block, 1), (int)std::min<long long>(max_n, g.V),
                                         dtype, prec.data(), prank.data(), sorted.data(), mom.data(), nullptr, nullptr,
                                         pts_block, nullptr, nullptr, 0, false);
    if (e != cudaSuccess) return -1;
    long long dirty = 0;
    for (int i = 0; i < k; i++)
        for (long long c = 0; c < g.Vext; c++) dirty += cnt[i][c] != 0ull;
    return dirty;
}
"""


class HostScan(C.Structure):
    _fields_ = [("pts", C.c_void_p), ("n", C.c_longlong), ("stride", C.c_longlong), ("tmode", C.c_int),
                ("ego", C.c_double * 3), ("T", C.c_double * 12)]


REC = np.dtype([("mean", "<f4", 3), ("cov", "<f4", 6), ("count", "<f4"), ("hit", "<i4"), ("total", "<i4"),
                ("min_h", "<f4"), ("aux", "<i4", 3)])
CTR = np.dtype([("C", "<i4"), ("pts", "<i4"), ("overflow", "<i4"), ("pad", "<i4"), ("valid", "<u8"),
                ("hits", "<u8"), ("steps", "<u8")])
assert REC.itemsize == 64 and CTR.itemsize == 40


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("process")
    so = compile_units({"process_host.cpp": PRELUDE + SOURCE}, d, "libprocess.so")
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.process_scans.restype = C.c_longlong
    lib.process_scans.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_double, C.c_int, C.c_int, P, P, C.c_longlong, P]
    return lib


def _host_scan(pts, ego, T):
    s = HostScan()
    s.pts = pts.ctypes.data
    s.n = pts.shape[0]
    s.stride = pts.shape[1]
    s.tmode = 0 if T is None else (1 if np.asarray(T).dtype == np.float32 else 2)
    s.ego[:] = [float(v) for v in np.asarray(ego, np.float64).reshape(3)]
    if T is not None:
        s.T[:] = np.asarray(T, np.float64).reshape(4, 4)[:3].reshape(-1).tolist()
    return s


def _run(lib, p, scans, pts_block=256, num_sms=2):
    """Slots (index map, records, counters) of one process call over `scans`
    ((points, ego, T) with points of one dtype)."""
    X, Z = int(p[2]), int(p[3])
    V = X * X * Z
    k = len(scans)
    arr = (HostScan * k)(*[_host_scan(*s) for s in scans])
    cap = max(max(s[0].shape[0] for s in scans), 1)
    idx = [np.empty(V, np.int32) for _ in range(k)]
    rec = [np.zeros(cap, REC) for _ in range(k)]
    ctr = np.zeros(k, CTR)
    ip = (C.c_void_p * k)(*[a.ctypes.data for a in idx])
    rp = (C.c_void_p * k)(*[a.ctypes.data for a in rec])
    dtype = 0 if scans[0][0].dtype == np.float32 else 1
    dirty = lib.process_scans(arr, k, dtype, p[0], p[1], X, Z, int(p[12]), int(p[13]), p[5], num_sms, pts_block,
                              ip, rp, cap, ctr.ctypes.data)
    assert dirty == 0, f"{dirty} cell words left non-zero"
    out = []
    for i in range(k):
        c = int(ctr[i]["C"])
        assert ctr[i]["overflow"] == 0
        r = rec[i][:c]
        metrics = np.concatenate([r["mean"], r["cov"], r["count"][:, None]], axis=1).astype(np.float64)
        st = dict(index=idx[i], hit=r["hit"].copy(), total=r["total"].copy(), min_h=r["min_h"].copy(),
                  metrics=metrics)
        assert np.array_equal(r["aux"][:, 0], np.flatnonzero(idx[i] >= 0)[np.argsort(idx[i][idx[i] >= 0])]), \
            "record voxel ids"
        out.append((st, ctr[i]))
    return out


def _oracle_slots(fx):
    """Per process op: (points, ego, T) and the oracle's slot and scan counters."""
    p = params_of(fx)
    o = OracleGvom(*p)
    res = []
    for op in ops_of(fx):
        if op[0] != "P":
            continue
        _, pi, pts, ego, T = op
        pts = np.ascontiguousarray(pts)
        o.Process_pointcloud(pts, ego, T)
        _, last = o.ring_state()
        res.append(((pts, ego, T), o.slot_state(last), o.last_process_stats(), pi))
    return p, res


# fixtures of each kind (float32 / float64 points and transforms, voxel
# boundaries, rays, eigen distances (2, 0) and (1, 2), the 128 x 128 x 32
# grid); every fixture also replays through tests/test_pipeline_host.py and
# tests/test_capi_host.py
PROCESS_FIXTURES = ["kat_boundaries.npz", "kat_rays.npz", "synth_f64T_veg.npz", "synth_f64pts_eig20.npz",
                    "synth_aniso_z.npz", "small_32x512.npz"]


@pytest.mark.parametrize("name", PROCESS_FIXTURES)
def test_process_kernels_equal_oracle(lib, name):
    """Every scan of the fixture, one scan per call."""
    p, res = _oracle_slots(load(os.path.join(GOLDEN, name)))
    for scan, ref, stats, pi in res:
        (got, ctr), = _run(lib, p, [scan])
        what = f"{name} scan {pi}"
        compare_slot(canonical_state(got), canonical_state(ref), what)
        assert (int(ctr["valid"]), int(ctr["hits"]), int(ctr["steps"])) == \
            (stats["valid_points"], stats["hits"], stats["ray_steps"]), what


@pytest.mark.parametrize("name,k,pts_block", [("synth_ring16.npz", 16, 256), ("synth_f64T_veg.npz", 5, 128),
                                              ("synth_longrun.npz", 3, 256)])
def test_batched_launch_equals_oracle(lib, name, k, pts_block):
    """k scans of a fixture in one launch set (the batched form's scan table:
    the 4-scan and 16-scan launch templates, 128- and 256-thread blocks):
    every slot equals the oracle's slot of that scan."""
    p, res = _oracle_slots(load(os.path.join(GOLDEN, name)))
    res = res[:k]
    scans = [r[0] for r in res]
    got = _run(lib, p, scans, pts_block=pts_block, num_sms=3)
    for (st, ctr), (_, ref, stats, pi) in zip(got, res):
        what = f"{name} batched scan {pi}"
        compare_slot(canonical_state(st), canonical_state(ref), what)
        assert (int(ctr["valid"]), int(ctr["hits"]), int(ctr["steps"])) == \
            (stats["valid_points"], stats["hits"], stats["ray_steps"]), what
