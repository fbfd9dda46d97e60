"""The library's scan->map path end to end on the CPU: every process and
combine kernel (gvom_gb300/csrc/k_process.cu, k_combine.cu) compiled
unchanged for the host and launched through the library's own launchers
(launch_process, launch_combine), each block run with one fiber per CUDA
thread (tests/cpp/host_cuda/block_threads.h).  A small host mapper
keeps what the library's instance keeps -- the ring of slots, the
double-buffered combined map addressed by voxel id, the 2-D maps -- and
fills the launch parameters as prepare_scans / prepare_combine in
gvom_gb300/csrc/gvom_capi.cu do.  It is replayed through every golden fixture
with the comparison the GPU parity tests use (replay.replay_and_compare):
every slot, every combined map with its eigenvalues, every combine's maps
and the three debug exports, against the outputs of the reference
itself."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, golden_files
from hostbuild import CSRC, PRELUDE, compile_units, host_source
from oracle.canonical import canonical_state
from oracle.oracle import OracleGvom
from replay import compare_slot, load, params_of, replay_and_compare
# the GPU parity tests' own drivers (a mapper and the oracle side by side)
from test_parity_gpu import _compare_runs, _run_both

MAPPER = r"""
#include "host_scan.h"
#include <vector>

using namespace gvom;

namespace {

struct Slot {
    std::vector<int> idx;
    std::vector<VoxelRec> rec;
    int C = 0;
    double od[3] = {0, 0, 0};
    bool valid = false;
};

// what a library instance keeps (gvom_create in gvom_capi.cu), in host memory
struct HostMap {
    double p[14];  // the constructor's parameters, in order
    Geom g;
    int B;
    int buffer_index = 0, last_buffer_index = 0;
    std::vector<Slot> slots;
    std::vector<int> cidx[2], occ_list[2];
    std::vector<VoxelRec> crec[2];
    std::vector<int2> colinfo[2];
    int combC[2] = {0, 0};
    double cod[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int cur = 0;
    bool have_comb = false;
    std::vector<double> height, inferred, slope_x, slope_y, guess;
    std::vector<int> pos_density, zlow;
    std::vector<float> mlow;
    std::vector<double> out;  // roughness | positive | negative | visibility, as the device block
    double ego[3] = {0, 0, 0};
    long long last_stats[3] = {0, 0, 0};  // the last scan's valid points, hits, ray steps
    Tuning tun = kDefaultTuning;
    int num_sms = 2;
    double *rough() { return out.data(); }
    int *pos() { return reinterpret_cast<int *>(out.data() + (size_t)g.X * g.X); }
    int *neg() { return pos() + (size_t)g.X * g.X; }
    int *vis() { return neg() + (size_t)g.X * g.X; }
};

}  // namespace

extern "C" HostMap *hm_create(const double *params, int maps_tile, int merge_planes, int num_sms) {
    HostMap *h = new HostMap;
    for (int i = 0; i < 14; i++) h->p[i] = params[i];
    Geom &g = h->g;
    g.X = (int)params[2]; g.Z = (int)params[3]; g.exy = (int)params[12]; g.ez = (int)params[13];
    g.Xe = g.X + 2 * g.exy; g.Ze = g.Z + 2 * g.ez;
    g.V = (long long)g.X * g.X * g.Z; g.Vext = (long long)g.Xe * g.Xe * g.Ze;
    h->B = (int)params[4];
    h->slots.resize(h->B);
    const size_t X2 = (size_t)g.X * g.X;
    for (int b = 0; b < 2; b++) {
        h->cidx[b].assign(g.V, 0);
        h->occ_list[b].assign(g.V, 0);
        h->crec[b].assign(g.V, VoxelRec{});
        h->colinfo[b].assign(X2 * ((g.Z + 3) / 4), int2{0, 0});
    }
    for (auto *m : {&h->height, &h->inferred, &h->slope_x, &h->slope_y, &h->guess}) m->assign(X2, 0.0);
    h->pos_density.assign(X2, 0);
    h->zlow.assign(X2, 0);
    h->mlow.assign(X2, 0.f);
    h->out.assign((X2 * 20 + 7) / 8, 0.0);
    h->tun.maps_tile = maps_tile;
    h->tun.merge_planes = merge_planes;
    h->num_sms = num_sms;
    return h;
}

extern "C" void hm_destroy(HostMap *h) { delete h; }

// Process_pointcloud into the ring slot at buffer_index (prepare_scans,
// launch_scans, commit_scans); tdtype -1 none, 0 float32, 1 float64; T 16
// doubles
extern "C" int hm_process(HostMap *h, const void *pts, int dtype, long long n, long long stride, const double *ego,
                          const double *T, int tdtype) {
    const Geom &g = h->g;
    const ProcessConst pc = host_scan::process_const(g.X, g.Z, g.exy, g.ez, h->p[0], h->p[1], h->p[5], 1, h->num_sms);
    Slot &s = h->slots[h->buffer_index];
    s.idx.assign(g.V, -1);  // the slot's index map before the scan
    s.rec.assign(std::max<long long>(n, 1), VoxelRec{});
    std::vector<unsigned long long> cnt(g.Vext, 0ull);
    ScanCounters ctr;
    std::memset(&ctr, 0, sizeof ctr);
    double Tr[12] = {0};
    if (T)
        for (int r = 0; r < 12; r++) Tr[r] = T[r];
    ScanDesc d;
    host_scan::scan_desc(d, pc, pts, n, stride, T ? (tdtype == 0 ? 1 : 2) : 0, ego, Tr);
    d.block_begin = 0;
    d.nblocks = (int)((n + h->tun.pts_block - 1) / h->tun.pts_block);
    d.pt_base = 0;
    d.cnt = cnt.data();
    d.idx = s.idx.data();
    d.rec = s.rec.data();
    d.rec_cap = (long long)s.rec.size();
    d.ctr = &ctr;
    const long long np = std::max<long long>(n, 1);
    std::vector<float4> prec(np), sorted(np);
    std::vector<int> prank(np);
    std::vector<unsigned char> mom((size_t)np * kCellMomBytes);
    if (launch_process(pc, &d, 1, std::max(d.nblocks, 1), (int)std::min<long long>(n, g.V), dtype, prec.data(),
                       prank.data(), sorted.data(), mom.data(), nullptr, nullptr, h->tun.pts_block, nullptr, nullptr,
                       0, false) != cudaSuccess)
        return 4;
    if (ctr.overflow) return 4;
    h->last_stats[0] = (long long)ctr.valid;
    h->last_stats[1] = (long long)ctr.hits;
    h->last_stats[2] = (long long)ctr.steps;
    s.C = ctr.C;
    for (int a = 0; a < 3; a++) s.od[a] = d.od[a];
    s.valid = true;
    for (int a = 0; a < 3; a++) h->ego[a] = ego[a];
    h->last_buffer_index = h->buffer_index;
    h->buffer_index = (h->buffer_index + 1) % h->B;
    return 0;
}

// combine_maps (prepare_combine, launch_combine, commit_combine, copy_outputs)
extern "C" int hm_combine(HostMap *h, double *origin, int *pos, int *neg, double *rough, int *vis) {
    const Slot &ls = h->slots[h->last_buffer_index];
    if (!ls.valid) return 1;
    const Geom &g = h->g;
    const int nb = h->have_comb ? 1 - h->cur : 0;
    MergeParams mp;
    std::memset(&mp, 0, sizeof mp);
    mp.g = g;
    for (int a = 0; a < 3; a++) mp.co[a] = ls.od[a];
    int ns = 0;
    for (int i = 0; i < h->B; i++) {  // ring order
        const Slot &s = h->slots[i];
        if (!s.valid) continue;
        MergeSrc &m = mp.src[ns++];
        m.idx = s.idx.data();
        m.rec = s.rec.data();
        m.dx = (int)(mp.co[0] - s.od[0]);
        m.dy = (int)(mp.co[1] - s.od[1]);
        m.dz = (int)(mp.co[2] - s.od[2]);
        m.is_last = 0;
    }
    if (h->have_comb) {
        MergeSrc &m = mp.src[ns++];
        m.idx = h->cidx[h->cur].data();
        m.rec = h->crec[h->cur].data();
        m.dx = (int)(mp.co[0] - h->cod[h->cur][0]);
        m.dy = (int)(mp.co[1] - h->cod[h->cur][1]);
        m.dz = (int)(mp.co[2] - h->cod[h->cur][2]);
        m.is_last = 1;
    }
    mp.nsrc = ns;
    mp.out_idx = h->cidx[nb].data();
    mp.out_rec = h->crec[nb].data();
    mp.out_count = &h->combC[nb];
    mp.list = h->occ_list[nb].data();
    mp.num_sms = h->num_sms;
    mp.planes = h->tun.merge_planes;
    mp.stats_bpsm = h->tun.stats_bpsm;
    mp.colinfo = h->colinfo[nb].data();
    const double *p = h->p;
    ColumnParams cp;
    std::memset(&cp, 0, sizeof cp);
    cp.X = g.X;
    cp.Z = g.Z;
    cp.planes = h->tun.merge_planes;
    cp.idx = mp.out_idx;
    cp.rec = mp.out_rec;
    cp.colinfo = mp.colinfo;
    for (int a = 0; a < 3; a++) {
        cp.co[a] = mp.co[a];
        cp.ego[a] = h->ego[a];
    }
    cp.xy_res = p[0];
    cp.z_res = p[1];
    cp.robot_r2 = p[10] * p[10];
    cp.disc_h = h->ego[2] - p[11];
    cp.pos_thr = p[6];
    cp.robot_h = p[9];
    cp.pthr_v = (float)(p[6] / p[1]);
    cp.robh_v = (float)(p[9] / p[1]);
    cp.base_xf = (float)(mp.co[0] * p[0] - h->ego[0]);
    cp.base_yf = (float)(mp.co[1] * p[0] - h->ego[1]);
    cp.res_f = (float)p[0];
    cp.r2_f = (float)cp.robot_r2;
    cp.height = h->height.data();
    cp.inferred = h->inferred.data();
    cp.pos_density = h->pos_density.data();
    cp.zlow = h->zlow.data();
    cp.mlow = h->mlow.data();
    Maps2DParams m2;
    std::memset(&m2, 0, sizeof m2);
    m2.X = g.X;
    m2.xy_res = p[0];
    m2.z_res = p[1];
    m2.slope_thr = p[8];
    m2.slope_thr_f = (float)p[8];
    m2.neg_thr = p[7];
    m2.height = h->height.data();
    m2.inferred = h->inferred.data();
    m2.pos_density = h->pos_density.data();
    m2.zlow = h->zlow.data();
    m2.mlow = h->mlow.data();
    m2.slope_x = h->slope_x.data();
    m2.slope_y = h->slope_y.data();
    m2.rough = h->rough();
    m2.guess = h->guess.data();
    m2.pos = h->pos();
    m2.neg = h->neg();
    m2.vis = h->vis();
    m2.tile_cells = h->tun.maps_tile;
    h->combC[nb] = 0;
    if (launch_combine(mp, cp, m2, nullptr, nullptr) != cudaSuccess) return 4;
    for (int a = 0; a < 3; a++) h->cod[nb][a] = mp.co[a];
    h->cur = nb;
    h->have_comb = true;
    origin[0] = mp.co[0] * p[0];
    origin[1] = mp.co[1] * p[0];
    origin[2] = mp.co[2] * p[1];
    const size_t X2 = (size_t)g.X * g.X;
    std::memcpy(rough, h->rough(), X2 * 8);
    std::memcpy(pos, h->pos(), X2 * 4);
    std::memcpy(neg, h->neg(), X2 * 4);
    std::memcpy(vis, h->vis(), X2 * 4);
    return 0;
}

// gvom_last_process_stats
extern "C" void hm_last_stats(HostMap *h, long long *out) {
    for (int i = 0; i < 3; i++) out[i] = h->last_stats[i];
}

extern "C" void hm_ring_state(HostMap *h, long long *bi, long long *lbi) {
    *bi = h->buffer_index;
    *lbi = h->last_buffer_index;
}

static void unpack(const VoxelRec &v, long long c, int *hit, int *total, float *min_h, float *metrics, float *eigen) {
    hit[c] = v.hit;
    total[c] = v.total;
    min_h[c] = v.min_h;
    float *m = metrics + c * 10;
    for (int a = 0; a < 3; a++) m[a] = v.mean[a];
    for (int t = 0; t < 6; t++) m[3 + t] = v.cov[t];
    m[9] = v.count;
    if (eigen)
        for (int a = 0; a < 3; a++) eigen[c * 3 + a] = v.aux[a];
}

// gvom_slot_count / gvom_get_slot
extern "C" int hm_slot_count(HostMap *h, int slot) { return h->slots[slot].valid ? h->slots[slot].C : -1; }
extern "C" void hm_get_slot(HostMap *h, int slot, int *index, int *hit, int *total, float *min_h, float *metrics,
                            double *origin) {
    const Slot &s = h->slots[slot];
    std::memcpy(index, s.idx.data(), sizeof(int) * h->g.V);
    for (int c = 0; c < s.C; c++) unpack(s.rec[c], c, hit, total, min_h, metrics, nullptr);
    for (int a = 0; a < 3; a++) origin[a] = s.od[a];
}

// gvom_combined_count / gvom_get_combined: records in ascending voxel-id
// order, the index map renumbered to match
extern "C" int hm_combined_count(HostMap *h) {
    if (!h->have_comb) return -1;
    return h->combC[h->cur];
}
extern "C" void hm_get_combined(HostMap *h, int *index, int *hit, int *total, float *min_h, float *metrics,
                                float *eigen, double *origin) {
    const std::vector<int> &idx = h->cidx[h->cur];
    long long c = 0;
    for (long long v = 0; v < h->g.V; v++) {
        if (idx[v] >= 0) {
            unpack(h->crec[h->cur][v], c, hit, total, min_h, metrics, eigen);
            index[v] = (int)c++;
        } else {
            index[v] = idx[v];
        }
    }
    for (int a = 0; a < 3; a++) origin[a] = h->cod[h->cur][a];
}

// gvom_debug_voxel_map: per-block counts, their exclusive prefix on the
// host, then the rows in ascending voxel-id order; returns the row count
// (rows written when `out` holds `cap` rows)
extern "C" long long hm_debug_voxel_map(HostMap *h, float *out, long long cap) {
    if (!h->have_comb) return -1;
    const long long V = h->g.V;
    const int chunk = debug_chunk();
    const int nblocks = (int)((V + chunk - 1) / chunk);
    std::vector<int> offs(nblocks + 1, 0);
    if (launch_debug_count(h->cidx[h->cur].data(), V, offs.data(), nblocks, nullptr) != cudaSuccess) return -2;
    long long tot = 0;
    for (int b = 0; b < nblocks; b++) {
        const int c = offs[b];
        offs[b] = (int)tot;
        tot += c;
    }
    if (!out || tot == 0) return tot;
    DebugVoxParams p;
    std::memset(&p, 0, sizeof p);
    p.idx = h->cidx[h->cur].data();
    p.rec = h->crec[h->cur].data();
    p.block_off = offs.data();
    p.V = V;
    p.X = h->g.X;
    for (int a = 0; a < 3; a++) p.co[a] = h->cod[h->cur][a];
    p.xy_res = h->p[0];
    p.z_res = h->p[1];
    p.out = out;
    p.cap = std::min(tot, cap);
    if (launch_debug_voxels(p, nblocks, nullptr) != cudaSuccess) return -2;
    return tot;
}

// gvom_debug_height_map (out_h, X*X rows of 7) / gvom_debug_inferred_height_map (out_i, X*X rows of 3)
extern "C" int hm_debug_maps(HostMap *h, float *out_h, float *out_i) {
    if (!h->have_comb) return 1;
    DebugMapParams p;
    std::memset(&p, 0, sizeof p);
    p.X = h->g.X;
    for (int a = 0; a < 3; a++) p.co[a] = h->cod[h->cur][a];
    p.xy_res = h->p[0];
    p.z_res = h->p[1];
    p.height = h->height.data();
    p.rough = h->rough();
    p.slope_x = h->slope_x.data();
    p.slope_y = h->slope_y.data();
    p.guess = h->guess.data();
    p.out_h = out_h;
    p.out_i = out_i;
    return launch_debug_maps(p, nullptr) == cudaSuccess ? 0 : 4;
}

// gvom_get_maps
extern "C" void hm_get_maps(HostMap *h, double *height, double *inferred, double *slope_x, double *slope_y,
                            double *rough, double *guess) {
    const size_t b = (size_t)h->g.X * h->g.X * 8;
    std::memcpy(height, h->height.data(), b);
    std::memcpy(inferred, h->inferred.data(), b);
    std::memcpy(slope_x, h->slope_x.data(), b);
    std::memcpy(slope_y, h->slope_y.data(), b);
    std::memcpy(rough, h->rough(), b);
    std::memcpy(guess, h->guess.data(), b);
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("pipeline")
    comb = host_source(open(os.path.join(CSRC, "k_combine.cu")).read())
    so = compile_units({"proc.cpp": PRELUDE + '#include "k_process.cu"\n', "comb.cpp": PRELUDE + comb,
                        "mapper.cpp": PRELUDE + MAPPER}, d, "libpipeline.so")
    lib = C.CDLL(str(so))
    P = C.c_void_p
    lib.hm_create.restype = P
    lib.hm_create.argtypes = [P, C.c_int, C.c_int, C.c_int]
    lib.hm_destroy.argtypes = [P]
    lib.hm_process.argtypes = [P, P, C.c_int, C.c_longlong, C.c_longlong, P, P, C.c_int]
    lib.hm_combine.argtypes = [P, P, P, P, P, P]
    lib.hm_ring_state.argtypes = [P, P, P]
    lib.hm_last_stats.argtypes = [P, P]
    lib.hm_slot_count.argtypes = [P, C.c_int]
    lib.hm_get_slot.argtypes = [P, C.c_int, P, P, P, P, P, P]
    lib.hm_combined_count.argtypes = [P]
    lib.hm_get_combined.argtypes = [P, P, P, P, P, P, P, P]
    lib.hm_get_maps.argtypes = [P, P, P, P, P, P, P]
    lib.hm_debug_voxel_map.restype = C.c_longlong
    lib.hm_debug_voxel_map.argtypes = [P, P, C.c_longlong]
    lib.hm_debug_maps.argtypes = [P, P, P]
    return lib


def _ptr(a):
    return a.ctypes.data


class HostMapper:
    """The reference surface and the parity accessors over the host build
    (the methods replay.replay_and_compare drives)."""

    def __init__(self, lib, params, maps_tile=224, merge_planes=8, num_sms=2):
        self._l = lib
        self.params = np.asarray(params, np.float64)
        self.X, self.Z = int(params[2]), int(params[3])
        self.V = self.X * self.X * self.Z
        self._h = lib.hm_create(_ptr(self.params), maps_tile, merge_planes, num_sms)

    def close(self):
        if self._h:
            self._l.hm_destroy(self._h)
            self._h = None

    def Process_pointcloud(self, pts, ego, T=None):
        pts = np.ascontiguousarray(pts)
        e = np.ascontiguousarray(np.asarray(ego, np.float64).reshape(3))
        Td = None if T is None else np.ascontiguousarray(np.asarray(T, np.float64).reshape(4, 4))
        tdt = -1 if T is None else (0 if np.asarray(T).dtype == np.float32 else 1)
        rc = self._l.hm_process(self._h, _ptr(pts), 0 if pts.dtype == np.float32 else 1, pts.shape[0], pts.shape[1],
                                _ptr(e), None if Td is None else _ptr(Td), tdt)
        assert rc == 0, rc

    def combine_maps(self):
        X = self.X
        origin = np.zeros(3)
        pos, neg, vis = (np.empty((X, X), np.int32) for _ in range(3))
        rough = np.empty((X, X), np.float64)
        rc = self._l.hm_combine(self._h, _ptr(origin), _ptr(pos), _ptr(neg), _ptr(rough), _ptr(vis))
        if rc == 1:
            return None
        assert rc == 0, rc
        return origin, pos, neg, rough, vis

    def last_process_stats(self):
        v = np.zeros(3, np.int64)
        self._l.hm_last_stats(self._h, _ptr(v))
        return dict(valid_points=int(v[0]), hits=int(v[1]), ray_steps=int(v[2]))

    def ring_state(self):
        a, b = C.c_longlong(), C.c_longlong()
        self._l.hm_ring_state(self._h, C.byref(a), C.byref(b))
        return a.value, b.value

    def slot_state(self, slot):
        c = self._l.hm_slot_count(self._h, int(slot))
        if c < 0:
            return None
        st = dict(index=np.empty(self.V, np.int32), hit=np.empty(c, np.int32), total=np.empty(c, np.int32),
                  min_h=np.empty(c, np.float32), metrics=np.empty((c, 10), np.float32), origin=np.zeros(3))
        self._l.hm_get_slot(self._h, int(slot), *[_ptr(st[k]) for k in ("index", "hit", "total", "min_h", "metrics",
                                                                        "origin")])
        return st

    def combined_state(self):
        c = self._l.hm_combined_count(self._h)
        if c < 0:
            return None
        st = dict(index=np.empty(self.V, np.int32), hit=np.empty(c, np.int32), total=np.empty(c, np.int32),
                  min_h=np.empty(c, np.float32), metrics=np.empty((c, 10), np.float32),
                  eigen=np.empty((c, 3), np.float32), origin=np.zeros(3))
        self._l.hm_get_combined(self._h, *[_ptr(st[k]) for k in ("index", "hit", "total", "min_h", "metrics", "eigen",
                                                                 "origin")])
        return st

    def make_debug_voxel_map(self):
        n = self._l.hm_debug_voxel_map(self._h, None, 0)
        assert n >= 0, n
        out = np.zeros((n, 8), np.float32)
        if n:
            assert self._l.hm_debug_voxel_map(self._h, _ptr(out), n) == n
        return out

    def make_debug_height_map(self):
        out = np.zeros((self.X * self.X, 7), np.float32)
        assert self._l.hm_debug_maps(self._h, _ptr(out), None) == 0
        return out

    def make_debug_inferred_height_map(self):
        out = np.zeros((self.X * self.X, 3), np.float32)
        assert self._l.hm_debug_maps(self._h, None, _ptr(out)) == 0
        return out

    def maps_state(self):
        X = self.X
        keys = ("height", "inferred", "slope_x", "slope_y", "roughness", "guess")
        st = {k: np.empty((X, X), np.float64) for k in keys}
        self._l.hm_get_maps(self._h, *[_ptr(st[k]) for k in keys])
        return st


# the known-answer fixtures and the 16-slot ring; every fixture also replays
# through the host-built C ABI in tests/test_capi_host.py
MAPPER_FIXTURES = [n for n in golden_files() if n.startswith("kat_")] + ["synth_ring16.npz"]


@pytest.mark.parametrize("name", MAPPER_FIXTURES)
def test_host_build_replays_every_fixture(lib, name):
    fx = load(os.path.join(GOLDEN, name))
    m = HostMapper(lib, params_of(fx))
    try:
        replay_and_compare(m, fx, stats=True, debug=True)
    finally:
        m.close()


def _host(lib, **tuning):
    """A constructor with the reference's signature for the host build."""
    return lambda *params: HostMapper(lib, params, **tuning)


def _terrain_scans(n, beams, columns, extent, seed=0, offset=(0.0, 0.0, 0.0), **kw):
    from gvom_gb300.synthetic import Lidar, Terrain, make_scan, make_trajectory
    t = Terrain.make(seed, extent=extent, path_len=n * 0.4, offset=offset)
    lid = Lidar(beams=beams, columns=columns)
    return [make_scan(t, lid, p, i, **kw) for i, p in enumerate(make_trajectory(n))]


@pytest.mark.parametrize("tile,planes", [(256, 4), (128, 16), (64, 8)])
def test_launch_shapes_vs_oracle(lib, tile, planes):
    """The autotuner's other launch shapes against the oracle: k_maps2d tiles
    of 8 x 32 (288-thread blocks), 8 x 16 and 4 x 16 cells, k_merge chunks of
    4 and 16 planes, a combine after every scan."""
    params = (0.2, 0.2, 48, 16, 3, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    _run_both(_host(lib, maps_tile=tile, merge_planes=planes), params,
              _terrain_scans(4, 16, 256, 9.6, dropout=0.2))


@pytest.mark.parametrize("B", [1, 4, 8, 16])
def test_ring_sizes_every_source_class_vs_oracle(lib, B):
    """Rings of 1 to 16 slots, a combine after every scan: every source-count
    class of the merges (2, 3, 5, 9 and 17 sources), the ring full and after
    it wraps (scripts/gvom.py:242-298)."""
    params = (0.25, 0.25, 24, 8, B, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    _run_both(_host(lib), params, _terrain_scans(B + 3, 8, 128, 6.0, dropout=0.25))


def test_odd_grid_and_row_length(lib):
    """xy_size 63 (extended rows of 65 cells) and eigen distances (1, 2)."""
    params = (0.2, 0.2, 63, 21, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 2)
    _compare_runs(_host(lib), params, [(s.points, s.ego, s.transform) for s in _terrain_scans(2, 16, 256, 12.6)])


def test_eigen_distances_and_far_world_offset(lib):
    """Eigen distances (2, 0) and a 1e4 m world offset."""
    params = (0.1, 0.1, 64, 24, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 2, 0)
    _run_both(_host(lib), params, _terrain_scans(3, 16, 256, 6.4, offset=(1.0e4, 0.0, 0.0)))


def test_origin_beyond_float32_floor_range(lib):
    """A world origin past 2^22 voxels: ray indices take the float64 path."""
    params = (0.1, 0.1, 64, 24, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    runs = [(s.points, s.ego, s.transform) for s in
            _terrain_scans(2, 16, 256, 6.4, offset=(5.0e5, -2.0e5, 0.0), transform_dtype=np.float64)]
    _compare_runs(_host(lib), params, runs)


def test_empty_and_out_of_grid_scans(lib):
    params = (0.2, 0.2, 32, 16, 2, 1.0, 0.5, 0.5, 0.3, 2.0, 4.0, 1.0, 1, 1)
    g, o = _host(lib)(*params), OracleGvom(*params)
    assert g.combine_maps() is None
    empty = np.zeros((0, 3), np.float32)
    far = np.array([[500.0, 0.0, 0.0], [0.0, -400.0, 3.0]], np.float32)  # no hit inside the grid
    for pts in (empty, far, empty):
        g.Process_pointcloud(pts, (0.1, 0.2, 1.0))
        o.Process_pointcloud(pts, (0.1, 0.2, 1.0))
        _, last = g.ring_state()
        compare_slot(canonical_state(g.slot_state(last)), canonical_state(o.slot_state(last)), "scan")
        out, ref = g.combine_maps(), o.combine_maps()
        for a, b in zip(out, ref):
            np.testing.assert_array_equal(a, b)


def test_rays_inside_the_sliver_below_zero(lib):
    """Ray positions in (-2^-20, 0) voxels with a non-zero grid origin."""
    params = (0.2, 0.2, 32, 16, 2, 0.1, 0.5, 0.5, 0.3, 2.0, 1.0, 1.0, 1, 1)
    rng = np.random.default_rng(11)
    ex = np.float32(-1.0e-21)
    n = 1500
    pts = np.empty((n, 3), np.float32)
    pts[:, 0] = ex  # rays in the plane x = ego x stay inside the sliver for every step
    pts[:, 1] = rng.uniform(-3, 3, n)
    pts[:, 2] = rng.uniform(-1.5, 2.5, n)
    pts[: n // 3, 0] = np.float32(-1e-9) * rng.uniform(0, 1, n // 3).astype(np.float32)
    pts2 = pts.copy()
    pts2[:, 0] = np.float32(-4.0e-7)
    _compare_runs(_host(lib), params, [(pts, (float(ex), 0.05, 1.0), None), (pts2, (-2.0e-7, -0.03, 0.8), None)])
