/* The process call's constants and scan descriptors as the library's host
 * code fills them (prepare_scans and exact_res in
 * gvom_gb300/csrc/gvom_capi.cu), for host builds that run the process kernels
 * (tests/test_process_host.py, tests/test_pipeline_host.py).  Include after
 * gvom_internal.cuh.  Not part of the library. */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>

namespace host_scan {
using namespace gvom;

// r = mr 2^er (53-bit mr), W = floor(2^116 / mr)
inline ExactRes exact_res(double r) {
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

inline ProcessConst process_const(int X, int Z, int exy, int ez, double xy_res, double z_res, double min_distance,
                                  int nscans, int num_sms) {
    ProcessConst pc;
    std::memset(&pc, 0, sizeof pc);
    Geom &g = pc.g;
    g.X = X; g.Z = Z; g.exy = exy; g.ez = ez; g.Xe = X + 2 * exy; g.Ze = Z + 2 * ez;
    g.V = (long long)X * X * Z; g.Vext = (long long)g.Xe * g.Xe * g.Ze;
    pc.xy_res = xy_res; pc.z_res = z_res;
    pc.md2 = min_distance * min_distance;
    // smallest float32 whose value is >= md2
    float f = (float)pc.md2;
    if ((double)f < pc.md2) f = std::nextafter(f, INFINITY);
    while ((double)std::nextafter(f, -INFINITY) >= pc.md2) f = std::nextafter(f, -INFINITY);
    pc.md2_f32 = f;
    pc.rxy = exact_res(xy_res);
    pc.rz = exact_res(z_res);
    pc.step_cap = 2 * std::max(X, Z) + 8;
    pc.num_sms = num_sms;
    pc.xe_magic = ~0ull / (unsigned long long)g.Xe + 1ull;
    pc.nscans = nscans;
    return pc;
}

// a scan's descriptor but for its buffers (cnt, idx, rec, rec_cap, ctr) and
// its block and point bases; tmode 0 none, 1 float32, 2 float64 transform,
// T: rows 0..2 of the 4x4
inline void scan_desc(ScanDesc &d, const ProcessConst &pc, const void *pts, long long n, long long stride, int tmode,
                      const double ego[3], const double T[12]) {
    const int X = pc.g.X, Z = pc.g.Z;
    std::memset(&d, 0, sizeof d);
    d.pts = pts; d.n = n; d.stride = stride; d.tmode = tmode;
    for (int r = 0; r < 12; r++) { d.T[r] = T[r]; d.Tf[r] = (float)T[r]; }
    // ray_origin (scripts/gvom.py:138-141)
    d.od[0] = std::floor((ego[0] / pc.xy_res) - (double)X / 2.0);
    d.od[1] = std::floor((ego[1] / pc.xy_res) - (double)X / 2.0);
    d.od[2] = std::floor((ego[2] / pc.z_res) - (double)Z / 2.0);
    bool fast = true, exact = true;
    const double lim = 4194304.0 - (double)std::max(X, Z) - 2.0;
    for (int a = 0; a < 3; a++) {
        if (!(std::fabs(d.od[a]) < 2147483648.0)) exact = false;
        if (!(std::fabs(d.od[a]) < lim)) fast = false;
    }
    for (int a = 0; a < 3; a++) d.oi[a] = exact ? (int)d.od[a] : 0;
    d.fast_floor = fast; d.exact_ok = exact;
    d.pt0[0] = (float)(ego[0] / pc.xy_res); d.pt0[1] = (float)(ego[1] / pc.xy_res);
    d.pt0[2] = (float)(ego[2] / pc.z_res);
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
}

}  // namespace host_scan
