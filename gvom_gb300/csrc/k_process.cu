// Per-scan kernels: Gvom.Process_pointcloud (scripts/gvom.py:105-217).
//
//   k_voxelize_trace  transform + min-distance filter + hit voxel + ray march
//                     (scripts/gvom.py:1121-1231); also records every point's
//                     voxel fraction and cell for the statistics
//   k_assign          compact-index allocation and dense->compact move
//                     (scripts/gvom.py:1233-1247), point-group offsets
//   k_scatter         groups points by cell (rank from the hit atomic)
//   k_voxel_stats     neighbourhood mean / covariance / count and in-voxel
//                     minimum height (scripts/gvom.py:1249-1421)
//   k_cleanup         returns the dense count array to zero
//
// All float arithmetic that decides an integer result uses the IEEE-rounded
// intrinsics in the reference's operand types, without contraction.
#include "gvom_internal.cuh"

namespace gvom {

template <int NS>
__device__ __forceinline__ int find_scan(const ScanTable<NS> &tab, int nscans, int block) {
    int s = 0;
#pragma unroll
    for (int i = 1; i < NS; i++)
        if (i < nscans && block >= tab.s[i].block_begin) s = i;
    return s;
}

template <typename PT>
__device__ __forceinline__ void load_point(const ScanDesc &sd, long long i, PT &x, PT &y, PT &z) {
    const PT *p = static_cast<const PT *>(sd.pts) + i * sd.stride;
    x = p[0];
    y = p[1];
    z = p[2];
}

// __transform_pointcloud (scripts/gvom.py:1121-1138): all-float32 when both
// operands are float32, float64 otherwise; the result is stored back in the
// point dtype.
template <typename PT>
__device__ __forceinline__ void transform_point(const ScanDesc &sd, PT &x, PT &y, PT &z);

template <>
__device__ __forceinline__ void transform_point<float>(const ScanDesc &sd, float &x, float &y, float &z) {
    float o[3];
    if (sd.tmode == 1) {
#pragma unroll
        for (int r = 0; r < 3; r++) {
            float t0 = (float)sd.T[r * 4 + 0], t1 = (float)sd.T[r * 4 + 1];
            float t2 = (float)sd.T[r * 4 + 2], t3 = (float)sd.T[r * 4 + 3];
            float s = __fadd_rn(__fmul_rn(x, t0), __fmul_rn(y, t1));
            s = __fadd_rn(s, __fmul_rn(z, t2));
            o[r] = __fadd_rn(s, t3);
        }
    } else {
        double xd = x, yd = y, zd = z;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            double s = __dadd_rn(__dmul_rn(xd, sd.T[r * 4 + 0]), __dmul_rn(yd, sd.T[r * 4 + 1]));
            s = __dadd_rn(s, __dmul_rn(zd, sd.T[r * 4 + 2]));
            o[r] = __double2float_rn(__dadd_rn(s, sd.T[r * 4 + 3]));
        }
    }
    x = o[0];
    y = o[1];
    z = o[2];
}

template <>
__device__ __forceinline__ void transform_point<double>(const ScanDesc &sd, double &x, double &y, double &z) {
    double o[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        double s = __dadd_rn(__dmul_rn(x, sd.T[r * 4 + 0]), __dmul_rn(y, sd.T[r * 4 + 1]));
        s = __dadd_rn(s, __dmul_rn(z, sd.T[r * 4 + 2]));
        o[r] = __dadd_rn(s, sd.T[r * 4 + 3]);
    }
    x = o[0];
    y = o[1];
    z = o[2];
}

// d2 = x*x + y*y + z*z in the point dtype (scripts/gvom.py:1145-1148).
__device__ __forceinline__ double point_d2(float x, float y, float z) {
    float s = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
    return (double)__fadd_rn(s, __fmul_rn(z, z));
}
__device__ __forceinline__ double point_d2(double x, double y, double z) {
    double s = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    return __dadd_rn(s, __dmul_rn(z, z));
}

__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0 && v) atomicAdd(dst, v);
}

// ---------------------------------------------------------------------------
// k_voxelize_trace: one thread per point.
// ---------------------------------------------------------------------------
template <typename PT, int NS>
__global__ void __launch_bounds__(256) k_voxelize_trace(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                       float4 *__restrict__ prec, int *__restrict__ prank) {
    const int s = find_scan(tab, pc.nscans, blockIdx.x);
    const ScanDesc &sd = tab.s[s];
    const Geom g = pc.g;
    const long long i = (long long)(blockIdx.x - sd.block_begin) * blockDim.x + threadIdx.x;
    const bool active = i < sd.n;
    unsigned long long n_valid = 0, n_hit = 0, n_steps = 0;
    if (active) {
        const long long gi = sd.pt_base + i;
        float4 rec = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        int rank = 0;
        PT x, y, z;
        load_point<PT>(sd, i, x, y, z);
        if (sd.tmode) transform_point<PT>(sd, x, y, z);
        bool ok = isfinite((double)x) && isfinite((double)y) && isfinite((double)z);
        if (ok && point_d2(x, y, z) < pc.md2) ok = false;
        if (ok) {
            n_valid = 1;
            // hit voxel in float64 (scripts/gvom.py:1153-1171)
            const double q0 = __ddiv_rn((double)x, pc.xy_res);
            const double q1 = __ddiv_rn((double)y, pc.xy_res);
            const double q2 = __ddiv_rn((double)z, pc.z_res);
            const double t0 = __dsub_rn(q0, sd.od[0]), t1 = __dsub_rn(q1, sd.od[1]), t2 = __dsub_rn(q2, sd.od[2]);
            const double f0 = floor(t0), f1 = floor(t1), f2 = floor(t2);
            // extended cell (grid + neighbourhood halo)
            if (f0 >= -(double)g.exy && f0 < (double)(g.X + g.exy) && f1 >= -(double)g.exy &&
                f1 < (double)(g.X + g.exy) && f2 >= -(double)g.ez && f2 < (double)(g.Z + g.ez)) {
                const int bx = (int)f0, by = (int)f1, bz = (int)f2;
                const bool in_grid = bx >= 0 && bx < g.X && by >= 0 && by < g.X && bz >= 0 && bz < g.Z;
                const long long cell =
                    (long long)(bx + g.exy) + (long long)(by + g.exy) * g.Xe + (long long)(bz + g.ez) * g.Xe * g.Xe;
                const unsigned long long inc = in_grid ? ((1ull << 32) | 1ull) : (1ull << 32);
                const unsigned long long old = atomicAdd(&sd.cnt[cell], inc);
                rank = (int)(old >> 32);
                rec = make_float4(__double2float_rn(__dsub_rn(t0, f0)), __double2float_rn(__dsub_rn(t1, f1)),
                                  __double2float_rn(__dsub_rn(t2, f2)), __int_as_float((int)cell));
                n_hit = in_grid;
            }
            // ray march (scripts/gvom.py:1174-1231), float32 state
            float px = sd.pt0[0], py = sd.pt0[1], pz = sd.pt0[2];
            const float e0 = __double2float_rn(q0), e1 = __double2float_rn(q1), e2 = __double2float_rn(q2);
            float s0 = __fsub_rn(e0, px), s1 = __fsub_rn(e1, py), s2 = __fsub_rn(e2, pz);
            float ss = __fadd_rn(__fmul_rn(s0, s0), __fmul_rn(s1, s1));
            ss = __fadd_rn(ss, __fmul_rn(s2, s2));
            const float rl = __fsqrt_rn(ss);
            s0 = __fdiv_rn(s0, rl);
            s1 = __fdiv_rn(s1, rl);
            s2 = __fdiv_rn(s2, rl);
            const float a0 = fabsf(s0), a1 = fabsf(s1), a2 = fabsf(s2);
            const float inner = a2 > a1 ? a2 : a1;
            const float smax = inner > a0 ? inner : a0;
            int k = 0;
            if (smax == a1) k = 1;
            if (smax == a2) k = 2;
            const float sk = k == 0 ? s0 : (k == 1 ? s1 : s2);
            const float ak = fabsf(sk);
            const float ix = k == 0 ? __fdiv_rn(sk, ak) : __fdiv_rn(s0, ak);
            const float iy = k == 1 ? __fdiv_rn(sk, ak) : __fdiv_rn(s1, ak);
            const float iz = k == 2 ? __fdiv_rn(sk, ak) : __fdiv_rn(s2, ak);
            const double R = __dsub_rn((double)rl, 1.0);
            const double linc = fabs(__ddiv_rn(1.0, (double)sk));
            const int K = ray_step_count(R, linc, pc.step_cap);
            const int fast = sd.fast_floor;
            unsigned long long* __restrict__ cnt = sd.cnt;
            int st = 0;
            for (; st < K; st++) {
                px = __fadd_rn(px, ix);
                py = __fadd_rn(py, iy);
                pz = __fadd_rn(pz, iz);
                const int vx = ray_index(px, sd.oi[0], sd.od[0], fast);
                const int vy = ray_index(py, sd.oi[1], sd.od[1], fast);
                const int vz = ray_index(pz, sd.oi[2], sd.od[2], fast);
                if ((unsigned)vx >= (unsigned)g.X || (unsigned)vy >= (unsigned)g.X || (unsigned)vz >= (unsigned)g.Z) break;
                const long long cell =
                    (long long)(vx + g.exy) + (long long)(vy + g.exy) * g.Xe + (long long)(vz + g.ez) * g.Xe * g.Xe;
                atomicAdd(&cnt[cell], 1ull);
            }
            n_steps = st;
        }
        prec[gi] = rec;
        prank[gi] = rank;
    }
    warp_add_u64(&sd.ctr->valid, n_valid);
    warp_add_u64(&sd.ctr->hits, n_hit);
    warp_add_u64(&sd.ctr->steps, n_steps);
}

// ---------------------------------------------------------------------------
// k_assign: one thread per extended cell, blockIdx.y = scan.
// In-grid cells: hit > 0 -> compact index (warp-aggregated counter) and the
// record's hit/total/voxel id; else -(total)-1 (scripts/gvom.py:1233-1247).
// Cells holding points (occupied or halo) get a point-group offset; the count
// word is rewritten to (offset << 32 | points) for k_scatter / k_voxel_stats.
// Free cells are cleared here; point cells are cleared by k_cleanup.
// ---------------------------------------------------------------------------
template <int NS>
__global__ void __launch_bounds__(256) k_assign(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab) {
    const ScanDesc &sd = tab.s[blockIdx.y];
    const Geom g = pc.g;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v = 0;
    int ex = 0, ey = 0, ez = 0;
    bool inr = e < g.Vext;
    if (inr) {
        v = sd.cnt[e];
        long long t = e;
        ex = (int)(t % g.Xe);
        t /= g.Xe;
        ey = (int)(t % g.Xe);
        ez = (int)(t / g.Xe);
    }
    const int hit = (int)(v >> 32);
    const int total = (int)(v & 0xffffffffull);
    const int gx = ex - g.exy, gy = ey - g.exy, gz = ez - g.ez;
    const bool in_grid = inr && gx >= 0 && gx < g.X && gy >= 0 && gy < g.X && gz >= 0 && gz < g.Z;
    const bool occ = in_grid && hit > 0;
    const bool grp = inr && hit > 0;  // cell holds points
    const unsigned lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    // compact index
    const unsigned om = __ballot_sync(0xffffffffu, occ);
    int cbase = 0;
    if (om) {
        const int leader = __ffs(om) - 1;
        if ((int)lane == leader) cbase = atomicAdd(&sd.ctr->C, __popc(om));
        cbase = __shfl_sync(0xffffffffu, cbase, leader);
    }
    const int c = cbase + __popc(om & lt);
    // point-group offset: warp exclusive scan of hit counts
    int incl = grp ? hit : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += n;
    }
    const int wsum = __shfl_sync(0xffffffffu, incl, 31);
    int pbase = 0;
    if (wsum) {
        if (lane == 31) pbase = atomicAdd(&sd.ctr->pts, wsum);
        pbase = __shfl_sync(0xffffffffu, pbase, 31);
    }
    const int off = pbase + incl - (grp ? hit : 0);
    if (!inr) return;
    if (in_grid) {
        const long long gid = (long long)gx + (long long)gy * g.X + (long long)gz * g.X * g.X;
        if (occ) {
            if (c < sd.rec_cap) {
                VoxelRec *r = &sd.rec[c];
                r->hit = hit;
                r->total = total;
                r->aux[0] = __int_as_float((int)gid);
            } else {
                atomicOr(&sd.ctr->overflow, 1);
            }
            sd.idx[gid] = c;
        } else {
            sd.idx[gid] = -total - 1;
            if (total) sd.cnt[e] = 0ull;
        }
    }
    if (grp) sd.cnt[e] = ((unsigned long long)(unsigned)off << 32) | (unsigned)hit;
}

// ---------------------------------------------------------------------------
// k_scatter: one thread per point; places the point's voxel fraction at
// group offset + its rank in the cell.
// ---------------------------------------------------------------------------
template <int NS>
__global__ void __launch_bounds__(256) k_scatter(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                const float4 *__restrict__ prec, const int *__restrict__ prank,
                                                float4 *__restrict__ sorted) {
    const int s = find_scan(tab, pc.nscans, blockIdx.x);
    const ScanDesc &sd = tab.s[s];
    const long long i = (long long)(blockIdx.x - sd.block_begin) * blockDim.x + threadIdx.x;
    if (i >= sd.n) return;
    const long long gi = sd.pt_base + i;
    const float4 r = prec[gi];
    const int cell = __float_as_int(r.w);
    if (cell < 0) return;
    const unsigned long long v = sd.cnt[cell];
    const int off = (int)(v >> 32);
    sorted[sd.pt_base + off + prank[gi]] = make_float4(r.x, r.y, r.z, 0.f);
}

// ---------------------------------------------------------------------------
// k_voxel_stats: one thread per occupied voxel, blockIdx.y = scan.
// Two-pass mean / covariance over the points of the (2exy+1)^2 (2ez+1)
// neighbourhood (scripts/gvom.py:1249-1387), float32 on coordinates centred
// on the voxel centre with Kahan-compensated sums; minimum height over the
// voxel's own points (scripts/gvom.py:1389-1421), exact.
// ---------------------------------------------------------------------------
template <int NS>
__global__ void __launch_bounds__(128) k_voxel_stats(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                    const float4 *__restrict__ sorted) {
    const ScanDesc &sd = tab.s[blockIdx.y];
    const Geom g = pc.g;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int C = *(volatile int *)&sd.ctr->C;
    if (c >= C || c >= sd.rec_cap) return;
    VoxelRec *r = &sd.rec[c];
    const int gid = __float_as_int(r->aux[0]);
    const int x = gid % g.X, y = (gid / g.X) % g.X, z = gid / (g.X * g.X);
    const long long e0 = (long long)(x + g.exy) + (long long)(y + g.exy) * g.Xe + (long long)(z + g.ez) * g.Xe * g.Xe;
    const float4 *__restrict__ P = sorted + sd.pt_base;
    // own cell: min height
    float mh = 1.0f;
    {
        const unsigned long long v = sd.cnt[e0];
        const int off = (int)(v >> 32), n = (int)(v & 0xffffffffull);
        for (int j = 0; j < n; j++) mh = fminf(mh, P[off + j].z);
    }
    KSum sx, sy, sz;
    sx.init(); sy.init(); sz.init();
    int n_all = 0;
    for (int dz = -g.ez; dz <= g.ez; dz++)
        for (int dy = -g.exy; dy <= g.exy; dy++)
            for (int dx = -g.exy; dx <= g.exy; dx++) {
                const long long e = e0 + dx + (long long)dy * g.Xe + (long long)dz * g.Xe * g.Xe;
                const unsigned long long v = sd.cnt[e];
                const int n = (int)(v & 0xffffffffull);
                if (!n) continue;
                const int off = (int)(v >> 32);
                // centred coordinate of a neighbour point: frac + offset - 0.5
                const float ox = (float)dx - 0.5f, oy = (float)dy - 0.5f, oz = (float)dz - 0.5f;
                for (int j = 0; j < n; j++) {
                    const float4 p = P[off + j];
                    sx.add(__fadd_rn(p.x, ox));
                    sy.add(__fadd_rn(p.y, oy));
                    sz.add(__fadd_rn(p.z, oz));
                }
                n_all += n;
            }
    const float nf = (float)n_all;
    const float mx = __fdiv_rn(sx.s, nf), my = __fdiv_rn(sy.s, nf), mz = __fdiv_rn(sz.s, nf);
    KSum cxx, cxy, cxz, cyy, cyz, czz;
    cxx.init(); cxy.init(); cxz.init(); cyy.init(); cyz.init(); czz.init();
    for (int dz = -g.ez; dz <= g.ez; dz++)
        for (int dy = -g.exy; dy <= g.exy; dy++)
            for (int dx = -g.exy; dx <= g.exy; dx++) {
                const long long e = e0 + dx + (long long)dy * g.Xe + (long long)dz * g.Xe * g.Xe;
                const unsigned long long v = sd.cnt[e];
                const int n = (int)(v & 0xffffffffull);
                if (!n) continue;
                const int off = (int)(v >> 32);
                const float ox = (float)dx - 0.5f - mx, oy = (float)dy - 0.5f - my, oz = (float)dz - 0.5f - mz;
                for (int j = 0; j < n; j++) {
                    const float4 p = P[off + j];
                    const float ux = __fadd_rn(p.x, ox), uy = __fadd_rn(p.y, oy), uz = __fadd_rn(p.z, oz);
                    cxx.add(__fmul_rn(ux, ux));
                    cxy.add(__fmul_rn(ux, uy));
                    cxz.add(__fmul_rn(ux, uz));
                    cyy.add(__fmul_rn(uy, uy));
                    cyz.add(__fmul_rn(uy, uz));
                    czz.add(__fmul_rn(uz, uz));
                }
            }
    float4 *o = reinterpret_cast<float4 *>(r);
    o[0] = make_float4(mx + 0.5f, my + 0.5f, mz + 0.5f, __fdiv_rn(cxx.s, nf));
    o[1] = make_float4(__fdiv_rn(cxy.s, nf), __fdiv_rn(cxz.s, nf), __fdiv_rn(cyy.s, nf), __fdiv_rn(cyz.s, nf));
    reinterpret_cast<float2 *>(r)[4] = make_float2(__fdiv_rn(czz.s, nf), nf);
    r->min_h = mh;
}

// ---------------------------------------------------------------------------
// k_cleanup: one thread per point; the first point of each cell zeroes the
// cell's count word so the dense array is all-zero for the next scan.
// ---------------------------------------------------------------------------
template <int NS>
__global__ void __launch_bounds__(256) k_cleanup(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                const float4 *__restrict__ prec, const int *__restrict__ prank) {
    const int s = find_scan(tab, pc.nscans, blockIdx.x);
    const ScanDesc &sd = tab.s[s];
    const long long i = (long long)(blockIdx.x - sd.block_begin) * blockDim.x + threadIdx.x;
    if (i >= sd.n) return;
    const long long gi = sd.pt_base + i;
    const int cell = __float_as_int(prec[gi].w);
    if (cell >= 0 && prank[gi] == 0) sd.cnt[cell] = 0ull;
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <int NS>
static cudaError_t launch_ns(const ProcessConst &pc, const ScanDesc *table, int total_blocks, int max_n, int dtype,
                             float4 *prec, int *prank, float4 *sorted, cudaStream_t st, cudaEvent_t *ev) {
    ScanTable<NS> tab;
    for (int i = 0; i < NS; i++) tab.s[i] = i < pc.nscans ? table[i] : table[0];
    if (total_blocks < 1) total_blocks = 1;
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], st);
    };
    mark(0);
    if (dtype == 1)
        k_voxelize_trace<double, NS><<<total_blocks, 256, 0, st>>>(pc, tab, prec, prank);
    else
        k_voxelize_trace<float, NS><<<total_blocks, 256, 0, st>>>(pc, tab, prec, prank);
    mark(1);
    dim3 ga((unsigned)((pc.g.Vext + 255) / 256), pc.nscans);
    k_assign<NS><<<ga, 256, 0, st>>>(pc, tab);
    mark(2);
    k_scatter<NS><<<total_blocks, 256, 0, st>>>(pc, tab, prec, prank, sorted);
    mark(3);
    dim3 gs((unsigned)((max_n + 127) / 128 > 0 ? (max_n + 127) / 128 : 1), pc.nscans);
    k_voxel_stats<NS><<<gs, 128, 0, st>>>(pc, tab, sorted);
    mark(4);
    k_cleanup<NS><<<total_blocks, 256, 0, st>>>(pc, tab, prec, prank);
    mark(5);
    return cudaGetLastError();
}

cudaError_t launch_process(const ProcessConst &pc, const ScanDesc *table, int nscans, int total_blocks, int max_n,
                           int dtype, float4 *prec, int *prank, float4 *sorted, cudaStream_t st, cudaEvent_t *ev) {
    if (nscans == 1) return launch_ns<1>(pc, table, total_blocks, max_n, dtype, prec, prank, sorted, st, ev);
    if (nscans <= 4) return launch_ns<4>(pc, table, total_blocks, max_n, dtype, prec, prank, sorted, st, ev);
    return launch_ns<kMaxBatch>(pc, table, total_blocks, max_n, dtype, prec, prank, sorted, st, ev);
}

}  // namespace gvom
