// Per-scan kernels: Gvom.Process_pointcloud (scripts/gvom.py:105-217).
//
// The slot's index map is the pass-through counter: it is filled with -1
// (unknown) before the scan, and every ray step and every in-grid hit
// subtracts one from its voxel's word, which leaves a free voxel at
// -(total)-1, the reference's encoding (scripts/gvom.py:1233-1240).  The
// points' cells (grid plus the eigen-neighbourhood halo) count their points
// in a separate, sparsely touched word array (`cnt`, zero between scans).
//
//   k_voxelize_trace  transform + min-distance filter + hit voxel + ray march
//                     (scripts/gvom.py:1121-1231); also records every point's
//                     voxel fraction, cell and rank in its cell
//   k_assign          one thread per point-holding cell (its first point):
//                     compact index and record of occupied voxels, total =
//                     -(word)-1 read back from the index map
//                     (scripts/gvom.py:1233-1247), point-group offsets; the
//                     owner of an in-grid cell keeps the compact index in its
//                     rank word
//   k_scatter         groups points by cell (rank from the hit atomic)
//   k_cell_moments    per point-holding cell: moments of its points and their
//                     minimum height, which goes into the voxel's record
//                     (scripts/gvom.py:1390-1421)
//   k_voxel_stats     neighbourhood mean / covariance / count
//                     (scripts/gvom.py:1249-1387)
//   k_cleanup         returns the cell words to zero
//
// All float arithmetic that decides an integer result uses the IEEE-rounded
// intrinsics in the reference's operand types, without contraction.
#include <algorithm>

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

// float64 processing also serves PointCloud2 data: float32 fields widened to
// float64, as the reference's ROS node converts a cloud before mapping it
// (scripts/gvom_ros.py:108)
template <>
__device__ __forceinline__ void load_point<double>(const ScanDesc &sd, long long i, double &x, double &y,
                                                   double &z) {
    if (sd.pc2) {
        const char *b = static_cast<const char *>(sd.pts) + i * sd.stride;
        if (sd.pc2 == 1) {
            x = (double)*reinterpret_cast<const float *>(b + sd.off[0]);
            y = (double)*reinterpret_cast<const float *>(b + sd.off[1]);
            z = (double)*reinterpret_cast<const float *>(b + sd.off[2]);
        } else {
            x = *reinterpret_cast<const double *>(b + sd.off[0]);
            y = *reinterpret_cast<const double *>(b + sd.off[1]);
            z = *reinterpret_cast<const double *>(b + sd.off[2]);
        }
        return;
    }
    const double *p = static_cast<const double *>(sd.pts) + i * sd.stride;
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
            const float t0 = sd.Tf[r * 4 + 0], t1 = sd.Tf[r * 4 + 1];
            const float t2 = sd.Tf[r * 4 + 2], t3 = sd.Tf[r * 4 + 3];
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

// d2 = x*x + y*y + z*z in the point dtype, compared with min_distance^2 in
// float64 (scripts/gvom.py:1145-1148).  For float32 points the comparison
// (double)d2 < md2 equals d2 < md2_f32, the smallest float32 whose value is
// >= md2 (computed on the host), so it needs no float64 operation.
__device__ __forceinline__ bool below_min_distance(float x, float y, float z, const ProcessConst &pc) {
    float s = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
    s = __fadd_rn(s, __fmul_rn(z, z));
    return s < pc.md2_f32;
}
__device__ __forceinline__ bool below_min_distance(double x, double y, double z, const ProcessConst &pc) {
    double s = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    return __dadd_rn(s, __dmul_rn(z, z)) < pc.md2;
}

__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0 && v) atomicAdd(dst, v);
}

// ---------------------------------------------------------------------------
// k_voxelize_trace: one thread per point.
//
// Every ray starts at the ego, so the voxels around it receive a pass from
// almost every ray.  A ray's first steps, while they stay inside a kCube^3
// block of voxels around the ego voxel (sd.cube0, inside the grid), are
// counted in shared memory and flushed once per block (one global atomic per
// touched voxel).  The remaining steps go through a per-block shared hash
// table of (voxel, count): neighbouring rays of a block cross many of the
// same voxels, and a shared atomic is several times cheaper than a scattered
// global reduction; a step whose slot holds another voxel subtracts straight
// from the index map word.
// ---------------------------------------------------------------------------

// per-block shared hash table for the ray steps outside the cube
// (GVOM_TRACE_HASH_BITS = log2 slots; 0 = every such step adds globally)
#ifndef GVOM_TRACE_HASH_BITS
#define GVOM_TRACE_HASH_BITS 11
#endif
constexpr int kHashBits = GVOM_TRACE_HASH_BITS > 0 ? GVOM_TRACE_HASH_BITS : 1;
constexpr bool kHash = GVOM_TRACE_HASH_BITS > 0;
constexpr unsigned kHashEmpty = 0xffffffffu;

template <typename PT, int NS>
__global__ void __launch_bounds__(256) k_voxelize_trace(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                       float4 *__restrict__ prec, int *__restrict__ prank) {
    __shared__ unsigned cube[kCubeCells];
    __shared__ unsigned htag[1 << kHashBits], hcnt[1 << kHashBits];
    const int s = find_scan(tab, pc.nscans, blockIdx.x);
    const ScanDesc &sd = tab.s[s];
    const Geom g = pc.g;
    const int ffloor = sd.fast_floor;
    if (sd.cube_on)
        for (int k = threadIdx.x; k < kCubeCells; k += blockDim.x) cube[k] = 0u;
    if (kHash)
        for (int k = threadIdx.x; k < (1 << kHashBits); k += blockDim.x) {
            htag[k] = kHashEmpty;
            hcnt[k] = 0u;
        }
    __syncthreads();
    const long long i = (long long)(blockIdx.x - sd.block_begin) * blockDim.x + threadIdx.x;
    const bool active = i < sd.n;
    unsigned long long n_valid = 0, n_hit = 0, n_steps = 0;
    const int Xe = g.Xe, XeXe = g.Xe * g.Xe;
    const int XX = g.X * g.X;
    if (active) {
        const long long gi = sd.pt_base + i;
        float4 rec = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        // the hit atomic's return value (the point's rank in its cell) is read
        // only after the march, which hides the atomic's round trip
        unsigned long long hit_old = 0;
        PT x, y, z;
        load_point<PT>(sd, i, x, y, z);
        if (sd.tmode) transform_point<PT>(sd, x, y, z);
        bool ok = isfinite(x) && isfinite(y) && isfinite(z);
        if (ok && below_min_distance(x, y, z, pc)) ok = false;
        if (ok) {
            n_valid = 1;
            // hit voxel, fractions and ray end (scripts/gvom.py:1153-1171, 1182-1184):
            // the float64 results, computed exactly with integer arithmetic
            // (gvom_exact.cuh); float64 only for inputs it declines
            float e0, e1, e2, fr0, fr1, fr2;
            int bx = 0, by = 0, bz = 0;
            bool fast = false, rng_ok = true;
            if (sizeof(PT) == 4 && sd.exact_ok) {
                long long b0, b1, b2;
                bool r0, r1, r2;
                fast = gx_coord((float)x, pc.rxy, sd.oi[0], e0, b0, fr0, r0) &&
                       gx_coord((float)y, pc.rxy, sd.oi[1], e1, b1, fr1, r1) &&
                       gx_coord((float)z, pc.rz, sd.oi[2], e2, b2, fr2, r2);
                rng_ok = r0 && r1 && r2;
                bx = (int)b0;
                by = (int)b1;
                bz = (int)b2;
            }
            bool in_ext;
            if (!fast) {
                const double q0 = __ddiv_rn((double)x, pc.xy_res);
                const double q1 = __ddiv_rn((double)y, pc.xy_res);
                const double q2 = __ddiv_rn((double)z, pc.z_res);
                const double t0 = __dsub_rn(q0, sd.od[0]), t1 = __dsub_rn(q1, sd.od[1]), t2 = __dsub_rn(q2, sd.od[2]);
                const double f0 = floor(t0), f1 = floor(t1), f2 = floor(t2);
                in_ext = f0 >= -(double)g.exy && f0 < (double)(g.X + g.exy) && f1 >= -(double)g.exy &&
                         f1 < (double)(g.X + g.exy) && f2 >= -(double)g.ez && f2 < (double)(g.Z + g.ez);
                if (in_ext) {
                    bx = (int)f0;
                    by = (int)f1;
                    bz = (int)f2;
                    fr0 = __double2float_rn(__dsub_rn(t0, f0));
                    fr1 = __double2float_rn(__dsub_rn(t1, f1));
                    fr2 = __double2float_rn(__dsub_rn(t2, f2));
                }
                e0 = __double2float_rn(q0);
                e1 = __double2float_rn(q1);
                e2 = __double2float_rn(q2);
            } else {
                in_ext = rng_ok && bx >= -g.exy && bx < g.X + g.exy && by >= -g.exy && by < g.X + g.exy &&
                         bz >= -g.ez && bz < g.Z + g.ez;
            }
            if (in_ext) {
                const bool in_grid = bx >= 0 && bx < g.X && by >= 0 && by < g.X && bz >= 0 && bz < g.Z;
                const int cell = (bx + g.exy) + (by + g.exy) * Xe + (bz + g.ez) * XeXe;
                hit_old = atomicAdd(&sd.cnt[cell], 1ull);  // the point's rank in its cell
                if (in_grid) atomicAdd(&sd.idx[bx + g.X * by + XX * bz], -1);  // a hit counts toward the total
                rec = make_float4(fr0, fr1, fr2, __int_as_float(cell));
                n_hit = in_grid;
            }
            // ray march (scripts/gvom.py:1174-1231), float32 state
            float px = sd.pt0[0], py = sd.pt0[1], pz = sd.pt0[2];
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
            const int K = ray_step_count(rl, sk, pc.step_cap);
            int *__restrict__ vmap = sd.idx;  // the slot's index map, counting down from -1
            int st = 0;
            if (ffloor) {
                // float32 voxel indices: floor(p) from the bits of p + 1.5 * 2^23 rounded
                // down, offset by the origin (ray_index); positions in the sliver
                // (-2^-20, 0) take the float64 formula
                const int kx = 0x4B400000 + sd.oi[0], ky = 0x4B400000 + sd.oi[1], kz = 0x4B400000 + sd.oi[2];
                if (sd.cube_on) {
                    // phase 1: steps inside the cube around the ego.  Each axis index is
                    // monotone along the ray, so the first step outside the cube ends
                    // this phase for good; the cube lies inside the grid.
                    const int cx = kx + sd.cube0[0], cy = ky + sd.cube0[1], cz = kz + sd.cube0[2];
                    for (; st < K; st++) {
                        const float nx = __fadd_rn(px, ix), ny = __fadd_rn(py, iy), nz = __fadd_rn(pz, iz);
                        const unsigned ux = (unsigned)(__float_as_int(__fadd_rd(nx, 12582912.0f)) - cx);
                        const unsigned uy = (unsigned)(__float_as_int(__fadd_rd(ny, 12582912.0f)) - cy);
                        const unsigned uz = (unsigned)(__float_as_int(__fadd_rd(nz, 12582912.0f)) - cz);
                        if (((ux | uy | uz) >= (unsigned)kCube) | in_sliver(nx) | in_sliver(ny) | in_sliver(nz)) break;
                        px = nx;
                        py = ny;
                        pz = nz;
                        atomicAdd(&cube[ux + kCube * (uy + kCube * uz)], 1u);
                    }
                }
                // phase 2: everywhere else in the grid; the ray ends at its first step
                // outside the grid (scripts/gvom.py:1216-1225).  Steps are counted in
                // the block's shared hash table of (cell, count) when the cell owns or
                // claims its slot, else by a global reduction.
                for (; st < K; st++) {
                    px = __fadd_rn(px, ix);
                    py = __fadd_rn(py, iy);
                    pz = __fadd_rn(pz, iz);
                    int vx = __float_as_int(__fadd_rd(px, 12582912.0f)) - kx;
                    int vy = __float_as_int(__fadd_rd(py, 12582912.0f)) - ky;
                    int vz = __float_as_int(__fadd_rd(pz, 12582912.0f)) - kz;
                    if (in_sliver(px) | in_sliver(py) | in_sliver(pz)) {
                        vx = ray_index(px, sd.oi[0], sd.od[0], 1);
                        vy = ray_index(py, sd.oi[1], sd.od[1], 1);
                        vz = ray_index(pz, sd.oi[2], sd.od[2], 1);
                    }
                    if ((unsigned)vx >= (unsigned)g.X || (unsigned)vy >= (unsigned)g.X || (unsigned)vz >= (unsigned)g.Z)
                        break;
                    const unsigned vid = (unsigned)(vx + g.X * vy + XX * vz);
                    if (kHash) {
                        const unsigned h = (vid * 2654435761u) >> (32 - kHashBits);
                        unsigned tag = htag[h];
                        if (tag == kHashEmpty) {
                            tag = atomicCAS(&htag[h], kHashEmpty, vid);
                            if (tag == kHashEmpty) tag = vid;
                        }
                        if (tag == vid) atomicAdd(&hcnt[h], 1u);
                        else atomicAdd(&vmap[vid], -1);
                    } else {
                        atomicAdd(&vmap[vid], -1);
                    }
                }
            } else {
                // origin far from the world origin: float64 voxel indices
                for (; st < K; st++) {
                    px = __fadd_rn(px, ix);
                    py = __fadd_rn(py, iy);
                    pz = __fadd_rn(pz, iz);
                    const int vx = ray_index(px, sd.oi[0], sd.od[0], 0);
                    const int vy = ray_index(py, sd.oi[1], sd.od[1], 0);
                    const int vz = ray_index(pz, sd.oi[2], sd.od[2], 0);
                    if ((unsigned)vx >= (unsigned)g.X || (unsigned)vy >= (unsigned)g.X || (unsigned)vz >= (unsigned)g.Z)
                        break;
                    atomicAdd(&vmap[vx + g.X * vy + XX * vz], -1);
                }
            }
            n_steps = st;
        }
        prec[gi] = rec;
        prank[gi] = (int)(unsigned)(hit_old & 0xffffffffull);
    }
    // scan counters: one atomic per block and counter (valid, hits, steps are
    // adjacent words)
    __shared__ unsigned long long wsum[3][8];
    {
        unsigned long long v3[3] = {n_valid, n_hit, n_steps};
#pragma unroll
        for (int j = 0; j < 3; j++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v3[j] += __shfl_down_sync(0xffffffffu, v3[j], o);
            if (lane_id() == 0) wsum[j][threadIdx.x >> 5] = v3[j];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += wsum[threadIdx.x][w];
        if (t) atomicAdd(&sd.ctr->valid + threadIdx.x, t);
    }
    if (kHash)
        for (int k = threadIdx.x; k < (1 << kHashBits); k += blockDim.x) {
            const unsigned t = htag[k];
            if (t != kHashEmpty) atomicAdd(&sd.idx[t], -(int)hcnt[k]);
        }
    if (!sd.cube_on) return;
    for (int k = threadIdx.x; k < kCubeCells; k += blockDim.x) {
        const unsigned c = cube[k];
        if (c) {
            const int vx = sd.cube0[0] + (k % kCube), vy = sd.cube0[1] + ((k / kCube) % kCube),
                      vz = sd.cube0[2] + k / (kCube * kCube);
            atomicAdd(&sd.idx[vx + g.X * vy + XX * vz], -(int)c);
        }
    }
}

// ---------------------------------------------------------------------------
// block-wide exclusive scan of two counters (up to 8 warps); returns this
// thread's exclusive prefixes and the block totals
// ---------------------------------------------------------------------------
__device__ __forceinline__ void block_scan2(int a, int b, int &ea, int &eb, int &ta, int &tb) {
    __shared__ int wa[8], wb[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    int ia = a, ib = b;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int na = __shfl_up_sync(0xffffffffu, ia, o), nb = __shfl_up_sync(0xffffffffu, ib, o);
        if (lane >= o) {
            ia += na;
            ib += nb;
        }
    }
    if (lane == 31) {
        wa[w] = ia;
        wb[w] = ib;
    }
    __syncthreads();
    int pa = 0, pb = 0, sa = 0, sb = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if (k >= nw) break;
        if (k < w) {
            pa += wa[k];
            pb += wb[k];
        }
        sa += wa[k];
        sb += wb[k];
    }
    ea = pa + ia - a;
    eb = pb + ib - b;
    ta = sa;
    tb = sb;
}

// ---------------------------------------------------------------------------
// k_assign: one thread per point; the thread of each cell's first point
// (rank 0) owns the cell.  An owned in-grid cell is an occupied voxel
// (hit > 0, scripts/gvom.py:1233-1240): it takes a compact index, and its
// record gets hit = the cell's point count, total = -(word)-1 of the index
// map (the ray steps and hits counted there), and the voxel id
// (scripts/gvom.py:1242-1247); the index map word becomes the compact
// index.  Every owned cell (occupied or halo) gets its point-group offset:
// its cell word becomes (offset << 32 | points) for k_scatter /
// k_voxel_stats.  Compact indices and offsets are reserved with one 64-bit
// atomic per block.
// ---------------------------------------------------------------------------

// grid voxel of extended cell e = x + Xe (y + Xe z), divisions by Xe as a
// multiply-high by xe_magic = floor((2^64 - 1) / Xe) + 1, exact for e < 2^32
// (xe_magic wraps to 0 for Xe = 1, where the quotient is e itself)
__device__ __forceinline__ bool cell_in_grid(unsigned e, const Geom &g, unsigned long long magic, int &gid) {
    const unsigned row = magic ? (unsigned)__umul64hi((unsigned long long)e, magic) : e;
    const unsigned ez = magic ? (unsigned)__umul64hi((unsigned long long)row, magic) : row;
    const int ex = (int)(e - row * (unsigned)g.Xe), ey = (int)(row - ez * (unsigned)g.Xe);
    const int gx = ex - g.exy, gy = ey - g.exy, gz = (int)ez - g.ez;
    gid = gx + g.X * (gy + g.X * gz);
    return (unsigned)gx < (unsigned)g.X && (unsigned)gy < (unsigned)g.X && (unsigned)gz < (unsigned)g.Z;
}

// The owner of an in-grid cell (its point of rank 0) leaves its voxel's
// compact index in its rank word as -2 - index, for k_cell_moments; readers
// of the rank take max(rank, 0).
template <int NS>
__global__ void __launch_bounds__(256) k_assign(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                               const float4 *__restrict__ prec, int *__restrict__ prank) {
    const int s = find_scan(tab, pc.nscans, blockIdx.x);
    const ScanDesc &sd = tab.s[s];
    const long long i = (long long)(blockIdx.x - sd.block_begin) * blockDim.x + threadIdx.x;
    int cell = -1, gid = 0, occ = 0, npts = 0;
    const long long gi = sd.pt_base + i;
    if (i < sd.n) {
        const int c = __float_as_int(prec[gi].w);
        if (c >= 0 && prank[gi] == 0) {
            cell = c;
            npts = (int)(unsigned)(sd.cnt[c] & 0xffffffffull);
            occ = cell_in_grid((unsigned)c, pc.g, pc.xe_magic, gid) ? 1 : 0;
        }
    }
    int eo, ep, to, tp;
    block_scan2(occ, npts, eo, ep, to, tp);
    __shared__ int bases[2];
    if (threadIdx.x == 0) {
        // C and pts are adjacent 32-bit words: one 64-bit atomic reserves both
        // (C stays far below 2^32, so nothing carries into pts)
        unsigned long long old = 0;
        if (to | tp)
            old = atomicAdd(reinterpret_cast<unsigned long long *>(&sd.ctr->C),
                            ((unsigned long long)(unsigned)tp << 32) | (unsigned)to);
        bases[0] = (int)(unsigned)(old & 0xffffffffull);
        bases[1] = (int)(unsigned)(old >> 32);
    }
    __syncthreads();
    if (cell < 0) return;
    if (occ) {
        const int c = bases[0] + eo;
        const int total = -1 - sd.idx[gid];
        if (c < sd.rec_cap) {
            VoxelRec *r = &sd.rec[c];
            *reinterpret_cast<int2 *>(&r->hit) = make_int2(npts, total);
            r->aux[0] = __int_as_float(gid);
        } else {
            atomicOr(&sd.ctr->overflow, 1);
        }
        sd.idx[gid] = c;
        prank[gi] = -2 - c;
    }
    sd.cnt[cell] = ((unsigned long long)(unsigned)(bases[1] + ep) << 32) | (unsigned)npts;
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
    sorted[sd.pt_base + off + max(prank[gi], 0)] = make_float4(r.x, r.y, r.z, 0.f);
}

// ---------------------------------------------------------------------------
// Neighbourhood statistics (scripts/gvom.py:1249-1421) in two steps.
//
// k_cell_moments: one thread per cell that holds points (the thread of the
// cell's rank-0 point); cells of more than kSmallCell points are handed to a
// whole warp.  Over the cell's points: count, mean of the in-cell fraction
// and the second moments about that mean (float32, Kahan-compensated,
// coordinates centred on the cell centre), and the minimum height fraction
// (exact).  Stored at the cell's group offset.
//
// k_voxel_stats: one thread per occupied voxel.  Combines the moments of
// the (2exy+1)^2 (2ez+1) neighbour cells, each shifted by its offset from the
// voxel, with the pairwise (Chan) update in a fixed cell order; the result
// is the neighbourhood mean (relative to the voxel corner), covariance and
// count the reference accumulates point by point.
// ---------------------------------------------------------------------------
struct __align__(16) CellMom {
    float m[3];     // mean fraction - 0.5
    float n;        // points
    float c[6];     // second moments about the mean: xx xy xz yy yz zz
    float min_h;    // lowest height fraction
    float pad;
};

constexpr int kSmallCell = 16;  // cells with more points are summed by a whole warp

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// the record of an in-grid cell's voxel takes the cell's lowest height
// fraction (__calculate_min_height, scripts/gvom.py:1390-1421: the points of
// the voxel itself), so the count merge can read it before the neighbourhood
// statistics are done; `ci`: the voxel's compact index from the owner's rank
// word (k_assign), -1 for a cell outside the grid
__device__ __forceinline__ void store_min_h(const ScanDesc &sd, int ci, float mh) {
    if (ci >= 0 && ci < sd.rec_cap) sd.rec[ci].min_h = mh;
}

template <int NS>
__global__ void __launch_bounds__(256) k_cell_moments(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                     const float4 *__restrict__ prec, const int *__restrict__ prank,
                                                     const float4 *__restrict__ sorted, CellMom *__restrict__ mom) {
    __shared__ int hq_off[256], hq_n[256], hq_rec[256];
    __shared__ int hq_count;
    const int s = find_scan(tab, pc.nscans, blockIdx.x);
    const ScanDesc &sd = tab.s[s];
    if (threadIdx.x == 0) hq_count = 0;
    __syncthreads();
    const long long i = (long long)(blockIdx.x - sd.block_begin) * blockDim.x + threadIdx.x;
    bool mine = false;
    int off = 0, n = 0, ci = -1;
    if (i < sd.n) {
        const long long gi = sd.pt_base + i;
        const int cell = __float_as_int(prec[gi].w);
        const int rk = prank[gi];
        if (cell >= 0 && rk <= 0) {  // the cell's owner (rank 0)
            ci = rk < 0 ? -2 - rk : -1;
            const unsigned long long v = sd.cnt[cell];
            off = (int)(v >> 32);
            n = (int)(v & 0xffffffffull);
            if (n > kSmallCell) {
                const int q = atomicAdd(&hq_count, 1);
                hq_off[q] = off;
                hq_n[q] = n;
                hq_rec[q] = ci;
            } else {
                mine = true;
            }
        }
    }
    if (mine) {
        // the cell's points in ascending order, Kahan-compensated
        const float4 *__restrict__ P = sorted + sd.pt_base + off;
        KSum sx, sy, sz;
        sx.init(); sy.init(); sz.init();
        float mh = 1.0f;
        for (int j = 0; j < n; j++) {
            const float4 p = P[j];
            sx.add(__fsub_rn(p.x, 0.5f));
            sy.add(__fsub_rn(p.y, 0.5f));
            sz.add(__fsub_rn(p.z, 0.5f));
            mh = fminf(mh, p.z);
        }
        const float nf = (float)n;
        const float mx = __fdiv_rn(__fsub_rn(sx.s, sx.c), nf), my = __fdiv_rn(__fsub_rn(sy.s, sy.c), nf);
        const float mz = __fdiv_rn(__fsub_rn(sz.s, sz.c), nf);
        KSum cxx, cxy, cxz, cyy, cyz, czz;
        cxx.init(); cxy.init(); cxz.init(); cyy.init(); cyz.init(); czz.init();
        for (int j = 0; j < n; j++) {
            const float4 p = P[j];
            const float ux = __fsub_rn(__fsub_rn(p.x, 0.5f), mx), uy = __fsub_rn(__fsub_rn(p.y, 0.5f), my);
            const float uz = __fsub_rn(__fsub_rn(p.z, 0.5f), mz);
            cxx.add(__fmul_rn(ux, ux));
            cxy.add(__fmul_rn(ux, uy));
            cxz.add(__fmul_rn(ux, uz));
            cyy.add(__fmul_rn(uy, uy));
            cyz.add(__fmul_rn(uy, uz));
            czz.add(__fmul_rn(uz, uz));
        }
        float4 *o = reinterpret_cast<float4 *>(&mom[sd.pt_base + off]);
        o[0] = make_float4(mx, my, mz, nf);
        o[1] = make_float4(__fsub_rn(cxx.s, cxx.c), __fsub_rn(cxy.s, cxy.c), __fsub_rn(cxz.s, cxz.c),
                           __fsub_rn(cyy.s, cyy.c));
        o[2] = make_float4(__fsub_rn(cyz.s, cyz.c), __fsub_rn(czz.s, czz.c), mh, 0.f);
        store_min_h(sd, ci, mh);
    }
    __syncthreads();
    // cells with many points: one warp each, lanes striding over the points with
    // compensated partial sums, combined across the warp
    const int nh = hq_count, lane = threadIdx.x & 31;
    for (int q = threadIdx.x >> 5; q < nh; q += blockDim.x >> 5) {
        const int qo = hq_off[q], qn = hq_n[q];
        const float4 *__restrict__ P = sorted + sd.pt_base + qo;
        KSum sx, sy, sz;
        sx.init(); sy.init(); sz.init();
        float mh = 1.0f;
        for (int j = lane; j < qn; j += 32) {
            const float4 p = P[j];
            sx.add(__fsub_rn(p.x, 0.5f));
            sy.add(__fsub_rn(p.y, 0.5f));
            sz.add(__fsub_rn(p.z, 0.5f));
            mh = fminf(mh, p.z);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mh = fminf(mh, __shfl_xor_sync(0xffffffffu, mh, o));
        const float nf = (float)qn;
        const float mx = __fdiv_rn(warp_sum(__fsub_rn(sx.s, sx.c)), nf);
        const float my = __fdiv_rn(warp_sum(__fsub_rn(sy.s, sy.c)), nf);
        const float mz = __fdiv_rn(warp_sum(__fsub_rn(sz.s, sz.c)), nf);
        KSum cxx, cxy, cxz, cyy, cyz, czz;
        cxx.init(); cxy.init(); cxz.init(); cyy.init(); cyz.init(); czz.init();
        for (int j = lane; j < qn; j += 32) {
            const float4 p = P[j];
            const float ux = __fsub_rn(__fsub_rn(p.x, 0.5f), mx), uy = __fsub_rn(__fsub_rn(p.y, 0.5f), my);
            const float uz = __fsub_rn(__fsub_rn(p.z, 0.5f), mz);
            cxx.add(__fmul_rn(ux, ux));
            cxy.add(__fmul_rn(ux, uy));
            cxz.add(__fmul_rn(ux, uz));
            cyy.add(__fmul_rn(uy, uy));
            cyz.add(__fmul_rn(uy, uz));
            czz.add(__fmul_rn(uz, uz));
        }
        const float c0 = warp_sum(__fsub_rn(cxx.s, cxx.c)), c1 = warp_sum(__fsub_rn(cxy.s, cxy.c));
        const float c2 = warp_sum(__fsub_rn(cxz.s, cxz.c)), c3 = warp_sum(__fsub_rn(cyy.s, cyy.c));
        const float c4 = warp_sum(__fsub_rn(cyz.s, cyz.c)), c5 = warp_sum(__fsub_rn(czz.s, czz.c));
        if (lane == 0) {
            float4 *o = reinterpret_cast<float4 *>(&mom[sd.pt_base + qo]);
            o[0] = make_float4(mx, my, mz, nf);
            o[1] = make_float4(c0, c1, c2, c3);
            o[2] = make_float4(c4, c5, mh, 0.f);
            store_min_h(sd, hq_rec[q], mh);
        }
    }
}

// Chan update of the running neighbourhood statistics with one cell's moments,
// the cell mean shifted into this voxel's frame (centred on the voxel centre)
struct NbAcc {
    float n, m0, m1, m2, C0, C1, C2, C3, C4, C5;
    __device__ __forceinline__ void init() { n = m0 = m1 = m2 = C0 = C1 = C2 = C3 = C4 = C5 = 0.f; }
    __device__ __forceinline__ void add(const CellMom &cm, int dx, int dy, int dz) {
        const float b0 = __fadd_rn(cm.m[0], (float)dx), b1 = __fadd_rn(cm.m[1], (float)dy);
        const float b2 = __fadd_rn(cm.m[2], (float)dz);
        const float nb = cm.n, nn = __fadd_rn(n, nb);
        const float d0 = __fsub_rn(b0, m0), d1 = __fsub_rn(b1, m1), d2 = __fsub_rn(b2, m2);
        const float wb = __fdiv_rn(nb, nn);
        const float f = __fmul_rn(n, wb);  // n * nb / (n + nb)
        m0 = __fadd_rn(m0, __fmul_rn(d0, wb));
        m1 = __fadd_rn(m1, __fmul_rn(d1, wb));
        m2 = __fadd_rn(m2, __fmul_rn(d2, wb));
        C0 = __fadd_rn(__fadd_rn(C0, cm.c[0]), __fmul_rn(__fmul_rn(d0, d0), f));
        C1 = __fadd_rn(__fadd_rn(C1, cm.c[1]), __fmul_rn(__fmul_rn(d0, d1), f));
        C2 = __fadd_rn(__fadd_rn(C2, cm.c[2]), __fmul_rn(__fmul_rn(d0, d2), f));
        C3 = __fadd_rn(__fadd_rn(C3, cm.c[3]), __fmul_rn(__fmul_rn(d1, d1), f));
        C4 = __fadd_rn(__fadd_rn(C4, cm.c[4]), __fmul_rn(__fmul_rn(d1, d2), f));
        C5 = __fadd_rn(__fadd_rn(C5, cm.c[5]), __fmul_rn(__fmul_rn(d2, d2), f));
        n = nn;
    }
    // Chan combination with another partial sum in the same voxel frame
    __device__ __forceinline__ void merge(const NbAcc &o) {
        if (o.n == 0.f) return;
        if (n == 0.f) {
            *this = o;
            return;
        }
        const float nn = __fadd_rn(n, o.n);
        const float d0 = __fsub_rn(o.m0, m0), d1 = __fsub_rn(o.m1, m1), d2 = __fsub_rn(o.m2, m2);
        const float wb = __fdiv_rn(o.n, nn);
        const float f = __fmul_rn(n, wb);
        m0 = __fadd_rn(m0, __fmul_rn(d0, wb));
        m1 = __fadd_rn(m1, __fmul_rn(d1, wb));
        m2 = __fadd_rn(m2, __fmul_rn(d2, wb));
        C0 = __fadd_rn(__fadd_rn(C0, o.C0), __fmul_rn(__fmul_rn(d0, d0), f));
        C1 = __fadd_rn(__fadd_rn(C1, o.C1), __fmul_rn(__fmul_rn(d0, d1), f));
        C2 = __fadd_rn(__fadd_rn(C2, o.C2), __fmul_rn(__fmul_rn(d0, d2), f));
        C3 = __fadd_rn(__fadd_rn(C3, o.C3), __fmul_rn(__fmul_rn(d1, d1), f));
        C4 = __fadd_rn(__fadd_rn(C4, o.C4), __fmul_rn(__fmul_rn(d1, d2), f));
        C5 = __fadd_rn(__fadd_rn(C5, o.C5), __fmul_rn(__fmul_rn(d2, d2), f));
        n = nn;
    }
    __device__ __forceinline__ NbAcc shfl_down(int delta) const {
        NbAcc o;
        o.n = __shfl_down_sync(0xffffffffu, n, delta);
        o.m0 = __shfl_down_sync(0xffffffffu, m0, delta);
        o.m1 = __shfl_down_sync(0xffffffffu, m1, delta);
        o.m2 = __shfl_down_sync(0xffffffffu, m2, delta);
        o.C0 = __shfl_down_sync(0xffffffffu, C0, delta);
        o.C1 = __shfl_down_sync(0xffffffffu, C1, delta);
        o.C2 = __shfl_down_sync(0xffffffffu, C2, delta);
        o.C3 = __shfl_down_sync(0xffffffffu, C3, delta);
        o.C4 = __shfl_down_sync(0xffffffffu, C4, delta);
        o.C5 = __shfl_down_sync(0xffffffffu, C5, delta);
        return o;
    }
    // every field but hit, total (k_assign) and min_h (k_cell_moments)
    __device__ __forceinline__ void store(VoxelRec *r) const {
        float4 *o = reinterpret_cast<float4 *>(r);
        o[0] = make_float4(__fadd_rn(m0, 0.5f), __fadd_rn(m1, 0.5f), __fadd_rn(m2, 0.5f), __fdiv_rn(C0, n));
        o[1] = make_float4(__fdiv_rn(C1, n), __fdiv_rn(C2, n), __fdiv_rn(C3, n), __fdiv_rn(C4, n));
        reinterpret_cast<float2 *>(r)[4] = make_float2(__fdiv_rn(C5, n), n);
    }
};

// E3 = 1: the 3 x 3 x 3 neighbourhood of eigen distances (1, 1), four lanes
// per voxel: lane j of the group sums cells 7j .. 7j + 6 (z-major; the
// voxel's own cell, 13, in lane 1) with every count load issued first, and
// the four partial sums are combined as (0 + 1) + (2 + 3).  E3 = 0: any
// distances, one thread per voxel, cell by cell.
template <int NS, int E3>
__global__ void __launch_bounds__(256) k_voxel_stats(const ProcessConst pc, const __grid_constant__ ScanTable<NS> tab,
                                                    const CellMom *__restrict__ mom) {
    const ScanDesc &sd = tab.s[blockIdx.y];
    const Geom g = pc.g;
    const int C = min(*(volatile int *)&sd.ctr->C, (int)sd.rec_cap);
    const CellMom *__restrict__ M = mom + sd.pt_base;
    if constexpr (E3 != 0) {
        const int lane = (int)lane_id(), sub = lane & 3;
        const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
        const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
        const int XeXe = g.Xe * g.Xe;
        for (int base = warp * 8; base < C; base += nwarps * 8) {  // warp-uniform trip count
            const int c = base + (lane >> 2);
            NbAcc a;
            a.init();
            if (c < C) {
                const int gid = __float_as_int(sd.rec[c].aux[0]);
                const int x = gid % g.X, y = (gid / g.X) % g.X, z = gid / (g.X * g.X);
                const int e0 = (x + g.exy) + (y + g.exy) * g.Xe + (z + g.ez) * XeXe;
                unsigned long long v[7];
#pragma unroll
                for (int j = 0; j < 7; j++) {
                    const int k = sub * 7 + j;
                    const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
                    v[j] = k < 27 ? __ldg(&sd.cnt[e0 + dx + dy * g.Xe + dz * XeXe]) : 0ull;
                }
#pragma unroll
                for (int j = 0; j < 7; j++) {
                    const int k = sub * 7 + j;
                    if (!(v[j] & 0xffffffffull)) continue;
                    const CellMom cm = M[(int)(v[j] >> 32)];
                    a.add(cm, k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1);
                }
            }
            NbAcc o = a.shfl_down(1);
            if (!(sub & 1)) a.merge(o);
            o = a.shfl_down(2);
            if (sub == 0) a.merge(o);
            if (c < C && sub == 0) a.store(&sd.rec[c]);
        }
    } else {
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
            VoxelRec *r = &sd.rec[c];
            const int gid = __float_as_int(r->aux[0]);
            const int x = gid % g.X, y = (gid / g.X) % g.X, z = gid / (g.X * g.X);
            const int e0 = (x + g.exy) + (y + g.exy) * g.Xe + (z + g.ez) * g.Xe * g.Xe;
            NbAcc a;
            a.init();
            for (int dz = -g.ez; dz <= g.ez; dz++)
                for (int dy = -g.exy; dy <= g.exy; dy++)
                    for (int dx = -g.exy; dx <= g.exy; dx++) {
                        const unsigned long long v = sd.cnt[e0 + dx + dy * g.Xe + dz * g.Xe * g.Xe];
                        if (!(v & 0xffffffffull)) continue;
                        const CellMom cm = M[(int)(v >> 32)];
                        a.add(cm, dx, dy, dz);
                    }
            a.store(r);
        }
    }
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
    if (cell >= 0 && prank[gi] <= 0) sd.cnt[cell] = 0ull;  // the owner
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <int NS>
static cudaError_t launch_ns(const ProcessConst &pc, const ScanDesc *table, int total_blocks, int max_n, int dtype,
                             float4 *prec, int *prank, float4 *sorted, CellMom *mom, cudaStream_t st, cudaEvent_t *ev,
                             int bs, cudaEvent_t after_assign, cudaEvent_t after_moments, int part, bool external) {
    ScanTable<NS> tab;
    for (int i = 0; i < NS; i++) tab.s[i] = i < pc.nscans ? table[i] : table[0];
    if (total_blocks < 1) total_blocks = 1;
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], st);
    };
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    if (part == 0 || part == 1) {
        mark(0);
        if (dtype == 1)
            chk(rec_kernel(k_voxelize_trace<double, NS>, dim3(total_blocks), dim3(bs), 0, st, pc, tab, prec, prank));
        else
            chk(rec_kernel(k_voxelize_trace<float, NS>, dim3(total_blocks), dim3(bs), 0, st, pc, tab, prec, prank));
        mark(1);
        if (part == 1) return e != cudaSuccess ? e : cudaGetLastError();
    }
    chk(rec_kernel(k_assign<NS>, dim3(total_blocks), dim3(bs), 0, st, pc, tab, prec, prank));
    if (after_assign) chk(external ? rec_event_external(after_assign, st) : rec_event_internal(after_assign, st));
    mark(2);
    chk(rec_kernel(k_scatter<NS>, dim3(total_blocks), dim3(bs), 0, st, pc, tab, prec, prank, sorted));
    mark(3);
    chk(rec_kernel(k_cell_moments<NS>, dim3(total_blocks), dim3(bs), 0, st, pc, tab, prec, prank, sorted, mom));
    if (after_moments) chk(external ? rec_event_external(after_moments, st) : rec_event_internal(after_moments, st));
    mark(4);
    const bool e3 = pc.g.exy == 1 && pc.g.ez == 1;  // four lanes per voxel
    const long long want = ((e3 ? 4LL : 1LL) * max_n + 255) / 256;
    dim3 gs((unsigned)std::max<long long>(1, std::min<long long>(want, (long long)pc.num_sms * 8)), pc.nscans);
    if (e3) chk(rec_kernel(k_voxel_stats<NS, 1>, gs, dim3(256), 0, st, pc, tab, mom));
    else chk(rec_kernel(k_voxel_stats<NS, 0>, gs, dim3(256), 0, st, pc, tab, mom));
    mark(5);
    chk(rec_kernel(k_cleanup<NS>, dim3(total_blocks), dim3(bs), 0, st, pc, tab, prec, prank));
    mark(6);
    return e != cudaSuccess ? e : cudaGetLastError();
}

// Every process kernel a call can launch, loaded now (see
// preload_combine_kernels).
template <int NS>
static void add_process_kernels(std::vector<const void *> &k) {
    k.push_back(reinterpret_cast<const void *>(k_voxelize_trace<float, NS>));
    k.push_back(reinterpret_cast<const void *>(k_voxelize_trace<double, NS>));
    k.push_back(reinterpret_cast<const void *>(k_assign<NS>));
    k.push_back(reinterpret_cast<const void *>(k_scatter<NS>));
    k.push_back(reinterpret_cast<const void *>(k_cell_moments<NS>));
    k.push_back(reinterpret_cast<const void *>(k_voxel_stats<NS, 0>));
    k.push_back(reinterpret_cast<const void *>(k_voxel_stats<NS, 1>));
    k.push_back(reinterpret_cast<const void *>(k_cleanup<NS>));
}

cudaError_t preload_process_kernels() {
    std::vector<const void *> k;
    add_process_kernels<1>(k);
    add_process_kernels<4>(k);
    add_process_kernels<kMaxBatch>(k);
    for (const void *f : k) {
        cudaFuncAttributes a;
        const cudaError_t e = cudaFuncGetAttributes(&a, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_process(const ProcessConst &pc, const ScanDesc *table, int nscans, int total_blocks, int max_n,
                           int dtype, float4 *prec, int *prank, float4 *sorted, void *moments, cudaStream_t st,
                           cudaEvent_t *ev, int pts_block, cudaEvent_t after_assign, cudaEvent_t after_moments, int part,
                           bool external) {
    CellMom *mom = static_cast<CellMom *>(moments);
    if (part) ev = nullptr;
    if (nscans == 1)
        return launch_ns<1>(pc, table, total_blocks, max_n, dtype, prec, prank, sorted, mom, st, ev, pts_block,
                            after_assign, after_moments, part, external);
    if (nscans <= 4)
        return launch_ns<4>(pc, table, total_blocks, max_n, dtype, prec, prank, sorted, mom, st, ev, pts_block,
                            after_assign, after_moments, part, external);
    return launch_ns<kMaxBatch>(pc, table, total_blocks, max_n, dtype, prec, prank, sorted, mom, st, ev, pts_block,
                                after_assign, after_moments, part, external);
}

}  // namespace gvom
