// Map-combine kernels: Gvom.combine_maps (scripts/gvom.py:222-393).
//
//   k_merge    one thread per (x, y, z chunk of 4-16 planes): merges every
//              ring slot (slot order) and the previous combined map with
//              their ego shifts and the clearing rule (scripts/gvom.py:
//              1009-1063) into the combined index map, addressed by voxel id
//              so nothing is allocated; lists the occupied voxels and leaves
//              the lowest occupied / known-free z of each chunk.
//   k_merge_counts  one thread per listed occupied voxel: the sources' hit
//              and total sums and lowest in-voxel height (scripts/gvom.py:
//              888-980), all the columns pass reads
//   k_merge_stats  one thread per listed occupied voxel: Chan merge of the
//              statistics (scripts/gvom.py:926-980) and eigenvalues
//              (scripts/gvom.py:1423-1487)
//   k_columns  one thread per column: height (lowest occupied voxel or the
//              robot disc), inferred height (lowest known-free voxel) and the
//              positive-obstacle band density (scripts/gvom.py:515-590)
//   k_maps2d   one thread per cell on a shared-memory tile with a 15-cell
//              halo: slope / roughness, guessed height delta, positive,
//              negative and visibility maps (scripts/gvom.py:444-805)
//   debug      make_debug_voxel_map / height / inferred exporters
//              (scripts/gvom.py:395-503)
//
// GB300's float64 rate is a small fraction of its float32 rate, so integer
// and threshold decisions are taken in float32 wherever an error bound shows
// the float64 result cannot differ, and fall back to the reference's float64
// sequence only near a boundary.
#include "gvom_internal.cuh"

namespace gvom {

constexpr int kOcc = 0x7fffffff;

// Doubles compared and widened on their bit patterns: a float64 warp
// instruction holds this part's slow float64 pipe for as long as any other,
// so conversions and compares stay off it.

// a == b for doubles that are not NaN: equal bits, or +0 against -0
__device__ __forceinline__ bool same_double(double a, double b) {
    const unsigned long long x = (unsigned long long)__double_as_longlong(a);
    const unsigned long long y = (unsigned long long)__double_as_longlong(b);
    return x == y || ((x | y) << 1) == 0;
}

// a signed key that orders doubles that are not NaN as < does, except that
// -0 sorts below +0
__device__ __forceinline__ long long double_order(double a) {
    const long long b = __double_as_longlong(a);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// (double)f: a normal float's bits moved into place (exponent rebiased by
// 1023 - 127); zero, subnormals, inf and NaN take the conversion instruction
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)f;
    return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) |
                                            ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// ---------------------------------------------------------------------------
// k_merge
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// eigenvalues (scripts/gvom.py:1423-1487): cyclic Jacobi in float32, which is
// backward stable -- every eigenvalue, and the gap between nearly equal ones
// (which the closed form loses), is within a few ulp of |A|.  Near-degenerate
// voxels (smallest / largest eigenvalue below 1e-6) with a well-separated
// middle eigenvalue get the smallest one in float64 from the determinant:
// l2 = det(A) / (l0 l1).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void jacobi_rot(float &app, float &aqq, float &apq, float &arp, float &arq) {
    if (apq == 0.0f) return;
    const float theta = __fdividef(aqq - app, 2.0f * apq);
    float t;
    if (fabsf(theta) > 1.0e18f) t = __fdividef(0.5f, theta);
    else t = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
    const float c = rsqrtf(t * t + 1.0f);
    const float s = t * c;
    const float tau = __fdividef(s, 1.0f + c);
    app -= t * apq;
    aqq += t * apq;
    apq = 0.0f;
    const float rp = arp, rq = arq;
    arp = rp - s * (rq + tau * rp);
    arq = rq + s * (rp - tau * rq);
}

__device__ __forceinline__ void eigen3(const float C[6], float e[3]) {
    float a00 = C[0], a01 = C[1], a02 = C[2], a11 = C[3], a12 = C[4], a22 = C[5];
    const float scale = fabsf(a00) + fabsf(a11) + fabsf(a22) + fabsf(a01) + fabsf(a02) + fabsf(a12);
    const float tol = 2.0e-7f * scale;
#pragma unroll 1
    for (int sweep = 0; sweep < 8; sweep++) {
        if (fabsf(a01) + fabsf(a02) + fabsf(a12) <= tol) break;
        jacobi_rot(a00, a11, a01, a02, a12);
        jacobi_rot(a00, a22, a02, a01, a12);
        jacobi_rot(a11, a22, a12, a01, a02);
    }
    float l0 = a00, l1 = a11, l2 = a22, t;
    if (l0 < l1) { t = l0; l0 = l1; l1 = t; }
    if (l1 < l2) { t = l1; l1 = l2; l2 = t; }
    if (l0 < l1) { t = l0; l0 = l1; l1 = t; }
    if (!(fabsf(l2) >= 1e-6f * fabsf(l0)) && fabsf(l1) >= 1e-6f * fabsf(l0)) {
        const double b00 = C[0], b01 = C[1], b02 = C[2], b11 = C[3], b12 = C[4], b22 = C[5];
        const double det = b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) + b02 * (b01 * b12 - b11 * b02);
        l2 = (float)(det / ((double)l0 * (double)l1));
    }
    e[0] = l0;
    e[1] = l1;
    e[2] = l2;
}

// Chan merge of every occupied source voxel, in source order, into the
// combined record at `vid` (scripts/gvom.py:926-980), float32, then its
// eigenvalues.  The sources' compact indices are gathered first and the
// records loaded kMergeChunk at a time, so the loads of a chunk overlap.
constexpr int kMergeChunk = 4;

template <int NSRC>
__device__ __forceinline__ void merge_voxel(const MergeParams &mp, int vid) {
    const int X = mp.g.X, Z = mp.g.Z;
    const int x = vid % X, y = (vid / X) % X, z = vid / (X * X);
    int o[NSRC];
#pragma unroll
    for (int s = 0; s < NSRC; s++) {
        o[s] = -1;
        if (s < mp.nsrc) {
            const int xs = x + mp.src[s].dx, ys = y + mp.src[s].dy, zs = z + mp.src[s].dz;
            if ((unsigned)xs < (unsigned)X && (unsigned)ys < (unsigned)X && (unsigned)zs < (unsigned)Z)
                o[s] = __ldg(&mp.src[s].idx[xs + ys * X + zs * X * X]);
        }
    }
    float n = 0.f, m0 = 0.f, m1 = 0.f, m2 = 0.f;
    float C[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int s0 = 0; s0 < NSRC; s0 += kMergeChunk) {
        float4 ra[kMergeChunk], rb[kMergeChunk], rc[kMergeChunk], rd[kMergeChunk];
#pragma unroll
        for (int j = 0; j < kMergeChunk; j++) {
            const int s = s0 + j;
            if (s < NSRC && o[s] >= 0) {
                const float4 *p = reinterpret_cast<const float4 *>(&mp.src[s].rec[o[s]]);
                ra[j] = __ldg(p);
                rb[j] = __ldg(p + 1);
                rc[j] = __ldg(p + 2);
                rd[j] = __ldg(p + 3);
            }
        }
#pragma unroll
        for (int j = 0; j < kMergeChunk; j++) {
            const int s = s0 + j;
            if (!(s < NSRC && o[s] >= 0)) continue;
            // ra = mean0 mean1 mean2 xx | rb = xy xz yy yz | rc = zz count hit total | rd = minh aux
            const float4 a = ra[j], bq = rb[j], cc = rc[j], d = rd[j];
            const float n2 = cc.y;
            const float o_m[3] = {a.x, a.y, a.z};
            const float o_c[6] = {a.w, bq.x, bq.y, bq.z, bq.w, cc.x};
            const float den = __fadd_rn(n, n2);
            // one rounded reciprocal per source instead of nine divisions (the
            // merged statistics are compared at a tolerance, not bit for bit)
            const float inv = __frcp_rn(den);
            const float nm0 = __fmul_rn(__fadd_rn(__fmul_rn(m0, n), __fmul_rn(o_m[0], n2)), inv);
            const float nm1 = __fmul_rn(__fadd_rn(__fmul_rn(m1, n), __fmul_rn(o_m[1], n2)), inv);
            const float nm2 = __fmul_rn(__fadd_rn(__fmul_rn(m2, n), __fmul_rn(o_m[2], n2)), inv);
            const float cm[3] = {m0, m1, m2};
            const float mn[3] = {nm0, nm1, nm2};
            const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
            for (int t = 0; t < 6; t++) {
                const float t1 = __fmul_rn(n, C[t]);
                const float t2 = __fmul_rn(n2, o_c[t]);
                const float t3 =
                    __fmul_rn(__fmul_rn(n, __fsub_rn(cm[pa[t]], mn[pa[t]])), __fsub_rn(cm[pb[t]], mn[pb[t]]));
                const float t4 =
                    __fmul_rn(__fmul_rn(n2, __fsub_rn(o_m[pa[t]], mn[pa[t]])), __fsub_rn(o_m[pb[t]], mn[pb[t]]));
                C[t] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(t1, t2), t3), t4), inv);
            }
            m0 = nm0;
            m1 = nm1;
            m2 = nm2;
            n = den;
            (void)d;
        }
    }
    float e[3];
    eigen3(C, e);
    // every field but hit, total and min_h, which k_merge_counts writes
    float *out = reinterpret_cast<float *>(&mp.out_rec[vid]);
    reinterpret_cast<float4 *>(out)[0] = make_float4(m0, m1, m2, C[0]);
    reinterpret_cast<float4 *>(out)[1] = make_float4(C[1], C[2], C[3], C[4]);
    reinterpret_cast<float2 *>(out)[4] = make_float2(C[5], n);
    out[13] = e[0];
    reinterpret_cast<float2 *>(out)[7] = make_float2(e[1], e[2]);
}

// hit and total counts (sums) and the lowest in-voxel height (minimum) of a
// listed voxel over its sources -- everything the columns pass reads, so the
// 2-D maps need not wait for the statistics merge
template <int NSRC>
__device__ __forceinline__ void merge_counts(const MergeParams &mp, int vid) {
    const int X = mp.g.X, Z = mp.g.Z;
    const int x = vid % X, y = (vid / X) % X, z = vid / (X * X);
    int o[NSRC];
#pragma unroll
    for (int s = 0; s < NSRC; s++) {
        o[s] = -1;
        if (s < mp.nsrc) {
            const int xs = x + mp.src[s].dx, ys = y + mp.src[s].dy, zs = z + mp.src[s].dz;
            if ((unsigned)xs < (unsigned)X && (unsigned)ys < (unsigned)X && (unsigned)zs < (unsigned)Z)
                o[s] = __ldg(&mp.src[s].idx[xs + ys * X + zs * X * X]);
        }
    }
    int hit = 0, total = 0;
    float minh = 1.0f;
#pragma unroll
    for (int s = 0; s < NSRC; s++) {
        if (!(s < NSRC && o[s] >= 0)) continue;
        const VoxelRec *r = &mp.src[s].rec[o[s]];
        const int2 ht = __ldg(reinterpret_cast<const int2 *>(&r->hit));
        hit += ht.x;
        total += ht.y;
        minh = fminf(minh, __ldg(&r->min_h));
    }
    VoxelRec *out = &mp.out_rec[vid];
    *reinterpret_cast<int2 *>(&out->hit) = make_int2(hit, total);
    out->min_h = minh;
}

// k_merge: every thread decides its ZC voxels (index merge), writes the
// combined index map and queues occupied voxels in shared memory; the block
// appends its queue to the global list of occupied voxels (one atomic).
// k_merge_stats then merges the listed voxels' statistics with full warps
// (occupied voxels are sparse: merging in place would run one lane per warp
// and hold the whole block on that lane's dependent loads).
template <int NSRC, int kZC>
__global__ void __launch_bounds__(256) k_merge(const __grid_constant__ MergeParams mp) {
    __shared__ int queue[256 * kZC];
    __shared__ int qn;
    const int X = mp.g.X, Z = mp.g.Z;
    // a block: 256 consecutive x of one row (eight warps of 32), so that each
    // plane of a source is read as one contiguous 1 KB segment
    const int x = blockIdx.x * 256 + threadIdx.y * 32 + threadIdx.x;
    const int y = blockIdx.y;
    const int z0 = blockIdx.z * kZC;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const bool col = x < X && y < X;
    const int plane = X * X;
    if (tid == 0) qn = 0;
    // index merge, source by source in source order (scripts/gvom.py:242-298).
    // The reference's state per plane, c, is -1 (unknown), a pass count <= -2
    // (free) or occupied: a source's occupied entry (>= 0) makes c occupied,
    // a free entry o (<= -2) adds o + 1, and neither acts once c is occupied.
    // A ring slot's step is held here as two ints: occ, the AND of the
    // entries merged so far (its sign bit clears once an entry was >= 0), and
    // cnt = -1 + the sum of min(o, -1) + 1 over them (o = -1 and o >= 0 add
    // nothing).  While no entry was occupied c = cnt, and an occupied c
    // becomes the voxel id whatever cnt holds -- the same result in three
    // integer operations per entry.  Entries outside a shifted source read as
    // -1, which changes neither.  The previous combined map applies its
    // clearing rule on c itself.  A source's kZC loads are independent.
    int occ[kZC], cnt[kZC];
#pragma unroll
    for (int k = 0; k < kZC; k++) {
        occ[k] = -1;
        cnt[k] = -1;
    }
    // up to kG sources' loads are issued together (kG * kZC in flight per
    // thread), then merged in source order
    constexpr int kG = NSRC < 5 ? NSRC : 5;
#pragma unroll
    for (int s0 = 0; s0 < NSRC; s0 += kG) {
        if (s0 >= mp.nsrc) break;
        int vs[kG][kZC];
#pragma unroll
        for (int j = 0; j < kG; j++) {
            const int s = s0 + j;
            bool in = s < NSRC && s < mp.nsrc;
            int klo = 0, khi = 0, off0 = 0;
            const int *base = mp.src[0].idx;
            if (in) {
                const MergeSrc &src = mp.src[s];
                const int xs = x + src.dx, ys = y + src.dy;
                in = col && (unsigned)xs < (unsigned)X && (unsigned)ys < (unsigned)X;
                // planes k with 0 <= z0 + k + dz < Z (and z0 + k < Z)
                klo = max(0, -(z0 + src.dz));
                khi = min(min(kZC, Z - z0), Z - z0 - src.dz);
                base = src.idx;
                off0 = xs + ys * X + (z0 + src.dz) * plane;  // plane k at off0 + k plane, read for klo <= k < khi
            }
#pragma unroll
            for (int k = 0; k < kZC; k++) vs[j][k] = (in && k >= klo && k < khi) ? __ldg(base + (off0 + k * plane)) : -1;
        }
#pragma unroll
        for (int j = 0; j < kG; j++) {
            const int s = s0 + j;
            if (s >= NSRC || s >= mp.nsrc) break;
            if (mp.src[s].is_last) {
                // previous combined map: an occupied voxel comes back only if at most
                // 10 new rays passed through it (scripts/gvom.py:1058)
#pragma unroll
                for (int k = 0; k < kZC; k++) {
                    const int o = vs[j][k];
                    int c = occ[k] >= 0 ? kOcc : cnt[k];
                    if (c <= -1) c = (o >= 0) ? (c >= -11 ? kOcc : c) : (o < -1 ? c + o + 1 : c);
                    occ[k] = c == kOcc ? 0 : -1;
                    cnt[k] = c;
                }
            } else {
#pragma unroll
                for (int k = 0; k < kZC; k++) {
                    occ[k] &= vs[j][k];
                    cnt[k] += min(vs[j][k], -1) + 1;
                }
            }
        }
    }
    int cmb[kZC];  // c: kOcc or the pass count
#pragma unroll
    for (int k = 0; k < kZC; k++) cmb[k] = occ[k] >= 0 ? kOcc : cnt[k];
    __syncthreads();
    int occ_z = Z, free_z = Z;
#pragma unroll
    for (int k = 0; k < kZC; k++) {
        const int z = z0 + k;
        int comb = cmb[k];
        const bool occ = col && z < Z && comb == kOcc;
        const unsigned m = __ballot_sync(0xffffffffu, occ);
        if (m) {
            int base = 0;
            if (threadIdx.x == 0) base = atomicAdd(&qn, __popc(m));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (occ) queue[base + __popc(m & ((1u << threadIdx.x) - 1u))] = x + y * X + z * plane;
        }
        if (col && z < Z) {
            const int vid = x + y * X + z * plane;
            if (occ) {
                comb = vid;
                if (occ_z == Z) occ_z = z;
            } else if (comb < -1 && free_z == Z) {
                free_z = z;
            }
            mp.out_idx[vid] = comb;
        }
    }
    if (col) mp.colinfo[blockIdx.z * plane + y * X + x] = make_int2(occ_z, free_z);
    __syncthreads();
    const int n_q = qn;
    __shared__ int lbase;
    if (tid == 0) lbase = n_q ? atomicAdd(mp.out_count, n_q) : 0;
    __syncthreads();
    for (int i = tid; i < n_q; i += 256) mp.list[lbase + i] = queue[i];
}

template <int NSRC>
#ifndef GVOM_MERGE_STATS_MINB
#define GVOM_MERGE_STATS_MINB 1  // minimum resident blocks per SM asked of the register allocator
#endif
__global__ void __launch_bounds__(256, GVOM_MERGE_STATS_MINB) k_merge_stats(const __grid_constant__ MergeParams mp) {
    const int n = *mp.out_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        merge_voxel<NSRC>(mp, mp.list[i]);
}

template <int NSRC>
__global__ void __launch_bounds__(256) k_merge_counts(const __grid_constant__ MergeParams mp) {
    const int n = *mp.out_count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        merge_counts<NSRC>(mp, mp.list[i]);
}

// ---------------------------------------------------------------------------
// k_columns
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool near_integer(float w, float margin) {
    const float f = floorf(w);
    return !(w - f > margin && f + 1.0f - w > margin);
}

// (int)(dens / nn * 100.0) of the positive-obstacle band (scripts/gvom.py:
// 548-555) in float64, dens and nn >= 0 integer-valued sums (exact): the two
// roundings move the exact value 100 dens / nn by at most 2.3e-16 of itself.
// Below 2^44 a non-integer value lies at least 1 / nn from every integer,
// more than that, so its truncation is the integer quotient; an integer value
// (and a larger one) takes the float64 sequence, whose rounding can fall just
// below it.  nn > 0.
__device__ __forceinline__ int band_density(long long dens, long long nn) {
    const long long P = 100 * dens;
    long long q = -1;
    if (P < (1LL << 32) && nn < (1LL << 32)) {  // 32-bit division where it fits
        const unsigned p32 = (unsigned)P, n32 = (unsigned)nn;
        if (p32 % n32 != 0u) q = p32 / n32;
    } else if (P < (1LL << 44) && P % nn != 0) {
        q = P / nn;
    }
    return q >= 0 ? (int)q : (int)__dmul_rn(__ddiv_rn((double)dens, (double)nn), 100.0);
}

__global__ void __launch_bounds__(256) k_columns(const __grid_constant__ ColumnParams cp) {
    const int X = cp.X, Z = cp.Z;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * 8 + threadIdx.y;
    if (x >= X || y >= X) return;
    const int plane = X * X;
    int occ_z = Z, free_z = Z;
#pragma unroll 8
    for (int ch = 0; ch * cp.planes < Z; ch++) {
        const int2 ci = cp.colinfo[ch * plane + y * X + x];
        if (occ_z == Z) occ_z = ci.x;
        if (free_z == Z) free_z = ci.y;
    }
    double h = -1000.0;
    int zl = -1;
    float ml = 0.f;
    int pd = 0;
    if (occ_z < Z) {
        // lowest occupied voxel -> height (scripts/gvom.py:572-576)
        const float minh = cp.rec[x + y * X + occ_z * plane].min_h;
        h = __dmul_rn(__dadd_rn(__dadd_rn(widen(minh), widen((float)occ_z)), cp.co[2]), cp.z_res);
        zl = occ_z;
        ml = minh;
        // positive-obstacle band (scripts/gvom.py:529-555):
        // zmin = floor((h + pos_thr) / z_res - oz) + 1, zmax = floor((h + robot_h) / z_res - oz);
        // in exact arithmetic these are occ_z + floor(minh + thr / z_res) (+1)
        int zmin, zmax;
        const float wmin = minh + cp.pthr_v, wmax = minh + cp.robh_v;
        if (!near_integer(wmin, 1e-4f) && !near_integer(wmax, 1e-4f)) {
            zmin = occ_z + (int)floorf(wmin) + 1;
            zmax = occ_z + (int)floorf(wmax);
        } else {
            const double mino = __dadd_rn(h, cp.pos_thr), maxo = __dadd_rn(h, cp.robot_h);
            const double fmin = floor(__dsub_rn(__ddiv_rn(mino, cp.z_res), cp.co[2]));
            const double fmax = floor(__dsub_rn(__ddiv_rn(maxo, cp.z_res), cp.co[2]));
            zmin = (fabs(fmin) < 1e9) ? (int)fmin + 1 : -1;
            zmax = (fabs(fmax) < 1e9) ? (int)fmax : -1;
        }
        if (zmin >= 0 && zmin < Z && zmax >= 0 && zmax < Z) {
            long long nn = 0, dens = 0;
            // 16 planes at a time: every index load, then every record load, in flight together
            for (int z0 = zmin; z0 <= zmax; z0 += 16) {
                int idx[16];
#pragma unroll
                for (int j = 0; j < 16; j++) idx[j] = z0 + j <= zmax ? cp.idx[x + y * X + (z0 + j) * plane] : -1;
                float2 ht[16];
#pragma unroll
                for (int j = 0; j < 16; j++)
                    ht[j] = idx[j] >= 0 ? reinterpret_cast<const float2 *>(&cp.rec[idx[j]])[5]  // hit, total
                                        : make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int hit = __float_as_int(ht[j].x);
                    if (hit > 10) {
                        nn += __float_as_int(ht[j].y);
                        dens += hit;
                    }
                }
            }
            if (nn > 0) pd = band_density(dens, nn);
        }
    } else {
        // robot disc (scripts/gvom.py:566-570): decided in float32 unless near the rim
        const float xp = cp.base_xf + (float)x * cp.res_f, yp = cp.base_yf + (float)y * cp.res_f;
        const float s = xp * xp + yp * yp;
        bool in;
        if (fabsf(s - cp.r2_f) > 1e-3f * cp.r2_f + 1e-4f) {
            in = s <= cp.r2_f;
        } else {
            const double xd = __dsub_rn(__dmul_rn(__dadd_rn(cp.co[0], (double)x), cp.xy_res), cp.ego[0]);
            const double yd = __dsub_rn(__dmul_rn(__dadd_rn(cp.co[1], (double)y), cp.xy_res), cp.ego[1]);
            in = __dadd_rn(__dmul_rn(xd, xd), __dmul_rn(yd, yd)) <= cp.robot_r2;
        }
        if (in) h = cp.disc_h;
    }
    const double ih = free_z < Z ? __dmul_rn(__dadd_rn(widen((float)free_z), cp.co[2]), cp.z_res) : -1000.0;
    const int m2d = x * X + y;
    cp.height[m2d] = h;
    cp.inferred[m2d] = ih;
    cp.pos_density[m2d] = pd;
    cp.zlow[m2d] = zl;
    cp.mlow[m2d] = ml;
}

// gathers occupied combined records in ascending voxel-id order (state export)
__global__ void k_gather_records(const VoxelRec *__restrict__ rec, const int *__restrict__ vids, int n,
                                 VoxelRec *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = rec[vids[i]];
}

// ---------------------------------------------------------------------------
// k_maps2d: tile of 8 (x) by 32 (y) cells plus a 15-cell halo in shared
// memory: heights, lowest occupied z / in-voxel height of each column,
// known-height flags and, per column / row, the next known cell (so each
// ring segment of the guess search is one lookup).
// ---------------------------------------------------------------------------
constexpr int kHalo = 15;
constexpr long long kMinus1000Bits = (long long)0xC08F400000000000ULL;  // -1000.0

// h > -1000.0 on the bit pattern (no float64 compare)
__device__ __forceinline__ bool height_known(double h) {
    const long long b = __double_as_longlong(h);
    return b >= 0 || (b & 0x7fffffffffffffffLL) < 0x408F400000000000LL;  // |h| < 1000
}

// atan2(a, im) with im = RN(1/m), m = sqrt(a0^2 + a1^2 + 1) >= 1: atan2f of
// the rounded arguments (relative error a few 1e-7); for |a| below the
// float32 normal range the angle is a * m to within (a m)^2 / 3 relative.
__device__ __forceinline__ double slope_angle(double a, double m, double im) {
    if (fabs(a) < 1e-30) return __dmul_rn(a, m);
    return (double)atan2f((float)a, (float)im);
}

// log and atan2 of exact float64 values in float32: the results are compared
// at 1e-3 relative, and the float32 functions stay within a few 1e-7 relative
// here.  log(err) near err = 1 goes through log1p of the exact err - 1;
// values outside the float32 range keep float64.  err = 0 stays 0.
__device__ __forceinline__ double rough_of(double err) {
    if (err > 0.0) {
        if (err >= 0.5 && err <= 2.0) return (double)log1pf((float)__dsub_rn(err, 1.0));
        if (err > 1e-30 && err < 1e30) return (double)logf((float)err);
        return log(err);
    }
    return err;
}

// The reference's mean of n copies of the coordinate c * res (float64,
// summed in order, then divided by n) equals c * res exactly.
__device__ __forceinline__ bool axis_mean_exact(int c, double res, int n) {
    const double v = __dmul_rn((double)c, res);
    double sum = 0.0;
    for (int j = 0; j < n; j++) sum = __dadd_rn(sum, v);
    return __ddiv_rn(sum, (double)n) == v;
}

// __calculate_slope (scripts/gvom.py:717-805) in the reference's float64
// operation order up to the final log / atan2, for four queued cells per
// warp, eight lanes (g = 0..7) per cell.  The reference forms every point's
// x * res, y * res and their offsets from the means point by point; the
// neighbourhood has at most three distinct x and three distinct y, so those
// values (and x * x, y * y, a0 * x, a1 * y of the offsets) are formed once
// per column / row with the same rounded operations and reused.  Sums run
// over the known neighbours in the reference's order (x major, y minor).
//
// This part's float64 pipe holds a warp instruction as long with one active
// lane as with 32, so the independent operations of each step are spread
// over the cell's lanes and one instruction does up to eight of them; values
// move between lanes by shuffles.  Each value is the same IEEE operation on
// the same operands as the one-lane sequence.  Lane roles:
//   coordinates  lanes 0-2: x of column a, (xl + a) res; lanes 3-5: y of row b
//   means        lane 0: x, lane 1: y, lane 2: z
//   offsets      lanes 0-2: dx[a] = x[a] - mean x; lanes 3-5: dy[b]
//   neighbours   lane g: neighbour g = (g / 3, g % 3); neighbour 8 on all lanes
//   sums         lanes 0-4: sxx, sxy, sxz, syy, syz
//   solve        lane 0: det, lane 1: a0, lane 2: a1
// Called by the whole warp, converged.  A group with `active` false has no
// cell (x0, y0 name a cell of the tile, so its loads stay in bounds) and its
// result is not used.  Returns, in lane 0 of the group, the roughness, in
// lane 1 the x slope, in lane 2 the y slope.
template <int kSY>
__device__ __forceinline__ double slope_f64_group(const double (*sh)[kSY], const unsigned char (*kn)[kSY], int x0t,
                                                  int y0t, int x0, int y0, bool active, int X, double res, int g) {
    constexpr unsigned kFull = 0xffffffffu;
    const int xl = max(0, x0 - 1), xh = min(X, x0 + 2), yl = max(0, y0 - 1), yh = min(X, y0 + 2);
    // known neighbours (bit j: neighbour (j / 3, j % 3)) and their heights;
    // hzg: neighbour g's height
    unsigned km = 0;
    double hz[9], hzg = 0.0;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int sx = xl + j / 3 - x0t + kHalo, sy = yl + j % 3 - y0t + kHalo;
        const bool k = active && xl + j / 3 < xh && yl + j % 3 < yh && kn[sx][sy];
        km |= (unsigned)k << j;
        hz[j] = k ? sh[sx][sy] : 0.0;
        if (j == g) hzg = hz[j];
    }
    const double pv = __dmul_rn(widen((float)(g < 3 ? xl + g : yl + min(g - 3, 2))), res);
    double px[3], py[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        px[a] = __shfl_sync(kFull, pv, a, 8);
        py[a] = __shfl_sync(kFull, pv, 3 + a, 8);
    }
    double acc = 0.0;
    int n = 0;
#pragma unroll
    for (int j = 0; j < 9; j++)
        if ((km >> j) & 1u) {
            acc = __dadd_rn(acc, g == 0 ? px[j / 3] : g == 1 ? py[j % 3] : hz[j]);
            n++;
        }
    // a group without a cell (n = 0) and a singular fit (det = 0) divide by
    // 1 instead: a zero divisor would send the whole warp's division down its
    // slow path, and those quotients are not used (a cell has n >= 3)
    const double dn = widen((float)max(n, 1));
    const double mean = __ddiv_rn(acc, dn);
    const double mx = __shfl_sync(kFull, mean, 0, 8), my = __shfl_sync(kFull, mean, 1, 8);
    const double mz = __shfl_sync(kFull, mean, 2, 8);
    const double d = __dsub_rn(pv, g < 3 ? mx : my);
    const double dd = __dmul_rn(d, d);
    // neighbour g's residual height and products, then neighbour 8's: lane 0
    // dx dy, lane 1 dx dz, lane 2 dy dz
    const double dxg = __shfl_sync(kFull, d, g / 3, 8), dyg = __shfl_sync(kFull, d, 3 + g % 3, 8);
    const double dx2 = __shfl_sync(kFull, d, 2, 8), dy2 = __shfl_sync(kFull, d, 5, 8);
    const double dzg = __dsub_rn(hzg, mz), dz8 = __dsub_rn(hz[8], mz);
    const double pxy = __dmul_rn(dxg, dyg), pxz = __dmul_rn(dxg, dzg), pyz = __dmul_rn(dyg, dzg);
    const double p8 = __dmul_rn(g == 2 ? dy2 : dx2, g == 0 ? dy2 : dz8);
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const double tsq = __shfl_sync(kFull, dd, g == 0 ? j / 3 : 3 + j % 3, 8);  // dx[a]^2 (lane 0), dy[b]^2 (lane 3)
        double txy, txz, tyz;
        if (j < 8) {
            txy = __shfl_sync(kFull, pxy, j, 8);
            txz = __shfl_sync(kFull, pxz, j, 8);
            tyz = __shfl_sync(kFull, pyz, j, 8);
        } else {
            txy = txz = tyz = __shfl_sync(kFull, p8, g == 1 ? 0 : g == 2 ? 1 : 2, 8);
        }
        const double term = (g == 0 || g == 3) ? tsq : g == 1 ? txy : g == 2 ? txz : tyz;
        if ((km >> j) & 1u) s = __dadd_rn(s, term);
    }
    const double sxx = __shfl_sync(kFull, s, 0, 8), sxy = __shfl_sync(kFull, s, 1, 8);
    const double sxz = __shfl_sync(kFull, s, 2, 8), syy = __shfl_sync(kFull, s, 3, 8);
    const double syz = __shfl_sync(kFull, s, 4, 8);
    // det = sxx syy - sxy sxy, a0 = (syy sxz - sxy syz) / det, a1 = (sxx syz - sxy sxz) / det:
    // the six products on lanes 0-5, the three differences on lanes 0-2
    const double fa = g == 0 ? sxx : g == 2 ? syy : g == 4 ? sxx : sxy;
    const double fb = g == 0 ? syy : g == 1 ? sxy : g == 2 ? sxz : g == 3 ? syz : g == 4 ? syz : sxz;
    const double pr = __dmul_rn(fa, fb);
    const double r = __dsub_rn(__shfl_sync(kFull, pr, (2 * g) & 7, 8), __shfl_sync(kFull, pr, (2 * g + 1) & 7, 8));
    const double det = __shfl_sync(kFull, r, 0, 8);
    const bool singular = ((unsigned long long)__double_as_longlong(det) << 1) == 0;  // det == 0
    const double a = __ddiv_rn(r, singular ? 1.0 : det);  // lane 1 a0, lane 2 a1
    const double asq = __dmul_rn(a, a);
    const double m = sqrt(__dadd_rn(__dadd_rn(__shfl_sync(kFull, asq, 1, 8), __shfl_sync(kFull, asq, 2, 8)), 1.0));
    const double an = __ddiv_rn(a, m);  // lane 1 a0 / m, lane 2 a1 / m
    const double a0 = __shfl_sync(kFull, an, 1, 8), a1 = __shfl_sync(kFull, an, 2, 8);
    const double axy = __dmul_rn(g < 3 ? a0 : a1, d);  // lanes 0-2 a0 dx[a], lanes 3-5 a1 dy[b]
    const double eg = __dsub_rn(dzg, __dadd_rn(__shfl_sync(kFull, axy, g / 3, 8), __shfl_sync(kFull, axy, 3 + g % 3, 8)));
    const double e2g = __dmul_rn(eg, eg);
    const double e8 = __dsub_rn(dz8, __dadd_rn(__shfl_sync(kFull, axy, 2, 8), __shfl_sync(kFull, axy, 5, 8)));
    const double e28 = __dmul_rn(e8, e8);
    double err = 0.0;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const double t = j < 8 ? __shfl_sync(kFull, e2g, j, 8) : e28;
        if ((km >> j) & 1u) err = __dadd_rn(err, t);
    }
    const double qv = __ddiv_rn(g == 0 ? err : 1.0, g == 0 ? dn : m);  // lane 0 err / n, lane 1 1 / m
    const double im = __shfl_sync(kFull, qv, 1, 8);
    // det == 0: the reference leaves roughness -1 and the slopes 0 (scripts/gvom.py:769-771)
    if (singular) return g == 0 ? -1.0 : 0.0;
    return g == 0 ? rough_of(qv) : slope_angle(g == 1 ? a0 : a1, m, im);
}

// The block has one thread per cell plus one more warp (kTY = 32: one more
// row of threads; kTY = 16: two) that takes no cell: once the float64 queue
// is complete it drains it, 32 cells per warp instruction, while the cell
// threads run their guess search.  A float64 warp instruction holds the slow
// float64 pipe as long with one lane active as with 32, so the queue goes
// through in as few warp instructions as it can.  Cell warps that finish
// their search early take what is left, also 32 cells at a time.
template <int kTX, int kTY>
__global__ void __launch_bounds__(kTX * kTY + 32) k_maps2d(const __grid_constant__ Maps2DParams mp) {
    constexpr int kSX = kTX + 2 * kHalo, kSY = kTY + 2 * kHalo;
    constexpr int kCells = kTX * kTY, kThreads = kCells + 32;
    static_assert(kSX <= 64 && kSY <= 64 && kCells % 32 == 0 && 32 % kTY == 0, "tile shape");
    __shared__ double sh[kSX][kSY];
    // lowest occupied z and in-voxel height per column for the float32 plane
    // fit; afterwards reused for the results of the float64 queue
    __shared__ __align__(16) unsigned char fit_buf[kSX * kSY * 8];
    int (*szl)[kSY] = reinterpret_cast<int (*)[kSY]>(fit_buf);
    float (*sml)[kSY] = reinterpret_cast<float (*)[kSY]>(fit_buf + kSX * kSY * 4);
    double (*qres)[3] = reinterpret_cast<double (*)[3]>(fit_buf);
    __shared__ int qcell[kTX * kTY];
    __shared__ int qn, qtake;
    __shared__ unsigned char kn[kSX][kSY];
    __shared__ unsigned char nky[kSX][kSY + 2];  // next known y index (in tile coords) at or after sy, kSY if none
    __shared__ unsigned char nkx[kSY][kSX + 2];  // next known x index at or after sx
    const int X = mp.X;
    const int x0t = blockIdx.y * kTX, y0t = blockIdx.x * kTY;
    const int tid = threadIdx.y * kTY + threadIdx.x;
    if (tid == 0) {
        qn = 0;
        qtake = 0;
    }
#pragma unroll
    for (int k = tid; k < kSX * kSY; k += kThreads) {
        const int sx = k / kSY, sy = k % kSY;
        const int gx = x0t + sx - kHalo, gy = y0t + sy - kHalo;
        const bool in = gx >= 0 && gx < X && gy >= 0 && gy < X;
        const int c = gx * X + gy;
        const double hv = in ? mp.height[c] : -1000.0;
        sh[sx][sy] = hv;
        kn[sx][sy] = (in && height_known(hv)) ? 1 : 0;
        szl[sx][sy] = in ? mp.zlow[c] : -1;
        sml[sx][sy] = in ? mp.mlow[c] : 0.f;
    }
    __syncthreads();
    // next-known tables, one warp per row or column: the known flags of up to
    // 64 entries as two ballots, and for each entry the lowest set bit at or
    // after it
    {
        const int lane = tid & 31, warp = tid >> 5;
        for (int r = warp; r < kSX + kSY; r += kThreads / 32) {
            const bool is_row = r < kSX;  // row sx: along y (kSY entries); else column sy: along x (kSX entries)
            const int len = is_row ? kSY : kSX;
            const int fixed = is_row ? r : r - kSX;
            unsigned m[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = h * 32 + lane;
                const bool k = j < len && (is_row ? kn[fixed][j] : kn[j][fixed]);
                m[h] = __ballot_sync(0xffffffffu, k);
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int j = h * 32 + lane;
                if (j >= len) continue;
                const unsigned below = (1u << lane) - 1u;
                int nxt;
                const unsigned a = m[h] & ~below;
                if (a) nxt = h * 32 + __ffs(a) - 1;
                else if (h == 0 && m[1]) nxt = 32 + __ffs(m[1]) - 1;
                else nxt = len;
                if (is_row) nky[fixed][j] = (unsigned char)nxt;
                else nkx[fixed][j] = (unsigned char)nxt;
            }
        }
    }
    __syncthreads();
    const int x0 = x0t + threadIdx.y, y0 = y0t + threadIdx.x;
    const bool cell_thread = tid < kCells;  // the last warp takes no cell
    const bool valid = cell_thread && x0 < X && y0 < X;
    const int tx = threadIdx.y + kHalo, ty = threadIdx.x + kHalo;  // this cell in tile coords
    const int cell = x0 * X + y0;
    const bool known = kn[tx][ty];

    // slope / roughness: a float32 plane fit on the neighbours' height
    // differences (exact sums of a voxel count and an in-voxel fraction, or
    // a float64 difference where a neighbour is a robot-disc height); the
    // reference's float64 sequence where the fit is near a cancellation
    // (singular normal matrix, residual far below the height spread, log near
    // 0, a slope component near 0); closed form where every neighbour has
    // the same height
    double rough = -1.0, slx = 0.0, sly = 0.0;
    float slxf = 0.f, slyf = 0.f;  // the slopes in float32, for the slope gate
    bool need_exact = false;
    {
        const int xl = max(0, x0 - 1), xh = min(X, x0 + 2), yl = max(0, y0 - 1), yh = min(X, y0 + 2);
        int n_good = 0, sxi = 0, syi = 0, sxxi = 0, syyi = 0, sxyi = 0;
        bool all_vox = true, all_eq = true;
        int zr = 0;
        float mr = 0.f;
        double h0 = 0.0;
        int xf = 0, yf = 0;  // the first known neighbour
        for (int xx = xl; xx < xh; xx++)
            for (int yy = yl; yy < yh; yy++) {
                const int sx = xx - x0t + kHalo, sy = yy - y0t + kHalo;
                if (kn[sx][sy]) {
                    if (n_good == 0) {
                        zr = szl[sx][sy];
                        mr = sml[sx][sy];
                        h0 = sh[sx][sy];
                        xf = xx;
                        yf = yy;
                    }
                    all_vox = all_vox && szl[sx][sy] >= 0;
                    all_eq = all_eq && same_double(sh[sx][sy], h0);
                    n_good++;
                    sxi += xx - x0;
                    syi += yy - y0;
                    sxxi += (xx - x0) * (xx - x0);
                    syyi += (yy - y0) * (yy - y0);
                    sxyi += (xx - x0) * (yy - y0);
                }
            }
        // the neighbours' offsets are not collinear (the float64 normal matrix is then regular)
        const int dxx = n_good * sxxi - sxi * sxi, dyy = n_good * syyi - syi * syi, dxy = n_good * sxyi - sxi * syi;
        if (valid && n_good >= 3 && all_eq && dxx * dyy - dxy * dxy != 0) {
            // Every known neighbour has the same height h (the robot disc, or a
            // flat floor): in the float64 sequence every residual height is
            // dz = h - mean(h), so sxz and syz are dz times a sum of rounded
            // offsets from their mean (|sum| < 1e-13 m), the fitted slopes stay
            // below 1e-12 |dz| / res and err = dz^2 (1 + O(1e-13)).  So slope
            // 0 and roughness log(dz^2), with dz from the reference's own
            // sequential mean -- equal to the float64 sequence far inside the
            // 1e-3 tolerance, without its ~350 dependent float64 operations.
            double sum = 0.0;
            for (int j = 0; j < n_good; j++) sum = __dadd_rn(sum, h0);
            const double dz = __dsub_rn(h0, __ddiv_rn(sum, (double)n_good));
            rough = rough_of(__dmul_rn(dz, dz));
            slx = 0.0;
            sly = 0.0;
        } else if (valid && n_good >= 3 && (dxx == 0 || dyy == 0) &&
                   axis_mean_exact(dxx == 0 ? xf : yf, mp.xy_res, n_good)) {
            // every known neighbour in one row (column) of the map, whose float64
            // coordinate the reference's sequential mean gives back exactly: every
            // offset along that axis is 0, so its normal matrix has det = 0 and it
            // leaves roughness -1 and the slopes 0 (scripts/gvom.py:769-771)
            rough = -1.0;
            slx = 0.0;
            sly = 0.0;
        } else if (valid && n_good >= 3) {
            bool exact = false;
            float a0 = 0.f, a1 = 0.f, m = 1.f, err = 0.f, szz = 0.f;
            const float nf = (float)n_good;
            if (!exact) {
                const float res = (float)mp.xy_res, zres = (float)mp.z_res;
                const float cx = (float)sxi / nf, cy = (float)syi / nf;
                // neighbour (a, b) is cell (x0 - 1 + a, y0 - 1 + b); its x offset
                // depends on a only and its y offset on b only
                bool kk[3][3];
                float dzs[3][3], dxa[3], dyb[3];
                float zsum = 0.f;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    dxa[a] = ((float)(a - 1) - cx) * res;
                    dyb[a] = ((float)(a - 1) - cy) * res;
                }
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int b = 0; b < 3; b++) {
                        const int xx = x0 - 1 + a, yy = y0 - 1 + b;
                        const int sx = xx - x0t + kHalo, sy = yy - y0t + kHalo;
                        kk[a][b] = xx >= xl && xx < xh && yy >= yl && yy < yh && kn[sx][sy];
                        // from voxels: an exact count plus a fraction
                        dzs[a][b] = kk[a][b] ? ((sml[sx][sy] - mr) + (float)(szl[sx][sy] - zr)) * zres : 0.f;
                    }
                if (!all_vox) {
                    // with a robot-disc height: the float64 difference, rounded once
#pragma unroll
                    for (int a = 0; a < 3; a++)
#pragma unroll
                        for (int b = 0; b < 3; b++)
                            if (kk[a][b])
                                dzs[a][b] = (float)__dsub_rn(sh[x0 - 1 + a - x0t + kHalo][y0 - 1 + b - y0t + kHalo], h0);
                }
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int b = 0; b < 3; b++)
                        if (kk[a][b]) zsum += dzs[a][b];
                const float zm = zsum / nf;
                float sxx = 0.f, sxy = 0.f, sxz = 0.f, syy = 0.f, syz = 0.f;
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int b = 0; b < 3; b++)
                        if (kk[a][b]) {
                            const float dz = dzs[a][b] - zm;
                            dzs[a][b] = dz;
                            sxx += dxa[a] * dxa[a];
                            sxy += dxa[a] * dyb[b];
                            sxz += dxa[a] * dz;
                            syy += dyb[b] * dyb[b];
                            syz += dyb[b] * dz;
                            szz += dz * dz;
                        }
                const float det = sxx * syy - sxy * sxy;
                exact = !(fabsf(det) > 1e-3f * sxx * syy);
                if (!exact) {
                    a0 = (syy * sxz - sxy * syz) / det;
                    a1 = (sxx * syz - sxy * sxz) / det;
                    m = sqrtf(a0 * a0 + a1 * a1 + 1.0f);
                    a0 /= m;
                    a1 /= m;
#pragma unroll
                    for (int a = 0; a < 3; a++)
#pragma unroll
                        for (int b = 0; b < 3; b++)
                            if (kk[a][b]) {
                                const float e = dzs[a][b] - (a0 * dxa[a] + a1 * dyb[b]);
                                err += e * e;
                            }
                    err /= nf;
                }
            }
            float rf = 0.f, sxf = 0.f, syf = 0.f;
            if (!exact) {
                rf = logf(err);
                const float im = 1.0f / m;
                sxf = atan2f(a0, im);
                syf = atan2f(a1, im);
                // a slope component much smaller than the other is ill-conditioned in any
                // precision: take the reference's float64 sequence for it
                const float big = fmaxf(fabsf(sxf), fabsf(syf)), small = fminf(fabsf(sxf), fabsf(syf));
                // the residual keeps at least 1e-4 of the height spread, so err is
                // good to ~1e-5 relative and log(err) to ~1e-5 absolute: exact where
                // that is not far below 1e-3 of |log err|
                exact = !(err > 1e-4f * (szz / nf)) || fabsf(rf) < 0.1f || small < 5e-3f * big || big < 2e-3f;
            }
            if (exact) {
                need_exact = true;
                qcell[atomicAdd(&qn, 1)] = tid;
            } else {
                rough = widen(rf);
                slx = widen(sxf);
                sly = widen(syf);
                slxf = sxf;
                slyf = syf;
            }
        }
    }
    // cells that need the float64 sequence are compacted into a queue so that
    // whole warps run it, instead of one lane in every warp that has one
    __syncthreads();  // queue complete; szl / sml no longer read (qres reuses their space)
    // the float64 queue, four cells per warp pass (eight lanes each): each
    // warp takes the next four queued cells until none are left (called with
    // the warp converged)
    auto drain = [&]() {
        const int nq = qn, lane = tid & 31;
        while (true) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&qtake, 4);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= nq) break;
            const int q = base + (lane >> 3);
            const bool act = q < nq;
            const int t = act ? qcell[q] : 0;
            const double v = slope_f64_group<kSY>(sh, kn, x0t, y0t, x0t + t / kTY, y0t + t % kTY, act, X, mp.xy_res,
                                                  lane & 7);
            if (act && (lane & 7) < 3) qres[t][lane & 7] = v;
            __syncwarp();
        }
    };
    if (!cell_thread) drain();  // the extra warp starts at once, beside the guess search

    // __guess_height (scripts/gvom.py:592-714), loop-condition and y_nh quirks
    // included; each ring segment is scanned in increasing order, so its first
    // known cell is one lookup in the next-known tables
    double guess = 0.0;
    if (valid && !known && __double_as_longlong(mp.inferred[cell]) != kMinus1000Bits) {
        bool xpd = false, xnd = false, ypd = false, ynd = false;
        bool xpf = false, xnf = false, ypf = false, ynf = false;  // a known height found
        int xp = x0, xn = x0, yp = y0, yn = y0;
        double xph = -1000.0, xnh = -1000.0, yph = -1000.0, ynh = -1000.0;
        int i = 0;
        while (i < 15 && !(xnd && xnd && ypd && ynd)) {
            xp += 1; xn -= 1; yp += 1; yn -= 1;
            i += 1;
            if (!xpd) {
                if (xp < X) {
                    const int lo = max(y0 - i, 0), hi = min(y0 + i, X);  // dy in [-i, i)
                    if (lo < hi) {
                        const int sx = xp - x0t + kHalo;
                        const int f = nky[sx][lo - y0t + kHalo];
                        if (f < hi - y0t + kHalo) { xph = sh[sx][f]; xpd = xpf = true; }
                    }
                } else xpd = true;
            }
            if (!xnd) {
                if (xn >= 0) {
                    const int lo = max(y0 - i + 1, 0), hi = min(y0 + i + 1, X);  // dy in [-i+1, i+1)
                    if (lo < hi) {
                        const int sx = xn - x0t + kHalo;
                        const int f = nky[sx][lo - y0t + kHalo];
                        if (f < hi - y0t + kHalo) { xnh = sh[sx][f]; xnd = xnf = true; }
                    }
                } else xnd = true;
            }
            if (!ypd) {
                if (yp < X) {
                    const int lo = max(x0 - i + 1, 0), hi = min(x0 + i + 1, X);  // dx in [-i+1, i+1)
                    if (lo < hi) {
                        const int sy = yp - y0t + kHalo;
                        const int f = nkx[sy][lo - x0t + kHalo];
                        if (f < hi - x0t + kHalo) { yph = sh[f][sy]; ypd = ypf = true; }
                    }
                } else ypd = true;
            }
            if (!ynd) {
                if (yn >= 0) {
                    const int lo = max(x0 - i, 0), hi = min(x0 + i, X);  // dx in [-i, i)
                    if (lo < hi) {
                        const int sy = yn - y0t + kHalo;
                        const int f = nkx[sy][lo - x0t + kHalo];
                        if (f < hi - x0t + kHalo) { ynh = sh[f][sy]; ynd = ynf = true; }
                    }
                } else ynd = true;
            }
        }
        // a height found is known (> -1000), so each "> -1000" test is its
        // found flag; the extremes are taken on ordered keys (a -0 / +0 tie
        // can pick the other zero, which leaves mx - mn > 0 unchanged)
        double mn = 1000.0, mx = mp.inferred[cell];
        long long kmn = double_order(mn), kmx = double_order(mx);
        auto take = [&](double v) {
            const long long k = double_order(v);
            if (k < kmn) { kmn = k; mn = v; }
            if (k > kmx) { kmx = k; mx = v; }
        };
        if (xpf) take(xph);
        if (xnf) take(xnh);
        if (ypf) take(yph);
        if (xnf) take(ynh);  // x_nh's test guards y_nh (scripts/gvom.py:704-706); -1000 when not found
        const double dh = __dsub_rn(mx, mn);
        const long long db = __double_as_longlong(dh);
        if (db > 0 && db <= 0x7ff0000000000000LL) guess = dh;  // dh > 0
    }
    // cell warps that finish their search take what the extra warp has not
    __syncwarp();
    drain();
    __syncthreads();
    if (!valid) return;
    if (need_exact) {
        rough = qres[tid][0];
        slx = qres[tid][1];
        sly = qres[tid][2];
        slxf = (float)slx;
        slyf = (float)sly;
    }

    // __make_positive_obstacle_map slope gate (scripts/gvom.py:524-526): in
    // float32 unless |slope| is near the threshold
    bool steep;
    {
        const float sn = sqrtf(slxf * slxf + slyf * slyf);
        if (fabsf(sn - mp.slope_thr_f) > 1e-5f * mp.slope_thr_f + 1e-6f) steep = sn >= mp.slope_thr_f;
        else steep = sqrt(__dadd_rn(__dmul_rn(slx, slx), __dmul_rn(sly, sly))) >= mp.slope_thr;
    }
    mp.pos[cell] = steep ? 100 : mp.pos_density[cell];
    mp.neg[cell] = guess > mp.neg_thr ? 100 : 0;  // scripts/gvom.py:505-512
    mp.vis[cell] = known ? 1 : 0;                 // scripts/gvom.py:444-452
    mp.rough[cell] = rough;
    mp.slope_x[cell] = slx;
    mp.slope_y[cell] = sly;
    mp.guess[cell] = guess;
}

// ---------------------------------------------------------------------------
// k_ros_grids: the OccupancyGrid payloads of the reference's ROS node
// (scripts/gvom_ros.py:141-164) from the last combine's maps, one thread per
// cell, written in the node's column-major order (x fastest).  Each value is
// cast to int8 as numpy does on the node's x86 host: truncation toward zero
// through a 32-bit integer, then the low 8 bits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ signed char int8_wrap(double v) {
    // numpy's float64 -> int8 cast on x86 truncates through a 32-bit integer:
    // a value whose truncation lies outside int32, or NaN, becomes the integer
    // indefinite 0x80000000, whose low byte is 0
    if (!(v > -2147483649.0 && v < 2147483648.0)) return 0;
    const int t = (int)v;  // truncation toward zero
    return (signed char)(unsigned char)(t & 0xff);
}

__global__ void __launch_bounds__(256) k_ros_grids(const __grid_constant__ RosGridParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // payload index x + y X
    const int X = p.X;
    if (i >= X * X) return;
    const int x = i % X, y = i / X, c = x * X + y;  // maps are [x, y], y fastest
    const double obs = (double)p.pos[c];
    const int neg = p.neg[c];
    if (p.hard) {  // max(100 (obs > density threshold), neg)   (:142)
        const int h = obs > p.density_thr ? 100 : 0;
        p.hard[i] = int8_wrap((double)(h > neg ? h : neg));
    }
    if (p.soft) p.soft[i] = (obs <= p.density_thr && obs > 0.0) ? 100 : 0;  // (:147)
    if (p.certainty) p.certainty[i] = int8_wrap((double)(p.vis[c] * 100));      // (:152)
    if (p.negative) p.negative[i] = int8_wrap((double)neg);                     // (:158)
    if (p.roughness) {  // ((clip(r, min, max) + min) / (max - min)) * 100     (:162-164)
        const double r = p.rough[c];
        double v = (r < p.max_r || isnan(r)) ? r : p.max_r;  // np.minimum / np.maximum keep NaN
        v = (v > p.min_r || isnan(v)) ? v : p.min_r;
        v = __dmul_rn(__ddiv_rn(__dadd_rn(v, p.min_r), __dsub_rn(p.max_r, p.min_r)), 100.0);
        p.roughness[i] = int8_wrap(v);
    }
}

cudaError_t launch_ros_grids(const RosGridParams &p, cudaStream_t st) {
    const int n = p.X * p.X;
    k_ros_grids<<<(n + 255) / 256, 256, 0, st>>>(p);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// debug exporters
// ---------------------------------------------------------------------------
constexpr int kDbgChunk = 1024;  // voxels per block (256 threads x 4)

__global__ void __launch_bounds__(256) k_debug_count(const int *__restrict__ idx, long long V, int *__restrict__ counts) {
    const long long base = (long long)blockIdx.x * kDbgChunk + threadIdx.x * 4;
    int n = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (base + k < V && idx[base + k] >= 0) n++;
    __shared__ int ws[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < 8; w++) t += ws[w];
        counts[blockIdx.x] = t;
    }
}



// rows in ascending voxel-id order: [x, y, z, hit/total, hit, l0-l1, l1-l2, l2]
__global__ void __launch_bounds__(256) k_debug_voxels(DebugVoxParams p) {
    const long long base = (long long)blockIdx.x * kDbgChunk + threadIdx.x * 4;
    int flags[4];
    int n = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        flags[k] = (base + k < p.V) ? p.idx[base + k] : -1;
        if (flags[k] >= 0) n++;
    }
    // block exclusive scan of n
    __shared__ int ws[8];
    int incl = n;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    int woff = 0;
    for (int k = 0; k < w; k++) woff += ws[k];
    long long row = (long long)p.block_off[blockIdx.x] + woff + incl - n;
    const long long plane = (long long)p.X * p.X;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (flags[k] < 0) continue;
        if (row < p.cap) {
            const long long vid = base + k;
            const int x = (int)(vid % p.X), y = (int)((vid / p.X) % p.X), z = (int)(vid / plane);
            const VoxelRec r = p.rec[flags[k]];
            float *o = p.out + row * 8;
            o[0] = __double2float_rn(__dmul_rn(__dadd_rn((double)x, p.co[0]), p.xy_res));
            o[1] = __double2float_rn(__dmul_rn(__dadd_rn((double)y, p.co[1]), p.xy_res));
            o[2] = __double2float_rn(__dmul_rn(__dadd_rn((double)z, p.co[2]), p.z_res));
            o[3] = __double2float_rn(__ddiv_rn((double)r.hit, (double)r.total));
            o[4] = (float)r.hit;
            o[5] = __fsub_rn(r.aux[0], r.aux[1]);
            o[6] = __fsub_rn(r.aux[1], r.aux[2]);
            o[7] = r.aux[2];
        }
        row++;
    }
}



// rows indexed x + y*X (scripts/gvom.py:455-479)
__global__ void k_debug_maps(DebugMapParams p) {
    const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)p.X * p.X;
    if (cell >= n) return;
    const int x = (int)(cell / p.X), y = (int)(cell % p.X);
    const long long row = (long long)x + (long long)y * p.X;
    const float fx = __double2float_rn(__dmul_rn(__dadd_rn((double)x, p.co[0]), p.xy_res));
    const float fy = __double2float_rn(__dmul_rn(__dadd_rn((double)y, p.co[1]), p.xy_res));
    if (p.out_h) {
        float *o = p.out_h + row * 7;
        const double sx = p.slope_x[cell], sy = p.slope_y[cell];
        o[0] = fx;
        o[1] = fy;
        o[2] = __double2float_rn(__dsub_rn(p.height[cell], p.z_res));
        o[3] = __double2float_rn(p.rough[cell]);
        o[4] = __double2float_rn(sx);
        o[5] = __double2float_rn(sy);
        o[6] = __double2float_rn(sqrt(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy))));
    }
    if (p.out_i) {
        float *o = p.out_i + row * 3;
        o[0] = fx;
        o[1] = fy;
        o[2] = __double2float_rn(__dsub_rn(p.guess[cell], p.z_res));
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <int TX, int TY>
static cudaError_t launch_maps2d(const Maps2DParams &m2, cudaStream_t st) {
    const int X = m2.X;
    dim3 g2((X + TY - 1) / TY, (X + TX - 1) / TX);
    return rec_kernel(k_maps2d<TX, TY>, g2, dim3(TY, TX + 32 / TY), 0, st, m2);
}
template <int NSRC>
static cudaError_t launch_merge_idx(const MergeParams &mp, cudaStream_t st) {
    const int X = mp.g.X, Z = mp.g.Z, zc = mp.planes;
    dim3 gm((X + 255) / 256, X, (Z + zc - 1) / zc);
    if (zc == 4) return rec_kernel(k_merge<NSRC, 4>, gm, dim3(32, 8), 0, st, mp);
    if (zc == 16) return rec_kernel(k_merge<NSRC, 16>, gm, dim3(32, 8), 0, st, mp);
    return rec_kernel(k_merge<NSRC, 8>, gm, dim3(32, 8), 0, st, mp);
}

template <int NSRC>
static cudaError_t launch_merge_stats(const MergeParams &mp, cudaStream_t st) {
    return rec_kernel(k_merge_stats<NSRC>, dim3(mp.num_sms * mp.stats_bpsm), dim3(256), 0, st, mp);
}

template <int NSRC>
static cudaError_t launch_merge_counts(const MergeParams &mp, cudaStream_t st) {
    return rec_kernel(k_merge_counts<NSRC>, dim3(mp.num_sms * 8), dim3(256), 0, st, mp);
}

// source-count class of a merge (2, 3, 5, 9 or 17 sources)
template <template <int> class F>
static cudaError_t by_nsrc(const MergeParams &mp, cudaStream_t st) {
    if (mp.nsrc <= 2) return F<2>::run(mp, st);
    if (mp.nsrc <= 3) return F<3>::run(mp, st);
    if (mp.nsrc <= 5) return F<5>::run(mp, st);
    if (mp.nsrc <= 9) return F<9>::run(mp, st);
    return F<kMaxSources>::run(mp, st);
}
template <int N>
struct MergeIdx {
    static cudaError_t run(const MergeParams &mp, cudaStream_t st) { return launch_merge_idx<N>(mp, st); }
};
template <int N>
struct MergeStats {
    static cudaError_t run(const MergeParams &mp, cudaStream_t st) { return launch_merge_stats<N>(mp, st); }
};
template <int N>
struct MergeCounts {
    static cudaError_t run(const MergeParams &mp, cudaStream_t st) { return launch_merge_counts<N>(mp, st); }
};

cudaError_t launch_merge_index(const MergeParams &mp, cudaStream_t st) {
    const cudaError_t e = by_nsrc<MergeIdx>(mp, st);
    return e != cudaSuccess ? e : cudaGetLastError();
}

// count merge, statistics merge, columns and 2-D maps (events ev[1..5] when timing)
cudaError_t launch_combine_rest(const MergeParams &mp, const ColumnParams &cp, const Maps2DParams &m2, cudaStream_t st,
                                cudaEvent_t *ev, int part) {
    const int X = mp.g.X;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    if (part) ev = nullptr;
    if (ev) cudaEventRecord(ev[1], st);
    if (part == 0 || part == 1) chk(by_nsrc<MergeCounts>(mp, st));
    if (ev) cudaEventRecord(ev[2], st);
    if (part == 0 || part == 4) chk(by_nsrc<MergeStats>(mp, st));
    if (ev) cudaEventRecord(ev[3], st);
    if (part == 0 || part == 2) {
        dim3 gc((X + 31) / 32, (X + 7) / 8);
        chk(rec_kernel(k_columns, gc, dim3(32, 8), 0, st, cp));
    }
    if (ev) cudaEventRecord(ev[4], st);
    if (part == 0 || part == 3) {
        if (m2.tile_cells == 64) chk(launch_maps2d<4, 16>(m2, st));
        else if (m2.tile_cells == 128) chk(launch_maps2d<8, 16>(m2, st));
        else if (m2.tile_cells == 224) chk(launch_maps2d<14, 16>(m2, st));
        else chk(launch_maps2d<8, 32>(m2, st));
    }
    if (ev) cudaEventRecord(ev[5], st);
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_combine(const MergeParams &mp, const ColumnParams &cp, const Maps2DParams &m2, cudaStream_t st,
                           cudaEvent_t *ev) {  // every kernel in sequence on `st`
    if (ev) cudaEventRecord(ev[0], st);
    const cudaError_t e = by_nsrc<MergeIdx>(mp, st);
    if (e != cudaSuccess) return e;
    return launch_combine_rest(mp, cp, m2, st, ev);
}

cudaError_t launch_debug_count(const int *idx, long long V, int *counts, int nblocks, cudaStream_t st) {
    k_debug_count<<<nblocks, 256, 0, st>>>(idx, V, counts);
    return cudaGetLastError();
}

cudaError_t launch_debug_voxels(const DebugVoxParams &p, int nblocks, cudaStream_t st) {
    k_debug_voxels<<<nblocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_debug_maps(const DebugMapParams &p, cudaStream_t st) {
    const long long n = (long long)p.X * p.X;
    k_debug_maps<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p);
    return cudaGetLastError();
}

int debug_chunk() { return kDbgChunk; }

// Every combine kernel a call can launch, loaded now: with CUDA's lazy module
// loading a kernel is otherwise loaded at its first launch, which stalls the
// device for milliseconds in the middle of a request loop (a ring that fills
// up reaches a new source-count class, a batch a new size).
template <int N>
static void add_merge_kernels(std::vector<const void *> &k) {
    k.push_back(reinterpret_cast<const void *>(k_merge<N, 4>));
    k.push_back(reinterpret_cast<const void *>(k_merge<N, 8>));
    k.push_back(reinterpret_cast<const void *>(k_merge<N, 16>));
    k.push_back(reinterpret_cast<const void *>(k_merge_counts<N>));
    k.push_back(reinterpret_cast<const void *>(k_merge_stats<N>));
}

cudaError_t preload_combine_kernels() {
    std::vector<const void *> k;
    add_merge_kernels<2>(k);
    add_merge_kernels<3>(k);
    add_merge_kernels<5>(k);
    add_merge_kernels<9>(k);
    add_merge_kernels<kMaxSources>(k);
    for (const void *f : {reinterpret_cast<const void *>(k_columns), reinterpret_cast<const void *>(k_maps2d<8, 32>),
                          reinterpret_cast<const void *>(k_maps2d<8, 16>), reinterpret_cast<const void *>(k_maps2d<4, 16>),
                          reinterpret_cast<const void *>(k_maps2d<14, 16>),
                          reinterpret_cast<const void *>(k_ros_grids), reinterpret_cast<const void *>(k_debug_count),
                          reinterpret_cast<const void *>(k_debug_voxels), reinterpret_cast<const void *>(k_debug_maps),
                          reinterpret_cast<const void *>(k_gather_records)})
        k.push_back(f);
    for (const void *f : k) {
        cudaFuncAttributes a;
        const cudaError_t e = cudaFuncGetAttributes(&a, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_gather_records(const VoxelRec *rec, const int *vids, int n, VoxelRec *out, cudaStream_t st) {
    if (n > 0) k_gather_records<<<(n + 255) / 256, 256, 0, st>>>(rec, vids, n, out);
    return cudaGetLastError();
}

}  // namespace gvom
