// Map-combine kernels: Gvom.combine_maps (scripts/gvom.py:222-393).
//
//   k_merge    one thread per (x, y) column, walking z: merges every ring slot
//              (slot order) and the previous combined map with their ego
//              shifts and the clearing rule (scripts/gvom.py:1009-1063),
//              allocates compact indices, Chan-merges the statistics
//              (scripts/gvom.py:888-980), solves the 3x3 eigenvalues
//              (scripts/gvom.py:1423-1487), and in the same walk reduces the
//              column to its height, inferred height and positive-obstacle
//              band density (scripts/gvom.py:515-590)
//   k_maps2d   one thread per cell on a shared-memory tile with a 15-cell
//              halo: slope / roughness, guessed height delta, positive,
//              negative and visibility maps (scripts/gvom.py:444-805)
//   debug      make_debug_voxel_map / height / inferred exporters
//              (scripts/gvom.py:395-503)
#include "gvom_internal.cuh"

namespace gvom {

constexpr int kOcc = 0x7fffffff;
constexpr int kOutside = INT32_MIN;

// ---------------------------------------------------------------------------
// eigenvalues of a symmetric 3x3 matrix, trigonometric closed form
// (scripts/gvom.py:1423-1487)
// ---------------------------------------------------------------------------
// float64 restatement in the reference's operand types (inputs float32).
__device__ void eigen_f64(float xx, float xy, float xz, float yy, float yz, float zz, float e[3]) {
    const float p1 = __fadd_rn(__fadd_rn(__fmul_rn(xy, xy), __fmul_rn(xz, xz)), __fmul_rn(yz, yz));
    const float tr = __fadd_rn(__fadd_rn(xx, yy), zz);
    const double q = __ddiv_rn((double)tr, 3.0);
    if (p1 == 0.0f) {
        const float m12 = yy > zz ? yy : zz;
        e[0] = xx > m12 ? xx : m12;
        const float n12 = yy < zz ? yy : zz;
        e[2] = xx < n12 ? xx : n12;
        e[1] = __double2float_rn(__dsub_rn(__dsub_rn(__dmul_rn(3.0, q), (double)e[0]), (double)e[2]));
        return;
    }
    const double dxx = __dsub_rn((double)xx, q), dyy = __dsub_rn((double)yy, q), dzz = __dsub_rn((double)zz, q);
    double p2 = __dadd_rn(__dmul_rn(dxx, dxx), __dmul_rn(dyy, dyy));
    p2 = __dadd_rn(p2, __dmul_rn(dzz, dzz));
    p2 = __dadd_rn(p2, __dmul_rn(2.0, (double)p1));
    const double p = sqrt(__ddiv_rn(p2, 6.0));
    const double B0 = __ddiv_rn(dxx, p), B1 = __ddiv_rn((double)xy, p), B2 = __ddiv_rn((double)xz, p);
    const double B3 = __ddiv_rn(dyy, p), B4 = __ddiv_rn((double)yz, p), B5 = __ddiv_rn(dzz, p);
    double r = __dsub_rn(__dmul_rn(B0, __dsub_rn(__dmul_rn(B3, B5), __dmul_rn(B4, B4))),
                         __dmul_rn(B1, __dsub_rn(__dmul_rn(B1, B5), __dmul_rn(B4, B2))));
    r = __dadd_rn(r, __dmul_rn(B2, __dsub_rn(__dmul_rn(B1, B4), __dmul_rn(B3, B2))));
    r = __ddiv_rn(r, 2.0);
    double phi;
    if (r <= -1.0) phi = __ddiv_rn(M_PI, 3.0);
    else if (r >= 1.0) phi = 0.0;
    else phi = __ddiv_rn(acos(r), 3.0);
    const double tp = __dmul_rn(2.0, p);
    e[0] = __double2float_rn(__dadd_rn(q, __dmul_rn(tp, cos(phi))));
    e[2] = __double2float_rn(__dadd_rn(q, __dmul_rn(tp, cos(__dadd_rn(phi, __ddiv_rn(2.0 * M_PI, 3.0))))));
    e[1] = __double2float_rn(__dsub_rn(__dsub_rn(__dmul_rn(3.0, q), (double)e[0]), (double)e[2]));
}

// One Jacobi rotation zeroing a_pq of a symmetric 3x3 matrix (eigenvalues
// only); r is the remaining index.
__device__ __forceinline__ void jacobi_rot(float &app, float &aqq, float &apq, float &arp, float &arq) {
    if (apq == 0.0f) return;
    const float theta = (aqq - app) / (2.0f * apq);
    float t;
    if (fabsf(theta) > 1.0e18f) t = 0.5f / theta;
    else t = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
    const float c = 1.0f / sqrtf(t * t + 1.0f);
    const float s = t * c;
    const float tau = s / (1.0f + c);
    app -= t * apq;
    aqq += t * apq;
    apq = 0.0f;
    const float rp = arp, rq = arq;
    arp = rp - s * (rq + tau * rp);
    arq = rq + s * (rp - tau * rq);
}

// Eigenvalues (descending) of the symmetric 3x3 covariance.  Cyclic Jacobi in
// float32: backward stable, so each eigenvalue (and the gaps between nearly
// equal ones, which the closed form loses) is within ~1e-7 |A|.  Voxels whose
// smallest / largest eigenvalue ratio is below 1e-6 are re-solved in float64
// with the reference's closed form (eigen_f64).
__device__ void eigen_solve(float xx, float xy, float xz, float yy, float yz, float zz, float e[3]) {
    float a00 = xx, a01 = xy, a02 = xz, a11 = yy, a12 = yz, a22 = zz;
    const float scale = fabsf(a00) + fabsf(a11) + fabsf(a22) + fabsf(a01) + fabsf(a02) + fabsf(a12);
#pragma unroll 1
    for (int sweep = 0; sweep < 8; sweep++) {
        if (fabsf(a01) + fabsf(a02) + fabsf(a12) <= 1.0e-9f * scale) break;
        jacobi_rot(a00, a11, a01, a02, a12);
        jacobi_rot(a00, a22, a02, a01, a12);
        jacobi_rot(a11, a22, a12, a01, a02);
    }
    float l0 = a00, l1 = a11, l2 = a22, t;
    if (l0 < l1) { t = l0; l0 = l1; l1 = t; }
    if (l1 < l2) { t = l1; l1 = l2; l2 = t; }
    if (l0 < l1) { t = l0; l0 = l1; l1 = t; }
    if (!(fabsf(l2) >= 1e-6f * fabsf(l0))) {
        eigen_f64(xx, xy, xz, yy, yz, zz, e);
        return;
    }
    e[0] = l0;
    e[1] = l1;
    e[2] = l2;
}

// ---------------------------------------------------------------------------
// k_merge
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_rec(const VoxelRec *r, float4 &a, float4 &b, float4 &c, float4 &d) {
    const float4 *p = reinterpret_cast<const float4 *>(r);
    a = __ldg(p);
    b = __ldg(p + 1);
    c = __ldg(p + 2);
    d = __ldg(p + 3);
}

__global__ void __launch_bounds__(256) k_merge(MergeParams mp) {
    const Geom g = mp.g;
    const int X = g.X, Z = g.Z;
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int y = blockIdx.y * 8 + threadIdx.y;
    const bool col = x < X && y < X;
    const long long plane = (long long)X * X;
    const unsigned lane = (threadIdx.y * 32 + threadIdx.x) & 31u;  // blockDim.x == 32: lane == threadIdx.x
    (void)lane;

    double h = -1000.0;
    if (col) {
        // height disc around the ego (scripts/gvom.py:566-570)
        const double xp = __dsub_rn(__dmul_rn(__dadd_rn(mp.co[0], (double)x), mp.xy_res), mp.ego[0]);
        const double yp = __dsub_rn(__dmul_rn(__dadd_rn(mp.co[1], (double)y), mp.xy_res), mp.ego[1]);
        if (__dadd_rn(__dmul_rn(xp, xp), __dmul_rn(yp, yp)) <= mp.robot_r2) h = mp.disc_h;
    }
    bool hset = false, iset = false, band = false;
    double ih = -1000.0;
    long long zmin = 0, zmax = -1;
    double dens = 0.0, nn = 0.0;

    for (int z = 0; z < Z; z++) {
        int v[kMaxSources];
#pragma unroll
        for (int s = 0; s < kMaxSources; s++) {
            v[s] = kOutside;
            if (s < mp.nsrc && col) {
                const int xs = x + mp.src[s].dx, ys = y + mp.src[s].dy, zs = z + mp.src[s].dz;
                if (xs >= 0 && xs < X && ys >= 0 && ys < X && zs >= 0 && zs < Z)
                    v[s] = __ldg(&mp.src[s].idx[(long long)xs + (long long)ys * X + (long long)zs * plane]);
            }
        }
        int comb = -1;
#pragma unroll
        for (int s = 0; s < kMaxSources; s++) {
            if (s < mp.nsrc && v[s] != kOutside) {
                const int o = v[s];
                const bool alloc = mp.src[s].is_last ? (o >= 0 && comb <= -1 && comb >= -11) : (o >= 0 && comb <= -1);
                if (alloc) comb = kOcc;
                else if (o < -1 && comb <= -1) comb += o + 1;
            }
        }
        const bool occ = comb == kOcc;
        const unsigned om = __ballot_sync(0xffffffffu, occ);
        int base = 0;
        if (om) {
            const int leader = __ffs(om) - 1;
            if ((int)threadIdx.x == leader) base = atomicAdd(mp.out_count, __popc(om));
            base = __shfl_sync(0xffffffffu, base, leader);
        }
        int hit = 0, total = 0;
        float minh = 1.0f;
        if (occ) {
            const int c = base + __popc(om & ((1u << threadIdx.x) - 1u));
            float n = 0.f, m0 = 0.f, m1 = 0.f, m2 = 0.f;
            float C[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int s = 0; s < kMaxSources; s++) {
                if (s < mp.nsrc && v[s] >= 0 && v[s] != kOutside) {
                    float4 a, b, cc, d;
                    load_rec(&mp.src[s].rec[v[s]], a, b, cc, d);
                    // a = mean0 mean1 mean2 xx | b = xy xz yy yz | cc = zz count hit total | d = minh aux
                    const float n2 = cc.y;
                    const float o_m[3] = {a.x, a.y, a.z};
                    const float o_c[6] = {a.w, b.x, b.y, b.z, b.w, cc.x};
                    const float den = __fadd_rn(n, n2);
                    const float nm0 = __fdiv_rn(__fadd_rn(__fmul_rn(m0, n), __fmul_rn(o_m[0], n2)), den);
                    const float nm1 = __fdiv_rn(__fadd_rn(__fmul_rn(m1, n), __fmul_rn(o_m[1], n2)), den);
                    const float nm2 = __fdiv_rn(__fadd_rn(__fmul_rn(m2, n), __fmul_rn(o_m[2], n2)), den);
                    const float cm[3] = {m0, m1, m2};
                    const float mn[3] = {nm0, nm1, nm2};
                    const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
                    for (int t = 0; t < 6; t++) {
                        const float t1 = __fmul_rn(n, C[t]);
                        const float t2 = __fmul_rn(n2, o_c[t]);
                        const float t3 = __fmul_rn(__fmul_rn(n, __fsub_rn(cm[pa[t]], mn[pa[t]])), __fsub_rn(cm[pb[t]], mn[pb[t]]));
                        const float t4 = __fmul_rn(__fmul_rn(n2, __fsub_rn(o_m[pa[t]], mn[pa[t]])), __fsub_rn(o_m[pb[t]], mn[pb[t]]));
                        C[t] = __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(t1, t2), t3), t4), den);
                    }
                    m0 = nm0;
                    m1 = nm1;
                    m2 = nm2;
                    n = den;
                    hit += __float_as_int(cc.z);
                    total += __float_as_int(cc.w);
                    minh = fminf(minh, d.x);
                }
            }
            float e[3];
            eigen_solve(C[0], C[1], C[2], C[3], C[4], C[5], e);
            float4 *o = reinterpret_cast<float4 *>(&mp.out_rec[c]);
            o[0] = make_float4(m0, m1, m2, C[0]);
            o[1] = make_float4(C[1], C[2], C[3], C[4]);
            o[2] = make_float4(C[5], n, __int_as_float(hit), __int_as_float(total));
            o[3] = make_float4(minh, e[0], e[1], e[2]);
            comb = c;
        }
        if (col) {
            mp.out_idx[(long long)x + (long long)y * X + (long long)z * plane] = comb;
            if (comb >= 0 && !hset) {
                // lowest occupied voxel -> height (scripts/gvom.py:572-576)
                h = __dmul_rn(__dadd_rn(__dadd_rn((double)minh, (double)z), mp.co[2]), mp.z_res);
                hset = true;
                // positive-obstacle band above it (scripts/gvom.py:529-539)
                const double mino = __dadd_rn(h, mp.pos_thr), maxo = __dadd_rn(h, mp.robot_h);
                zmin = (long long)floor(__dsub_rn(__ddiv_rn(mino, mp.z_res), mp.co[2])) + 1;
                zmax = (long long)floor(__dsub_rn(__ddiv_rn(maxo, mp.z_res), mp.co[2]));
                band = zmin >= 0 && zmin < Z && zmax >= 0 && zmax < Z;
            }
            if (comb < -1 && !iset) {
                // lowest known-free voxel -> inferred height (scripts/gvom.py:585-590)
                ih = __dmul_rn(__dadd_rn((double)z, mp.co[2]), mp.z_res);
                iset = true;
            }
            if (band && z >= zmin && z <= zmax && comb >= 0 && hit > 10) {
                // scripts/gvom.py:541-549
                nn = __dadd_rn(nn, (double)total);
                dens = __dadd_rn(dens, (double)hit);
            }
        }
    }
    if (col) {
        int pd = 0;
        if (band) {
            if (nn > 0.0) dens = __ddiv_rn(dens, nn);
            pd = (int)__dmul_rn(dens, 100.0);
        }
        const long long m2d = (long long)x * X + y;
        mp.height[m2d] = h;
        mp.inferred[m2d] = ih;
        mp.pos_density[m2d] = pd;
    }
}

// ---------------------------------------------------------------------------
// k_maps2d: tile of 8 (x) by 32 (y) cells plus a 15-cell halo of heights.
// ---------------------------------------------------------------------------
constexpr int kTX = 8, kTY = 32, kHalo = 15;
constexpr int kSX = kTX + 2 * kHalo, kSY = kTY + 2 * kHalo;

__global__ void __launch_bounds__(256) k_maps2d(Maps2DParams mp) {
    __shared__ double sh[kSX][kSY];
    const int X = mp.X;
    const int x0t = blockIdx.y * kTX, y0t = blockIdx.x * kTY;
    const int tid = threadIdx.y * kTY + threadIdx.x;
    for (int k = tid; k < kSX * kSY; k += kTX * kTY) {
        const int sx = k / kSY, sy = k % kSY;
        const int gx = x0t + sx - kHalo, gy = y0t + sy - kHalo;
        sh[sx][sy] = (gx >= 0 && gx < X && gy >= 0 && gy < X) ? mp.height[(long long)gx * X + gy] : -1000.0;
    }
    __syncthreads();
    const int x0 = x0t + threadIdx.y, y0 = y0t + threadIdx.x;
    if (x0 >= X || y0 >= X) return;
#define H(gx, gy) sh[(gx) - x0t + kHalo][(gy) - y0t + kHalo]
    const long long cell = (long long)x0 * X + y0;
    const double hc = H(x0, y0);

    // __calculate_slope (scripts/gvom.py:717-805)
    double rough = -1.0, slx = 0.0, sly = 0.0;
    {
        const int xl = max(0, x0 - 1), xh = min(X, x0 + 2), yl = max(0, y0 - 1), yh = min(X, y0 + 2);
        int n_good = 0;
        for (int xx = xl; xx < xh; xx++)
            for (int yy = yl; yy < yh; yy++)
                if (H(xx, yy) > -1000.0) n_good++;
        if (n_good >= 3) {
            double px[9], py[9], pz[9];
            int i = 0;
            double mx = 0.0, my = 0.0, mz = 0.0;
            for (int xx = xl; xx < xh; xx++)
                for (int yy = yl; yy < yh; yy++)
                    if (H(xx, yy) > -1000.0) {
                        px[i] = __dmul_rn((double)xx, mp.xy_res);
                        py[i] = __dmul_rn((double)yy, mp.xy_res);
                        pz[i] = H(xx, yy);
                        mx = __dadd_rn(mx, px[i]);
                        my = __dadd_rn(my, py[i]);
                        mz = __dadd_rn(mz, pz[i]);
                        i++;
                    }
            mx = __ddiv_rn(mx, (double)i);
            my = __ddiv_rn(my, (double)i);
            mz = __ddiv_rn(mz, (double)i);
            double sxx = 0.0, sxy = 0.0, sxz = 0.0, syy = 0.0, syz = 0.0;
            for (int j = 0; j < n_good; j++) {
                const double dx = __dsub_rn(px[j], mx), dy = __dsub_rn(py[j], my), dz = __dsub_rn(pz[j], mz);
                sxx = __dadd_rn(sxx, __dmul_rn(dx, dx));
                sxy = __dadd_rn(sxy, __dmul_rn(dx, dy));
                sxz = __dadd_rn(sxz, __dmul_rn(dx, dz));
                syy = __dadd_rn(syy, __dmul_rn(dy, dy));
                syz = __dadd_rn(syz, __dmul_rn(dy, dz));
            }
            const double det = __dsub_rn(__dmul_rn(sxx, syy), __dmul_rn(sxy, sxy));
            if (det != 0.0) {
                double a0 = __ddiv_rn(__dsub_rn(__dmul_rn(syy, sxz), __dmul_rn(sxy, syz)), det);
                double a1 = __ddiv_rn(__dsub_rn(__dmul_rn(sxx, syz), __dmul_rn(sxy, sxz)), det);
                const double m = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(a0, a0), __dmul_rn(a1, a1)), 1.0));
                a0 = __ddiv_rn(a0, m);
                a1 = __ddiv_rn(a1, m);
                double err = 0.0;
                for (int j = 0; j < n_good; j++) {
                    const double e = __dsub_rn(__dsub_rn(pz[j], mz),
                                               __dadd_rn(__dmul_rn(a0, __dsub_rn(px[j], mx)),
                                                         __dmul_rn(a1, __dsub_rn(py[j], my))));
                    err = __dadd_rn(err, __dmul_rn(e, e));
                }
                err = __ddiv_rn(err, (double)n_good);
                if (err > 0.0) err = log(err);
                rough = err;
                const double im = __ddiv_rn(1.0, m);
                slx = atan2(a0, im);
                sly = atan2(a1, im);
            }
        }
    }

    // __guess_height (scripts/gvom.py:592-714), loop-condition and y_nh quirks included
    double guess = 0.0;
    if (!(hc > -1000.0) && !(mp.inferred[cell] == -1000.0)) {
        bool xpd = false, xnd = false, ypd = false, ynd = false;
        int xp = x0, xn = x0, yp = y0, yn = y0;
        double xph = -1000.0, xnh = -1000.0, yph = -1000.0, ynh = -1000.0;
        int i = 0;
        while (i < 15 && !(xnd && xnd && ypd && ynd)) {
            xp += 1; xn -= 1; yp += 1; yn -= 1;
            i += 1;
            if (!xpd) {
                if (xp < X) {
                    for (int dy = -i; dy < i; dy++) {
                        if (y0 + dy >= X || y0 + dy < 0) continue;
                        if (H(xp, y0 + dy) > -1000.0) { xph = H(xp, y0 + dy); xpd = true; break; }
                    }
                } else xpd = true;
            }
            if (!xnd) {
                if (xn >= 0) {
                    for (int dy = -i + 1; dy < i + 1; dy++) {
                        if (y0 + dy >= X || y0 + dy < 0) continue;
                        if (H(xn, y0 + dy) > -1000.0) { xnh = H(xn, y0 + dy); xnd = true; break; }
                    }
                } else xnd = true;
            }
            if (!ypd) {
                if (yp < X) {
                    for (int dx = -i + 1; dx < i + 1; dx++) {
                        if (x0 + dx >= X || x0 + dx < 0) continue;
                        if (H(x0 + dx, yp) > -1000.0) { yph = H(x0 + dx, yp); ypd = true; break; }
                    }
                } else ypd = true;
            }
            if (!ynd) {
                if (yn >= 0) {
                    for (int dx = -i; dx < i; dx++) {
                        if (x0 + dx >= X || x0 + dx < 0) continue;
                        if (H(x0 + dx, yn) > -1000.0) { ynh = H(x0 + dx, yn); ynd = true; break; }
                    }
                } else ynd = true;
            }
        }
        double mn = 1000.0, mx = mp.inferred[cell];
        if (xph > -1000.0) { mn = xph < mn ? xph : mn; mx = xph > mx ? xph : mx; }
        if (xnh > -1000.0) { mn = xnh < mn ? xnh : mn; mx = xnh > mx ? xnh : mx; }
        if (yph > -1000.0) { mn = yph < mn ? yph : mn; mx = yph > mx ? yph : mx; }
        if (xnh > -1000.0) { mn = ynh < mn ? ynh : mn; mx = ynh > mx ? ynh : mx; }
        const double dh = __dsub_rn(mx, mn);
        if (dh > 0.0) guess = dh;
    }
#undef H
    // __make_positive_obstacle_map slope gate (scripts/gvom.py:524-526)
    const double sn = sqrt(__dadd_rn(__dmul_rn(slx, slx), __dmul_rn(sly, sly)));
    mp.pos[cell] = sn >= mp.slope_thr ? 100 : mp.pos_density[cell];
    mp.neg[cell] = guess > mp.neg_thr ? 100 : 0;            // scripts/gvom.py:505-512
    mp.vis[cell] = hc > -1000.0 ? 1 : 0;                    // scripts/gvom.py:444-452
    mp.rough[cell] = rough;
    mp.slope_x[cell] = slx;
    mp.slope_y[cell] = sly;
    mp.guess[cell] = guess;
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
cudaError_t launch_combine(const MergeParams &mp, const Maps2DParams &m2, cudaStream_t st, cudaEvent_t *ev) {
    const int X = mp.g.X;
    if (ev) cudaEventRecord(ev[0], st);
    dim3 gm((X + 31) / 32, (X + 7) / 8);
    k_merge<<<gm, dim3(32, 8), 0, st>>>(mp);
    if (ev) cudaEventRecord(ev[1], st);
    dim3 g2((X + kTY - 1) / kTY, (X + kTX - 1) / kTX);
    k_maps2d<<<g2, dim3(kTY, kTX), 0, st>>>(m2);
    if (ev) cudaEventRecord(ev[2], st);
    return cudaGetLastError();
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

}  // namespace gvom
