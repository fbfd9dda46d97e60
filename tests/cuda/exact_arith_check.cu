// Randomised device check of the scan kernel's voxel arithmetic against the
// plain float64 sequence of the reference (scripts/gvom.py:1153-1231): the
// integer path (gvom_exact.cuh) on every case it accepts, the float32 ray step
// count and the fast ray index.  Prints counts and exits non-zero on any
// disagreement.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include "../../gvom_gb300/csrc/gvom_internal.cuh"
#include "../../gvom_gb300/csrc/gvom_exact.cuh"

using namespace gvom;

struct Counts {
    unsigned long long trials, accepted, bad_end, bad_b, bad_frac, rsc_trials, rsc_bad, ri_trials, ri_bad;
};

__device__ unsigned long long mix(unsigned long long x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

__global__ void check(double res, ExactRes R, int mode, unsigned long long seed, int per_thread, Counts *out) {
    const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    unsigned long long acc = 0, be = 0, bb = 0, bf = 0, rs_bad = 0, ri_bad = 0;
    for (int it = 0; it < per_thread; it++) {
        const unsigned long long h = mix(seed ^ (tid * 1315423911ULL + it));
        const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);       // [0, 1)
        const double u2 = (double)(mix(h) >> 11) * (1.0 / 9007199254740992.0);
        // point coordinate
        float p;
        if (mode == 0) p = (float)(u * 200.0 - 100.0);                                     // near origin
        else if (mode == 1) p = (float)(1.0e4 + u * 100.0 - 50.0);                          // far world
        else if (mode == 2) p = (float)(floor(u * 2000.0 - 1000.0) * res + (u2 - 0.5) * 1e-5);  // near voxel faces
        else p = __int_as_float((int)(mix(h + 7) & 0x7fffffff) % 0x45000000) * (u2 < 0.5 ? -1.f : 1.f);  // |p| < 2048
        const double ego = (mode == 1 ? 1.0e4 : 0.0) + (u2 - 0.5) * 20.0;
        const double od = floor(ego / res - 128.0);
        // reference float64 sequence
        const double q = __ddiv_rn((double)p, res);
        const double t = __dsub_rn(q, od);
        const double f = floor(t);
        const float end_ref = __double2float_rn(q);
        const float frac_ref = __double2float_rn(__dsub_rn(t, f));
        float end, frac;
        long long b;
        bool in_range;
        if (gx_coord(p, R, (long long)od, end, b, frac, in_range)) {
            acc++;
            if (__float_as_int(end) != __float_as_int(end_ref)) be++;
            if (in_range && (double)b != f) bb++;
            if (!in_range && fabs(t) < 2147483648.0) bb++;
            if (in_range && __float_as_int(frac) != __float_as_int(frac_ref)) bf++;
        }
        // ray step count: float32 path vs the float64 loop
        {
            const float rlen = (float)(u * (mode == 3 ? 700.0 : 300.0));
            const float sk = (float)(0.57735 + u2 * 0.43) * (h & 1 ? -1.f : 1.f);
            const int K = ray_step_count(rlen, sk, 1 << 20);
            int Kref = 0;
            if (rlen > 1.0f) {
                const double R = __dsub_rn((double)rlen, 1.0), inc = fabs(__ddiv_rn(1.0, (double)sk));
                double L = 0.0;
                while (L < R && Kref < (1 << 20)) { Kref++; L = __dadd_rn(L, inc); }
            }
            if (K != Kref) rs_bad++;
            // rays whose length sits at a step boundary (the float32 margin fails): the
            // integer count of the float64 loop, on the device, against that loop
            const double incb = fabs(__ddiv_rn(1.0, (double)sk));
            const float rb = (float)(1.0 + (floor(u * 500.0) + 1.0 + (u2 - 0.5) * 2e-5) * incb);
            const double Rb = __dsub_rn((double)rb, 1.0);
            int Kb = 0;
            double Lb = 0.0;
            while (Lb < Rb && Kb < 520) { Kb++; Lb = __dadd_rn(Lb, incb); }
            if (gx_step_count(Rb, incb, 520) != Kb || ray_step_count(rb, sk, 520) != Kb) rs_bad++;
        }
        // ray index fast floor
        {
            const float pt = (float)(od + (u2 * 300.0 - 20.0)) + (float)(u - 0.5);
            const int fast = fabs(od) < 16777216.0 ? 1 : 0;
            const int vi = ray_index(pt, (int)od, od, fast);
            const double tr = floor(__dsub_rn((double)pt, od));
            if (fabs(tr) < 1e9 && vi != (int)tr) ri_bad++;
            // small negative positions (ray near the world origin plane) with origins up to 2^24
            const float pn = -ldexpf((float)u + 1e-3f, -(int)(u2 * 40.0));
            const double on = floor((u2 - 0.5) * (mode == 1 ? 3.3e7 : 600.0));
            const int fn = fabs(on) < 16777216.0 ? 1 : 0;
            const int vn = ray_index(pn, (int)on, on, fn);
            const double tn = floor(__dsub_rn((double)pn, on));
            if (fabs(tn) < 1e9 && vn != (int)tn) ri_bad++;
        }
    }
    atomicAdd(&out->trials, (unsigned long long)per_thread);
    atomicAdd(&out->accepted, acc);
    atomicAdd(&out->bad_end, be);
    atomicAdd(&out->bad_b, bb);
    atomicAdd(&out->bad_frac, bf);
    atomicAdd(&out->rsc_trials, (unsigned long long)per_thread);
    atomicAdd(&out->rsc_bad, rs_bad);
    atomicAdd(&out->ri_trials, (unsigned long long)per_thread);
    atomicAdd(&out->ri_bad, ri_bad);
}

int main() {
    const double resolutions[] = {0.1, 0.15, 0.2, 0.4, 1.0, 1.0 / 3.0, 0.0625};
    Counts *d;
    if (cudaMalloc(&d, sizeof(Counts)) != cudaSuccess) return 2;
    int fail = 0;
    for (double res : resolutions) {
        int e;
        const double fr = std::frexp(res, &e);
        ExactRes R;
        R.mr = (unsigned long long)std::ldexp(fr, 53);
        R.er = e - 53;
        unsigned __int128 w = ((unsigned __int128)1 << 116) / R.mr;
        if (w >> 64) w = ~0ull;
        R.W = (unsigned long long)w;
        R.pad = 0;
        for (int mode = 0; mode < 4; mode++) {
            cudaMemset(d, 0, sizeof(Counts));
            check<<<152 * 4, 256>>>(res, R, mode, 0x9e3779b97f4a7c15ULL * (mode + 1) ^ (unsigned long long)(res * 1e6), 16, d);
            Counts c;
            if (cudaMemcpy(&c, d, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) {
                printf("cuda error %s\n", cudaGetErrorString(cudaGetLastError()));
                return 2;
            }
            const bool ok = !c.bad_end && !c.bad_b && !c.bad_frac && !c.rsc_bad && !c.ri_bad;
            printf("res %.6f mode %d: %llu trials, integer path accepted %.4f%%, bad end %llu b %llu frac %llu, "
                   "step-count bad %llu, ray-index bad %llu %s\n", res, mode, c.trials, 100.0 * c.accepted / c.trials,
                   c.bad_end, c.bad_b, c.bad_frac, c.rsc_bad, c.ri_bad, ok ? "OK" : "MISMATCH");
            if (!ok) fail = 1;
        }
    }
    cudaFree(d);
    return fail;
}
