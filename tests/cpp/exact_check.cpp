// Host check of gvom_gb300/csrc/gvom_exact.cuh against native IEEE float64:
// for random and adversarial (p, r, o) the integer path must give the
// reference's end = RN32(RN64(p/r)), b = floor(RN64(RN64(p/r) - o)) and
// frac = RN32(t - b) bit for bit.  Usage: exact_check [n_per_case]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "../../gvom_gb300/csrc/gvom_exact.cuh"

using namespace gvom;

static ExactRes make_res(double r) {
    int e;
    const double f = std::frexp(r, &e);  // r = f 2^e, f in [0.5, 1)
    ExactRes R;
    R.mr = (unsigned long long)std::ldexp(f, 53);
    R.er = e - 53;
    const unsigned __int128 num = (unsigned __int128)1 << 116;
    unsigned __int128 w = num / R.mr;
    if (w >> 64) w = ~(unsigned long long)0;
    R.W = (unsigned long long)w;
    R.pad = 0;
    return R;
}

static unsigned f2u(float f) { unsigned u; memcpy(&u, &f, 4); return u; }

int main(int argc, char **argv) {
    const long n = argc > 1 ? atol(argv[1]) : 200000;
    const double rs[] = {0.1, 0.15, 0.2, 0.4, 1.0, 1.0 / 3.0, 0.0625, 0.05, 0.3, 0.123456789, 2.5, 7.0};
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    long bad = 0, total = 0, declined = 0;
    for (double r : rs) {
        const ExactRes R = make_res(r);
        for (int mode = 0; mode < 6; mode++) {
            for (long i = 0; i < n; i++) {
                float p;
                const double u = U(g), u2 = U(g);
                switch (mode) {
                case 0: p = (float)(u * 200.0 - 100.0); break;                       // near origin
                case 1: p = (float)(1.0e4 + u * 200.0 - 100.0); break;               // far world
                case 2: p = (float)(std::floor(u * 4000.0 - 2000.0) * r + (u2 - 0.5) * 1e-6); break;  // voxel faces
                case 3: { unsigned b = (unsigned)(g() & 0x7fffffffu) % 0x46000000u; memcpy(&p, &b, 4); if (u2 < 0.5) p = -p; } break;
                case 4: p = (float)((u - 0.5) * 1e-3); break;                        // near zero
                default: p = (float)((std::floor(u * 1000) + 0.5) * r * (u2 < 0.5 ? -1 : 1)); break;  // mid-voxel
                }
                const double ego = (mode == 1 ? 1.0e4 : 0.0) + (u2 - 0.5) * 40.0;
                const long long o = (long long)std::floor(ego / r - 128.0);
                // reference float64 sequence
                const double q = (double)p / r;
                const double t = q - (double)o;
                const double fl = std::floor(t);
                const float end_ref = (float)q;
                const float frac_ref = (float)(t - fl);
                float end, frac;
                long long b;
                bool in_range;
                total++;
                if (!gx_coord(p, R, o, end, b, frac, in_range)) { declined++; continue; }
                bool ok = f2u(end) == f2u(end_ref);
                if (in_range) ok = ok && (double)b == fl && f2u(frac) == f2u(frac_ref);
                else ok = ok && std::fabs(t) >= 2147483648.0;
                if (!ok) {
                    if (bad < 20)
                        printf("MISMATCH r=%.17g p=%.9g (0x%08x) o=%lld: end %.9g/%.9g b %lld/%.17g frac %.9g/%.9g in_range %d\n",
                               r, p, f2u(p), o, end, end_ref, b, fl, frac, frac_ref, (int)in_range);
                    bad++;
                }
            }
        }
    }
    printf("%ld cases, %ld declined (non-normal input), %ld mismatches\n", total, declined, bad);

    // ray step count: gx_step_count against the float64 loop it replaces,
    // on random rays and on rays whose length sits at a step boundary
    long sbad = 0, stotal = 0, sdecl = 0;
    std::uniform_int_distribution<int> Ucap(1, 4200);
    for (long i = 0; i < 40 * n; i++) {
        const int mode = (int)(i % 5);
        const double u = U(g), u2 = U(g);
        // sk: the dominant component of a unit float32 direction, |sk| in [1/sqrt(3), 1]
        float sk = (float)(0.57735026918962573 + u * (1.0 - 0.57735026918962573));
        if (u2 < 0.5) sk = -sk;
        if (mode == 3) sk = (u2 < 0.5) ? -1.0f : 1.0f;
        double inc = std::fabs(1.0 / (double)sk);
        if (mode == 4 && (i / 5) % 2 == 0) {
            // increments whose mantissa ends at bit s0: additions tie at the 2^s0 grid
            const int s0 = 1 + (int)(g() % 13);
            inc = 1.0 + std::ldexp((double)(2 * (g() % 1000003) + 1), s0 - 1 - 52 + 1) * (u2 < 0.5 ? 1.0 : 0.5);
        }
        float rl;
        int cap = mode == 4 ? Ucap(g) : 520;
        if (mode == 0) rl = (float)(1.0 + U(g) * 600.0);
        else if (mode == 1 || mode == 3) {  // (rl - 1) |sk| within 1e-5 of an integer: the float32 margin fails here
            const double k = std::floor(U(g) * 400.0) + 1.0;
            rl = (float)(1.0 + (k + (U(g) - 0.5) * 2e-5) * inc);
        } else if (mode == 2) rl = (float)(1.0 + U(g) * 3.0);          // short rays
        else rl = (float)(1.0 + U(g) * 8000.0);                         // long rays, any cap
        const double R = (double)rl - 1.0;
        double L = 0.0;
        int Kref = 0;
        while (L < R && Kref < cap) {
            Kref++;
            L = L + inc;
        }
        const int K = gx_step_count(R, inc, cap);
        stotal++;
        if (K < 0) { sdecl++; continue; }
        if (K != Kref) {
            if (sbad < 20) printf("STEP MISMATCH rl=%.9g sk=%.9g cap=%d: %d vs %d\n", rl, sk, cap, K, Kref);
            sbad++;
        }
    }
    printf("%ld step-count cases, %ld declined, %ld step-count mismatches\n", stotal, sdecl, sbad);
    return (bad || sbad) ? 1 : 0;
}
