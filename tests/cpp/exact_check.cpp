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
    return bad ? 1 : 0;
}
