// Exact float64 voxel arithmetic of the reference without the float64 pipe.
//
// For a float32 coordinate p, a float64 voxel size r > 0 and an integer grid
// origin o, the reference computes in float64 (scripts/gvom.py:1153-1184,
// 1262-1264, 1399-1416):
//     q = RN64(p / r)          (the point in voxel units)
//     end = RN32(q)            (the ray end point, stored as float32)
//     t = RN64(q - o)
//     b = floor(t)             (the voxel index)
//     frac = RN32(t - b)       (the in-voxel fraction; t - b is exact)
// GB300 runs float64 at 1/64 of the float32 rate, so these are evaluated
// here with 64/128-bit integer arithmetic that reproduces IEEE round-to-
// nearest-even exactly:
//   * p = mp 2^ep (24-bit mp), r = mr 2^er (53-bit mr); with the host-made
//     W = floor(2^116 / mr), N = floor(mp W / 2^31) is floor(mp 2^85 / mr) or
//     one less; the exact remainder mp 2^85 - N mr fixes it and gives the
//     sticky bit, so rounding N (56-57 bits) to 53 bits is exact;
//   * q - o, its floor and fraction are fixed-point integer operations.
// Functions are __host__ __device__ so the host unit tests run the same code.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GX_HD __host__ __device__ __forceinline__
#else
#define GX_HD static inline
#endif

namespace gvom {

// Per-resolution constants (host-made): r = mr * 2^er, W = floor(2^116 / mr).
struct ExactRes {
    unsigned long long mr;
    unsigned long long W;
    int er;
    int pad;
};

GX_HD unsigned long long gx_mulhi(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

GX_HD int gx_clz64(unsigned long long x) {  // x != 0
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

GX_HD unsigned gx_f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

GX_HD float gx_u2f(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// 128-bit two's-complement value hi:lo
struct gx_i128 {
    unsigned long long hi, lo;
};

GX_HD gx_i128 gx_sub(gx_i128 a, gx_i128 b) {
    gx_i128 r;
    r.lo = a.lo - b.lo;
    r.hi = a.hi - b.hi - (a.lo < b.lo ? 1ull : 0ull);
    return r;
}

GX_HD bool gx_neg(gx_i128 a) { return (long long)a.hi < 0; }

GX_HD gx_i128 gx_negate(gx_i128 a) {
    gx_i128 z = {0, 0};
    return gx_sub(z, a);
}

// a << s for 0 <= s < 128 (a >= 0 assumed to fit)
GX_HD gx_i128 gx_shl(unsigned long long a, int s) {
    gx_i128 r;
    if (s == 0) {
        r.hi = 0;
        r.lo = a;
    } else if (s < 64) {
        r.hi = a >> (64 - s);
        r.lo = a << s;
    } else {
        r.hi = a << (s - 64);
        r.lo = 0;
    }
    return r;
}

// Round the positive 128-bit magnitude m to `bits` significant bits (half to
// even).  Returns the rounded mantissa (in [2^(bits-1), 2^bits]) and the
// binary exponent e with value = mant * 2^e (relative to m's scale).
GX_HD unsigned long long gx_round_mag(gx_i128 m, int bits, int &e) {
    int L;
    if (m.hi) L = 128 - gx_clz64(m.hi);
    else L = 64 - gx_clz64(m.lo);
    if (L <= bits) {
        e = 0;
        return m.lo;  // fits, exact (L <= 53 < 64)
    }
    const int sh = L - bits;  // 1 .. 127
    unsigned long long mant, rb_hi_bit_set, below;
    // mant = m >> sh; rb = m & (2^sh - 1); compare rb with 2^(sh-1)
    if (sh < 64) {
        mant = (m.lo >> sh) | (sh ? (m.hi << (64 - sh)) : 0ull);
        const unsigned long long rb = m.lo & ((1ull << sh) - 1ull);
        const unsigned long long half = 1ull << (sh - 1);
        rb_hi_bit_set = rb >= half;
        below = (rb & (half - 1ull)) != 0ull;
    } else if (sh == 64) {
        mant = m.hi;
        rb_hi_bit_set = m.lo >> 63;
        below = (m.lo & 0x7fffffffffffffffull) != 0ull;
    } else {
        const int s2 = sh - 64;
        mant = m.hi >> s2;
        const unsigned long long rbh = m.hi & ((1ull << s2) - 1ull);
        const unsigned long long half = 1ull << (s2 - 1);
        rb_hi_bit_set = rbh >= half;
        below = ((rbh & (half - 1ull)) != 0ull) || m.lo != 0ull;
    }
    const bool up = rb_hi_bit_set && (below || (mant & 1ull));
    mant += up ? 1ull : 0ull;
    e = sh;
    return mant;
}

// float32 bits of sign * mant * 2^e with mant < 2^25 already rounded to 24
// significant bits (mant may equal 2^24 after rounding).  Returns false
// outside the normal float32 range.
GX_HD bool gx_make_f32(unsigned sign, unsigned long long mant, int e, float &out) {
    if (mant == 0) {
        out = gx_u2f(sign << 31);
        return true;
    }
    // normalise mant into [2^23, 2^24)
    const int L = 64 - gx_clz64(mant);
    const int shift = L - 24;  // mant is exact at 24 bits: only exact shifts
    if (shift > 0) {
        mant >>= shift;
        e += shift;
    } else if (shift < 0) {
        mant <<= -shift;
        e -= -shift;
    }
    const int be = e + 23 + 127;
    if (be <= 0 || be >= 255) return false;
    out = gx_u2f((sign << 31) | ((unsigned)be << 23) | ((unsigned)mant & 0x7fffffu));
    return true;
}

// q = RN64(p / r) as sign * M * 2^E (M in [2^52, 2^53)); p finite nonzero normal float32.
GX_HD bool gx_quotient(float p, const ExactRes &R, unsigned &sign, unsigned long long &M, int &E) {
    const unsigned b = gx_f2u(p);
    sign = b >> 31;
    const int be = (b >> 23) & 0xff;
    if (be == 0 || be == 0xff) return false;  // zero, subnormal, inf, NaN
    const unsigned long long mp = (b & 0x7fffffu) | 0x800000u;
    const int ep = be - 127 - 23;
    // N ~= floor(mp 2^85 / mr)
    const unsigned long long plo = mp * R.W, phi = gx_mulhi(mp, R.W);
    unsigned long long N = (phi << 33) | (plo >> 31);
    // remainder mp 2^85 - N mr (exactly; expected in [0, 2 mr))
    unsigned long long nlo = N * R.mr, nhi = gx_mulhi(N, R.mr);
    gx_i128 num = {mp << 21, 0ull};
    gx_i128 rem = gx_sub(num, gx_i128{nhi, nlo});
    if (rem.hi != 0ull) return false;  // cannot happen (estimate error < 1)
    unsigned long long rlo = rem.lo;
    if (rlo >= R.mr) {
        N += 1ull;
        rlo -= R.mr;
    }
    if (rlo >= R.mr) return false;
    // round N (56..57 bits) to 53 bits, half to even, with the remainder as sticky
    const int L = 64 - gx_clz64(N);
    const int sh = L - 53;
    unsigned long long m = N >> sh;
    const unsigned long long rb = N & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    const bool up = rb > half || (rb == half && (rlo != 0ull || (m & 1ull)));
    m += up ? 1ull : 0ull;
    int e = sh;
    if (m == (1ull << 53)) {
        m >>= 1;
        e += 1;
    }
    M = m;
    E = e - 85 + ep - R.er;
    return true;
}

// All the reference quantities for one coordinate.  Returns false only for
// inputs outside what the grid arithmetic can mean (non-finite, subnormal,
// |o| >= 2^31); the caller then uses float64.  in_range = false when |t| is
// too large for any grid (b is then meaningless).
GX_HD bool gx_coord(float p, const ExactRes &R, long long o, float &end, long long &bidx, float &frac, bool &in_range) {
    in_range = true;
    if (!(o > -(1ll << 31) && o < (1ll << 31))) return false;
    if (gx_f2u(p) << 1 == 0u) {  // p = +-0: q = +-0, t = -o exactly
        end = p;
        bidx = -o;
        frac = 0.0f;
        return true;
    }
    unsigned s;
    unsigned long long M;
    int E;
    if (!gx_quotient(p, R, s, M, E)) return false;
    // end = RN32(q)
    {
        const unsigned long long m24 = M >> 29, rb = M & ((1ull << 29) - 1ull), half = 1ull << 28;
        const bool up = rb > half || (rb == half && (m24 & 1ull));
        if (!gx_make_f32(s, m24 + (up ? 1ull : 0ull), E + 29, end)) return false;
    }
    if (E >= 0) {  // |q| >= 2^52: outside any grid
        in_range = false;
        bidx = 0;
        frac = 0.0f;
        return true;
    }
    const int k = -E;  // fractional bits of q
    // |o| 2^k must fit the 128-bit fixed point: k <= 95 (|q| >= 2^-43); smaller
    // nonzero |q| (within 1e-13 voxel of a world axis plane) declines
    if (k > 95) return false;
    // D = s*M - o*2^k  (value t_exact * 2^k), as 128-bit
    gx_i128 A = {0ull, M};
    if (s) A = gx_negate(A);
    const unsigned long long ao = (unsigned long long)(o < 0 ? -o : o);
    gx_i128 Bv = gx_shl(ao, k);
    if (o < 0) Bv = gx_negate(Bv);
    gx_i128 D = gx_sub(A, Bv);
    const bool dneg = gx_neg(D);
    gx_i128 mag = dneg ? gx_negate(D) : D;
    if (mag.hi == 0ull && mag.lo == 0ull) {  // t = 0
        bidx = 0;
        frac = 0.0f;
        return true;
    }
    // t = RN64(D 2^-k) = tm * 2^(te - k), tm <= 2^53
    int te;
    const unsigned long long tm = gx_round_mag(mag, 53, te);
    const int ex = te - k;  // t = +-tm * 2^ex
    if (ex >= 0) {
        // integer t; |t| >= 2^31 is outside any grid
        if (ex > 30 || tm >= (1ull << (31 - ex))) {
            in_range = false;
            bidx = 0;
            frac = 0.0f;
            return true;
        }
        const long long tv = (long long)(tm << ex);
        bidx = dneg ? -tv : tv;
        frac = 0.0f;
        return true;
    }
    const int kk = -ex;  // fractional bits of t (tm < 2^54)
    // floor and fraction of +-tm * 2^-kk
    long long fl;
    unsigned long long F;  // fraction numerator, in [0, 2^kk)
    if (kk >= 64) {
        // |t| < 2^-10: floor is 0 or -1
        if (!dneg) {
            fl = 0;
            F = tm;
        } else {
            fl = -1;
            // F = 2^kk - tm; express with a reduced scale: frac = 1 - tm 2^-kk
            // (tm 2^-kk < 2^-10, so RN32(1 - tiny) below)
            F = 0;
        }
        if (dneg) {
            // frac = 1 - tm * 2^-kk: the exact value is in (1 - 2^-10, 1)
            gx_i128 one = gx_shl(1ull, kk >= 127 ? 126 : kk);
            if (kk >= 127) return false;
            gx_i128 fm = gx_sub(one, gx_i128{0ull, tm});
            int fe;
            const unsigned long long f24 = gx_round_mag(fm, 24, fe);
            if (!gx_make_f32(0u, f24, fe - kk, frac)) return false;
            bidx = fl;
            return true;
        }
    } else {
        const unsigned long long ip = tm >> kk;  // integer part of |t|
        const unsigned long long fp = tm & ((kk == 64 ? 0ull : (1ull << kk)) - 1ull);
        if (ip >= (1ull << 31)) {
            in_range = false;
            bidx = 0;
            frac = 0.0f;
            return true;
        }
        if (!dneg) {
            fl = (long long)ip;
            F = fp;
        } else if (fp == 0ull) {
            fl = -(long long)ip;
            F = 0ull;
        } else {
            fl = -(long long)ip - 1;
            F = (1ull << kk) - fp;
        }
    }
    bidx = fl;
    if (F == 0ull) {
        frac = 0.0f;
        return true;
    }
    int fe;
    const unsigned long long f24 = gx_round_mag(gx_i128{0ull, F}, 24, fe);
    return gx_make_f32(0u, f24, fe - kk, frac);
}

// Number of iterations of the reference's ray-length loop
//     L = 0; K = 0; while (L < R && K < cap) { K++; L = RN64(L + inc); }
// (scripts/gvom.py:1206-1231: R = ray_length - 1, inc = |1.0 / slope|, both
// float64), without float64 arithmetic.  After the first iteration L = inc
// and every later value is a multiple of inc's ulp u0; L is kept as q 2^s u0
// with q in [2^52, 2^53), so one addition is q + n + f / 2^s with
// n = I >> s, f = I mod 2^s (I = inc / u0).  Inside one binade that sum
// rounds the same way at every step -- q + n + (2f > 2^s) -- unless the
// fraction is a tie, so runs of steps are taken at once up to the binade's
// end or to R; ties and binade crossings are single steps, rounded to nearest
// even at the grid of the result.  Requires R, inc finite, inc > 0.
GX_HD unsigned long long gx_d2u(double d) {
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(d);
#else
    unsigned long long u;
    memcpy(&u, &d, 8);
    return u;
#endif
}

GX_HD int gx_step_count(double R, double inc, int cap) {
    if (!(R > 0.0) || cap <= 0) return 0;
    const unsigned long long ib = gx_d2u(inc), rb = gx_d2u(R);
    const int ie = (int)((ib >> 52) & 0x7ff), re = (int)((rb >> 52) & 0x7ff);
    if (ie == 0 || ie == 0x7ff || re == 0x7ff) return -1;  // subnormal or non-finite: caller's float64 path
    const unsigned long long I = (ib & 0xfffffffffffffull) | (1ull << 52);
    // R / u0 = mR 2^(re - ie); R subnormal: exponent as for re = 1, no implicit bit
    const unsigned long long mR = re ? ((rb & 0xfffffffffffffull) | (1ull << 52)) : (rb & 0xfffffffffffffull);
    const int rsh = (re ? re : 1) - ie;
    const unsigned long long top = 1ull << 53;
    unsigned long long q = I;
    int s = 0, K = 1;
    while (true) {
        // Rq = ceil(R / (u0 2^s)), clamped far above any q
        unsigned long long Rq;
        const int sh = rsh - s;
        if (sh >= 10) Rq = ~0ull;
        else if (sh >= 0) Rq = mR << sh;
        else if (sh > -64) Rq = (mR >> -sh) + ((mR & ((1ull << -sh) - 1ull)) ? 1ull : 0ull);
        else Rq = 1ull;
        if (q >= Rq) return K;
        if (K >= cap) return cap;
        if (s >= 52) return -1;  // far beyond any ray; caller's float64 path
        const unsigned long long n = I >> s, f = I & ((1ull << s) - 1ull), half = s ? 1ull << (s - 1) : 0ull;
        if (!(s > 0 && f == half) && q + n + 1ull < top) {
            // a run of steps inside the binade, each adding d
            const unsigned long long d = n + ((s > 0 && f > half) ? 1ull : 0ull);
            const unsigned long long tb = (top - 2ull - n - q) / d + 1ull;  // steps whose exact sum stays below 2^53
            const unsigned long long tr = Rq == ~0ull ? ~0ull : (Rq - q + d - 1ull) / d;  // steps until q >= Rq
            unsigned long long t = tb < tr ? tb : tr;
            if (t > (unsigned long long)(cap - K)) t = (unsigned long long)(cap - K);
            q += t * d;
            K += (int)t;
            continue;
        }
        // one step: exact sum T + f / 2^s in units of 2^s
        const unsigned long long T = q + n;
        unsigned long long nq;
        if (T < top) {  // stays below 2^53: round at grid 2^s
            const bool up = s > 0 && (f > half || (f == half && (T & 1ull)));
            nq = T + (up ? 1ull : 0ull);
        } else {  // crosses into the next binade: grid 2^(s+1)
            if (!(T & 1ull)) nq = T >> 1;
            else if (f > 0ull) nq = (T >> 1) + 1ull;
            else nq = ((T >> 1) & 1ull) ? (T >> 1) + 1ull : (T >> 1);  // tie: to even
            s++;
        }
        if (nq >= top) {  // rounded up to the next power of two
            nq >>= 1;
            s++;
        }
        q = nq;
        K++;
    }
}

}  // namespace gvom
