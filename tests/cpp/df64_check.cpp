// CPU check of the double-float helpers of q1tsim_gb300/csrc/df64.cuh, built
// with g++ -ffp-contract=off by tests/test_host_logic.py.  Prints one line of
// figures; exit status 1 on any failed check.
#define __host__
#define __device__
#define __forceinline__ inline
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "../../q1tsim_gb300/csrc/df64.cuh"

using namespace q1g;

static uint64_t dbits(double d)
{
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return u;
}
static double bitsd(uint64_t u)
{
    double d;
    std::memcpy(&d, &u, 8);
    return d;
}

int main()
{
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(-1, 1);
    int bad = 0;
    double worst_split = 0, worst_join = 0, worst_dot = 0, sum2 = 0;
    long cnt = 0;
    // split: h + l == x to 2^-48 relative in range, 2^-98 absolute below it
    for (int t = 0; t < 400000; ++t) {
        const double x = t % 97 == 0 ? 0.0 : U(rng) * std::ldexp(1.0, 60 - (int)(rng() % 200));
        DF v;
        if (!split_f64(dbits(x), v)) {
            if (std::fabs(x) < std::ldexp(1.0, 126)) ++bad;
            continue;
        }
        const long double err = std::fabs((long double)v.h + (long double)v.l - (long double)x);
        if (std::fabs(x) < std::ldexp(1.0, -74)) {
            if (err > std::ldexp(1.0L, -98)) ++bad;
            continue;
        }
        if (x != 0) worst_split = std::fmax(worst_split, (double)(err / std::fabs((long double)x)));
        // the fast form agrees bit for bit wherever it applies
        if (split_fast_ok(dbits(x))) {
            const DF f = split_fast(dbits(x));
            if (float_to_bits(f.h) != float_to_bits(v.h) || float_to_bits(f.l) != float_to_bits(v.l)) ++bad;
        }
    }
    // values whose rounding carries into the exponent
    for (int t = 0; t < 20000; ++t) {
        uint64_t b = dbits(1.0 + std::fabs(U(rng))) | 0x000FFFFFF0000000ull;
        const double x = bitsd(b) * std::ldexp(1.0, -(int)(rng() % 60));
        DF v;
        if (!split_f64(dbits(x), v)) ++bad;
        const long double err = std::fabs((long double)v.h + (long double)v.l - (long double)x);
        if (err > std::ldexp(1.0L, -47) * std::fabs((long double)x)) ++bad;
        if (split_fast_ok(dbits(x))) {
            const DF f = split_fast(dbits(x));
            if (float_to_bits(f.h) != float_to_bits(v.h) || float_to_bits(f.l) != float_to_bits(v.l)) ++bad;
        }
    }
    // join: normalised pairs (TwoSum of random floats, powers of two with
    // small terms of either sign)
    for (int t = 0; t < 400000; ++t) {
        float a = (float)U(rng) * std::ldexp(1.0f, -(int)(rng() % 60));
        const float b = (float)U(rng) * std::ldexp(1.0f, -(int)(rng() % 90));
        if (t % 7 == 0) a = std::ldexp(1.0f, -(int)(rng() % 60)) * (rng() % 2 ? 1.f : -1.f);
        volatile float h = a + b;
        volatile float bv = h - a;
        volatile float av = h - bv;
        const float l = (a - av) + (b - bv);
        if (h == 0 || std::fabs(h) < std::ldexp(1.0f, -73)) continue;
        const double got = bitsd(join_f64(DF{h, l}));
        const long double want = (long double)h + (long double)l;
        worst_join = std::fmax(worst_join, (double)(std::fabs((long double)got - want) / std::fabs(want)));
    }
    // 4-term dot products of split doubles, with forced cancellation
    for (int t = 0; t < 400000; ++t) {
        double av[4], bv[4];
        DF a[4], b[4];
        long double exact = 0, mag = 0;
        bool ok = true;
        for (int k = 0; k < 4; ++k) {
            av[k] = U(rng);
            bv[k] = U(rng) * std::ldexp(1.0, -(int)(rng() % 20));
            ok &= split_f64(dbits(av[k]), a[k]) && split_f64(dbits(bv[k]), b[k]);
            exact += (long double)av[k] * bv[k];
            mag = std::fmax((double)mag, std::fabs(av[k] * bv[k]));
        }
        if (!ok) continue;
        if (t % 5 == 0) {
            av[3] = -(double)((long double)av[0] * bv[0] + (long double)av[1] * bv[1] +
                              (long double)av[2] * bv[2]) / bv[3];
            if (std::fabs(av[3]) > 1e30) continue;
            split_f64(dbits(av[3]), a[3]);
            exact = 0;
            for (int k = 0; k < 4; ++k) exact += (long double)av[k] * bv[k];
            mag = 0;
            for (int k = 0; k < 4; ++k) mag = std::fmax((double)mag, std::fabs(av[k] * bv[k]));
        }
        const double got = bitsd(join_f64(dot4(a, b)));
        const double e = (double)(std::fabs((long double)got - exact) / mag);
        worst_dot = std::fmax(worst_dot, e);
        sum2 += e * e;
        ++cnt;
    }
    const double rms = std::sqrt(sum2 / cnt);
    if (worst_split > std::ldexp(1.0, -47)) ++bad;
    if (worst_join > std::ldexp(1.0, -52)) ++bad;
    if (worst_dot > std::ldexp(1.0, -43) || rms > std::ldexp(1.0, -47)) ++bad;
    std::printf("bad %d split %.3e join %.3e dot_worst %.3e dot_rms %.3e\n", bad, worst_split, worst_join, worst_dot,
                rms);
    return bad != 0;
}
