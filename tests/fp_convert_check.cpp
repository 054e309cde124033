// Host check of the integer-pipe conversions of csrc/fp_convert.h against the
// compiler's IEEE casts (round to nearest even): random bit patterns, random
// values over the binary32 exponent range, every tie and near-tie around
// random binary32 values at every exponent, and the range edges (zeros,
// largest finite, overflow to infinity, the smallest normal, subnormal
// results, infinities, NaN).  Exits non-zero on the first mismatch class.
#include "fp_convert.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

static long bad = 0, n = 0;

static void check(double v)
{
    const float a = mhfem::f64_to_f32_rn(v), b = (float)v;
    uint32_t ia, ib;
    std::memcpy(&ia, &a, 4);
    std::memcpy(&ib, &b, 4);
    ++n;
    if (ia != ib && !(std::isnan(a) && std::isnan(b))) {
        if (bad < 10) std::printf("f64_to_f32_rn(%a) = %a, cast gives %a\n", v, a, b);
        ++bad;
    }
    if (!std::isnan(b)) {
        const double w = mhfem::f32_to_f64(b), c = (double)b;
        if (std::memcmp(&w, &c, 8) != 0) {
            if (bad < 10) std::printf("f32_to_f64(%a) = %a, cast gives %a\n", (double)b, w, c);
            ++bad;
        }
    }
}

int main()
{
    std::mt19937_64 g(20261204);
    for (long i = 0; i < 2000000; ++i) {
        const uint64_t u = g();
        double v;
        std::memcpy(&v, &u, 8);
        check(v);
    }
    for (long i = 0; i < 2000000; ++i) {
        double v = std::ldexp((double)(g() >> 11), -53) * std::ldexp(1.0, (int)(g() % 300) - 150);
        check((g() & 1) ? -v : v);
    }
    const int64_t offsets[] = {0x10000000, 0x0fffffff, 0x10000001, -0x10000000, -0x0fffffff, 0x1fffffff, 1, -1};
    for (int ex = -149; ex <= 128; ++ex)
        for (int k = 0; k < 200; ++k) {
            const float fl = std::ldexp(1.0f + (float)(g() % 8388608) / 8388608.0f, ex);
            const double d = fl;
            uint64_t u;
            std::memcpy(&u, &d, 8);
            for (int64_t off : offsets) {
                const uint64_t w = u + (uint64_t)off;
                double v;
                std::memcpy(&v, &w, 8);
                check(v);
                check(-v);
            }
        }
    const double edges[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 3.40282357e38,
                            1e39, 1.1754943508222875e-38, 1.1754942e-38, 1e-45, 1e-300, (double)INFINITY,
                            -(double)INFINITY, (double)NAN};
    for (double v : edges) check(v);
    std::printf("%ld conversions checked, %ld mismatches\n", n, bad);
    return bad != 0;
}
