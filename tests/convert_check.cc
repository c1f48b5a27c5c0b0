// Checks psdgb::d2f_rn (csrc/convert.h, the integer-only binary64 -> binary32
// narrowing the copy and split kernels use) against the host compiler's own
// conversion: random bit patterns, values across and below the binary32
// range, exact ties and near-ties around every binary32 exponent, and the
// special values; and psdgb::f2d (the exact binary32 -> binary64 widening of
// the batch Lanczos) on every binary32 bit pattern.  Exit status 0 when every
// result has the same bits (NaN: any NaN).
#include "convert.h"

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

using psdgb::d2f_rn;
using psdgb::f2d;

static unsigned bits(float f) {
    unsigned b;
    std::memcpy(&b, &f, 4);
    return b;
}

static double from_bits(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

int main() {
    std::mt19937_64 rng(7);
    long checked = 0, bad = 0;
    auto check = [&](double x) {
        const float got = d2f_rn(x), want = static_cast<float>(x);
        ++checked;
        const bool ok = std::isnan(want) ? std::isnan(got) : bits(got) == bits(want);
        if (!ok && ++bad <= 10) std::printf("mismatch at %a: %a, expected %a\n", x, double(got), double(want));
    };
    for (long i = 0; i < 2000000; ++i) check(from_bits(rng()));
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (long i = 0; i < 1000000; ++i) check(std::ldexp(u(rng), static_cast<int>(rng() % 330) - 165));
    for (int ex = -160; ex <= 130; ++ex)
        for (int k = 0; k < 200; ++k) {
            const unsigned long long m = rng() & ((1ull << 23) - 1);
            const double base = std::ldexp(1.0 + double(m) / double(1 << 23), ex);
            const double ulp = std::ldexp(1.0, ex - 23);
            for (double off : {0.5, -0.5, 0.5 + 1e-12, 0.5 - 1e-12, 0.25, 0.75}) check(base + off * ulp);
        }
    const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, DBL_MIN, -DBL_MIN, DBL_MAX, FLT_MAX,
                               double(FLT_MAX) + std::ldexp(1.0, 103), double(FLT_MAX) + std::ldexp(0.999, 103),
                               FLT_MIN, FLT_TRUE_MIN, FLT_TRUE_MIN * 0.5, FLT_TRUE_MIN * 0.5000001,
                               FLT_TRUE_MIN * 0.4999999, FLT_TRUE_MIN * 1.5, FLT_TRUE_MIN * 2.5,
                               std::ldexp(1.0, -150), std::ldexp(1.0, -151), 1.0, -3.0, 1e300, -1e-300,
                               4.9406564584124654e-324};
    for (double s : specials) check(s);
    // f2d: all 2^32 binary32 patterns, every 7th one (every exponent, both
    // signs, subnormals, infinities, NaNs) plus the first and last 2^20
    auto check_w = [&](unsigned b) {
        float f;
        std::memcpy(&f, &b, 4);
        const double got = f2d(f), want = static_cast<double>(f);
        unsigned long long gb, wb;
        std::memcpy(&gb, &got, 8);
        std::memcpy(&wb, &want, 8);
        ++checked;
        const bool ok = std::isnan(want) ? std::isnan(got) : gb == wb;
        if (!ok && ++bad <= 10) std::printf("f2d mismatch at %08x: %a, expected %a\n", b, got, want);
    };
    for (unsigned long long b = 0; b < (1ull << 32); b += 7) check_w(static_cast<unsigned>(b));
    for (unsigned b = 0; b < (1u << 20); ++b) {
        check_w(b);
        check_w(0x80000000u | b);
        check_w(0x7F800000u - b);
        check_w(0xFFFFFFFFu - b);
    }
    std::printf("checked %ld values, %ld mismatches\n", checked, bad);
    return bad == 0 ? 0 : 1;
}
