// convert.h — IEEE 754 binary64 -> binary32 conversion with integer
// operations only.
//
// On this GPU an FP64 warp instruction, the double -> float conversion
// included, holds its scheduler for many cycles, which made the HBM-bound
// copy and split kernels FP64-issue-bound.  The conversion below is the
// standard round-to-nearest-even narrowing of the binary64 format (IEEE
// 754-2008, sections 3.4 and 4.3.1): rebias the exponent, round the 52-bit
// significand to 23 bits (or to fewer bits, including the implicit one, when
// the result is subnormal), carry into the exponent, and saturate to
// infinity; NaNs stay NaNs (quiet, sign kept).  It runs on the integer ALUs
// and compiles for the host too, where tests compare it with the host
// compiler's own conversion.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PSDGB_HD __host__ __device__ __forceinline__
#else
#define PSDGB_HD inline
#endif

namespace psdgb {

PSDGB_HD uint64_t bits_of_double(double x) {
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(x));
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

PSDGB_HD float float_of_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
#endif
}

PSDGB_HD uint32_t bits_of_float(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

PSDGB_HD double double_of_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

PSDGB_HD int clz32(uint32_t x) {  // x != 0
#if defined(__CUDA_ARCH__)
    return __clz(static_cast<int>(x));
#else
    return __builtin_clz(x);
#endif
}

// The binary32 value x as binary64, exactly (IEEE 754-2008, 5.4.2: every
// binary32 number is a binary64 number): rebias the exponent and widen the
// significand; a subnormal input is normalised; infinities carry over and
// NaNs stay NaNs (quiet, payload kept).
PSDGB_HD double f2d(float x) {
    const uint32_t b = bits_of_float(x);
    const uint64_t sign = static_cast<uint64_t>(b & 0x80000000u) << 32;
    const int e32 = static_cast<int>((b >> 23) & 0xFF);
    const uint32_t m = b & 0x007FFFFFu;
    if (e32 == 0xFF)
        return double_of_bits(sign | 0x7FF0000000000000ull | (static_cast<uint64_t>(m) << 29) |
                              (m ? 0x0008000000000000ull : 0ull));
    if (e32 != 0)
        return double_of_bits(sign | (static_cast<uint64_t>(e32 - 127 + 1023) << 52) |
                              (static_cast<uint64_t>(m) << 29));
    if (m == 0) return double_of_bits(sign);
    // m * 2^-149 with its top set bit at position t (0 .. 22): 1.f * 2^(t - 149)
    const int t = 31 - clz32(m);
    const uint64_t f = (static_cast<uint64_t>(m) << (52 - t)) & 0x000FFFFFFFFFFFFFull;
    return double_of_bits(sign | (static_cast<uint64_t>(t - 149 + 1023) << 52) | f);
}

// Round the binary64 value x to the nearest binary32 value, ties to even.
PSDGB_HD float d2f_rn(double x) {
    const uint64_t b = bits_of_double(x);
    const uint32_t sign = static_cast<uint32_t>(b >> 32) & 0x80000000u;
    const int e64 = static_cast<int>((b >> 52) & 0x7FF);
    const uint64_t frac = b & 0x000FFFFFFFFFFFFFull;
    if (e64 == 0x7FF)  // infinity or NaN (NaN: quiet, top payload bits kept)
        return float_of_bits(sign | 0x7F800000u | (frac ? (0x00400000u | static_cast<uint32_t>(frac >> 29)) : 0u));
    const int e = e64 - 1023 + 127;  // biased binary32 exponent of the value
    if (e >= 0xFF) return float_of_bits(sign | 0x7F800000u);  // overflow
    if (e >= 1) {
        // Normal result: 23 kept bits, 29 rounded off.
        uint32_t m = static_cast<uint32_t>(frac >> 29);
        const uint64_t rest = frac & 0x1FFFFFFFull;
        const uint64_t half = 0x10000000ull;
        if (rest > half || (rest == half && (m & 1u))) ++m;
        // A carry out of the significand bumps the exponent (possibly to
        // infinity): adding to the packed exponent|significand does both.
        const uint32_t packed = (static_cast<uint32_t>(e) << 23) + m;
        return float_of_bits(sign | packed);
    }
    // Subnormal or zero result: the significand with its implicit one,
    // shifted right by 29 + (1 - e) bits, rounded to nearest even.
    const int shift = 29 + (1 - e);
    if (e64 == 0 || shift > 53) return float_of_bits(sign);  // |x| < 2^-150: rounds to zero
    const uint64_t sig = frac | 0x0010000000000000ull;
    uint32_t m = static_cast<uint32_t>(sig >> shift);
    const uint64_t rest = sig & ((1ull << shift) - 1ull);
    const uint64_t half = 1ull << (shift - 1);
    if (rest > half || (rest == half && (m & 1u))) ++m;
    // m may round up to 0x800000, the smallest normal number: the packing
    // with exponent field 0 gives exactly that encoding.
    return float_of_bits(sign | m);
}

}  // namespace psdgb
