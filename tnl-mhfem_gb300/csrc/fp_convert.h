// FP64 -> FP32 conversion with round-to-nearest-even on the integer pipes.
//
// GB300 issues FP64 instructions at about 1/57 of the FP32 rate, and the
// hardware conversion F2F.F32.F64 shares that scarce pipe: the mixed form's
// assembly, which writes an FP32 copy of every matrix value beside the FP64
// one, spent most of its extra time in those conversions.  IEEE 754 binary64
// -> binary32 rounding is a pure bit-field operation for results in the
// binary32 normal range: keep the sign, rebias the exponent (1023 -> 127),
// keep the top 23 of the 52 fraction bits and round the dropped 29 bits to
// nearest, ties to even (a carry out of the fraction correctly increments
// the exponent, and one out of the largest finite exponent gives infinity,
// as IEEE rounding does).  That takes a handful of integer instructions.
// Zeros keep their sign; every other input outside the normal range (FP32
// subnormal results, infinities, NaN) takes the hardware conversion.
//
// The header compiles as plain C++ too, so the host test suite checks the
// function against the compiler's (IEEE) double -> float cast.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define MHFEM_HD __host__ __device__ __forceinline__
#else
#define MHFEM_HD inline
#endif

namespace mhfem {

MHFEM_HD float f64_to_f32_rn(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t e = (hi >> 20) & 0x7ffu;          // binary64 biased exponent
    uint32_t f;
    if (e >= 1023u - 126u && e <= 1023u + 127u) {
        // sign | rebiased exponent | top 23 fraction bits (20 from hi, 3 from lo)
        f = (hi & 0x80000000u) | ((e - (1023u - 127u)) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const uint32_t r = lo & 0x1fffffffu;          // the 29 dropped bits; a tie is 0x10000000
        f += (r + (f & 1u) > 0x10000000u) ? 1u : 0u;  // above the tie, or the tie with an odd result
    }
    else if ((b << 1) == 0)
        f = hi & 0x80000000u;                         // +-0
    else
        return (float)v;                              // subnormal results, infinities, NaN
    float out;
    std::memcpy(&out, &f, sizeof out);
    return out;
}

// FP32 -> FP64 (exact) on the integer pipes: normal inputs rebias the
// exponent and widen the fraction; zeros keep their sign; subnormals,
// infinities and NaN take the hardware conversion.
MHFEM_HD double f32_to_f64(float v)
{
    uint32_t f;
    std::memcpy(&f, &v, sizeof f);
    const uint32_t e = (f >> 23) & 0xffu;
    uint64_t b;
    if (e != 0u && e != 0xffu)
        b = ((uint64_t)(f & 0x80000000u) << 32) | ((uint64_t)(e + (1023u - 127u)) << 52) |
            ((uint64_t)(f & 0x7fffffu) << 29);
    else if ((f << 1) == 0)
        b = (uint64_t)(f & 0x80000000u) << 32;
    else
        return (double)v;
    double out;
    std::memcpy(&out, &b, sizeof out);
    return out;
}

}  // namespace mhfem
