// Float <-> double conversions with integer instructions, for the FP64
// residual replacement: the conversion instructions run on the FP64 pipe,
// which bounds that kernel, while its integer pipes are mostly idle.  Both
// are exact for every normal float (the widening places sign, rebiased
// exponent and mantissa bits; the narrowing rounds to nearest even by adding
// 2^28 - 1 plus the lowest kept mantissa bit below the cut and truncating,
// the carry running into the exponent).  They differ from the conversion
// instructions only where the solver has no use for the difference: float
// subnormals become a signed zero, and the narrowing turns a NaN into an
// infinity of its sign (still non-finite, as the solver's checks ask).
// Plain C++ as well, so that a host test checks them against the native
// conversions.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define FT_HD __host__ __device__ __forceinline__
#else
#define FT_HD inline
#endif

namespace ft {

FT_HD uint32_t f_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

FT_HD double widen_f(float f)
{
    const uint32_t u = f_bits(f);
    const uint32_t sgn = u & 0x80000000u, m = u & 0x7fffffffu;
    uint32_t hi = sgn | ((m >> 3) + (896u << 20));  // exponent rebias 127 -> 1023
    uint32_t lo = u << 29;
    if (m >= 0x7f800000u) hi = sgn | 0x7ff00000u | ((m >> 3) & 0xfffffu);  // infinity, NaN
    if (m < 0x00800000u) {  // zero, subnormal
        hi = sgn;
        lo = 0u;
    }
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}

FT_HD float narrow_d(double d)
{
#ifdef __CUDA_ARCH__
    const uint64_t u = (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
#endif
    const uint32_t sgn = (uint32_t)(u >> 32) & 0x80000000u;
    const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
    uint64_t v = u & 0x7fffffffffffffffull;
    v += 0x0fffffffull + ((v >> 29) & 1u);
    uint32_t r = (uint32_t)(v >> 29) - (896u << 23);  // low word of the rebiased exponent and mantissa
    if (e > 1150u) r = 0x7f800000u;                  // overflow, infinity, NaN
    if (e <= 896u) r = 0u;                           // subnormal or zero in FP32
#ifdef __CUDA_ARCH__
    return __uint_as_float(sgn | r);
#else
    const uint32_t b = sgn | r;
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

}  // namespace ft

#undef FT_HD
