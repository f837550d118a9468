// hc_f32split.h -- FP64 -> FP32 rounding and hi + lo splits with integer
// operations.
//
// GB300's FP64 pipe runs at a small fraction of its FP32 rate, and the
// conversion of a double to a float is an FP64-pipe instruction.  The tree
// build converts every body and every cell (node records: FP32 mass and the
// position as hi + lo floats), so it does the rounding on the double's bits:
//
//   hi = RN_f32(x): the 52-bit significand keeps its top 23 bits, rounded to
//        nearest, ties to even, on the 29 dropped bits (a carry out of the
//        significand moves into the exponent, which is the correctly rounded
//        value);
//   lo = RN_f32(x - hi): x - hi is the dropped part (rounded down) or minus
//        its complement (rounded up), an integer R < 2^29 times the double's
//        unit in the last place, so RN_f32(x - hi) = +-RN_f32(R) * ulp, one
//        integer-to-float conversion and an exact power-of-two scaling.
//
// Both are the IEEE results for doubles whose float result is normal; the
// rest (zeros, magnitudes below 2^-74 or at or above 2^126, infinities, NaN)
// take the FP64 conversions.  The file compiles as CUDA and as plain C++, so
// that a host program can check it against the host's IEEE conversions.
#pragma once
#include <stdint.h>
#include <string.h>
#include <stdbool.h>

#if defined(__CUDACC__)
#define HC_HD __host__ __device__ __forceinline__
#else
#define HC_HD static inline
#endif

HC_HD uint64_t hc_dbits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

HC_HD float hc_fbits(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
#endif
}

HC_HD uint32_t hc_f2bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof u);
    return u;
#endif
}

HC_HD float hc_u2f_rn(uint32_t r)
{
#if defined(__CUDA_ARCH__)
    return __uint2float_rn(r);
#else
    return (float)r;   // IEEE round to nearest even
#endif
}

HC_HD float hc_d2f_fp64(double x)
{
#if defined(__CUDA_ARCH__)
    return __double2float_rn(x);
#else
    return (float)x;
#endif
}

// biased double exponent range of the integer path: 2^-74 <= |x| < 2^126
#define HC_SPLIT_EMIN 949
#define HC_SPLIT_EMAX 1148

// RN_f32(x)
HC_HD float hc_d2f_rn(double x)
{
    const uint64_t b = hc_dbits(x);
    const int ef = (int)((b >> 52) & 0x7ff);
    if (ef < HC_SPLIT_EMIN || ef > HC_SPLIT_EMAX) return hc_d2f_fp64(x);
    const uint32_t m = (uint32_t)(b >> 29) & 0x7fffffu, rem = (uint32_t)b & 0x1fffffffu;
    uint32_t f = ((uint32_t)(b >> 32) & 0x80000000u) | ((uint32_t)(ef - 896) << 23) | m;
    f += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return hc_fbits(f);
}

// hi = RN_f32(x), lo = RN_f32(x - (double)hi)
HC_HD void hc_split_hilo(double x, float *hi, float *lo)
{
    const uint64_t b = hc_dbits(x);
    const int ef = (int)((b >> 52) & 0x7ff);
    if (ef < HC_SPLIT_EMIN || ef > HC_SPLIT_EMAX) {
        const float h = hc_d2f_fp64(x);
        *hi = h;
        *lo = hc_d2f_fp64(x - (double)h);
        return;
    }
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t m = (uint32_t)(b >> 29) & 0x7fffffu, rem = (uint32_t)b & 0x1fffffffu;
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (m & 1u));
    *hi = hc_fbits((sign | ((uint32_t)(ef - 896) << 23) | m) + (up ? 1u : 0u));
    // x - hi = +-R * 2^(ef - 1075): the sign of x when rounded down, the
    // opposite when rounded up; R = 0 gives +0 (x - x in round to nearest)
    const uint32_t R = up ? 0x20000000u - rem : rem;
    if (R == 0) {
        *lo = 0.0f;
        return;
    }
    const float scale = hc_fbits((uint32_t)(ef - 948) << 23);   // 2^(ef - 1075), a normal float
    const float r = hc_u2f_rn(R) * scale;                       // exact: power-of-two scaling
    *lo = hc_fbits(hc_f2bits(r) | (up ? sign ^ 0x80000000u : sign));
}
