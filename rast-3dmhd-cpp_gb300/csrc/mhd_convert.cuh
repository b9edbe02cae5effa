// mhd_convert.cuh -- float <-> double conversions on the integer pipe.
//
// GB300 executes FP64<->FP32 conversions on its FP64 pipe (2 per clock per
// SM, measured), the same scarce pipe the FP64 arithmetic needs.  These
// helpers build the converted bit patterns with integer operations instead;
// they return exactly what the hardware conversions return (widening is
// exact; narrowing rounds to nearest, ties to even, with subnormal results,
// overflow to infinity and NaN kept as NaN), which mhd_selftest_convert
// checks on the GPU against cvt.f64.f32 / cvt.rn.f32.f64.
#pragma once

#include <cuda_runtime.h>

namespace mhd {

// (double)f, exactly
__device__ __forceinline__ double widen_f32(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    const unsigned e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    unsigned long long r;
    if (e != 0u && e != 255u) {
        r = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (e == 255u) {
        r = sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29);
    } else if (m == 0u) {
        r = sign;
    } else {  // subnormal float: m * 2^-149, normal as a double
        const int p = 31 - __clz((int)m);  // leading one of m, 0..22
        r = sign | ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xfffffffffffffull);
    }
    return __longlong_as_double((long long)r);
}

// (float)d, rounded to nearest even
__device__ __forceinline__ float narrow_f64(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ffu);
    const unsigned long long m = b & 0xfffffffffffffull;
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x00400000u : 0u));
    const int fe = e - 1023 + 127;
    if (fe >= 255) return __uint_as_float(sign | 0x7f800000u);
    if (fe >= 1) {
        const unsigned q = (unsigned)(m >> 29);
        const unsigned rem = (unsigned)(m & 0x1fffffffull);
        const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (q & 1u))) ? 1u : 0u;
        // a carry out of the significand moves to the exponent (up to infinity)
        return __uint_as_float(sign | ((((unsigned)fe << 23) | q) + up));
    }
    // subnormal or zero float result: (1.m) * 2^(e-1023) = M * 2^(-149) / 2^sh
    if (e == 0) return __uint_as_float(sign);  // |d| < 2^-1022
    const unsigned long long M = m | (1ull << 52);
    const int sh = 29 + (1 - fe);  // right shift of M that leaves the subnormal significand
    if (sh > 54) return __uint_as_float(sign);  // below half the smallest subnormal
    const unsigned q = (unsigned)(M >> sh);
    const unsigned long long rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    const unsigned up = (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | (q + up));
}

}  // namespace mhd
