// Conversions between IEEE 754 binary64 and binary32 on the integer pipe.
//
// On GB300 the FP64 pipe runs at 1/64 of the FP32 rate and also executes the
// FP32<->FP64 conversion instructions, so a cell kernel that widens or rounds
// a few dozen values per cell spends most of its FP64 issue slots on them.
// These functions compute the same results from the bit patterns with 32-bit
// integer instructions, following the format definitions:
//   * to_f32_rn: round to nearest, ties to even; overflow to infinity, results
//     below the normal range as binary32 subnormals (or zero), infinities kept;
//   * to_f64: exact (every binary32 value is a binary64 value); subnormals
//     normalised, infinities kept;
//   * a NaN keeps its sign and leading payload bits and becomes quiet, as the
//     GPU's conversion instructions do (checked bit for bit on the GPU).
// The header compiles as device code and, with the small shims in its test, as
// host C++ (tests/test_bitconv.py checks both against the hardware casts).
#pragma once

#ifndef BITCONV_FN
#define BITCONV_FN __device__ __forceinline__
#endif

namespace bitconv {

BITCONV_FN float to_f32_rn(double x) {
    const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
    const unsigned int sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned int mhi = hi & 0xfffffu;  // top 20 of the 52 fraction bits
    if (e == 0x7ff)
        return __uint_as_float((mhi | lo) ? (sign | 0x7fc00000u | (mhi << 3) | (lo >> 29)) : (sign | 0x7f800000u));
    const int e32 = e - 896;  // rebias 1023 -> 127
    if (e32 >= 1) {
        if (e32 >= 255) return __uint_as_float(sign | 0x7f800000u);
        // keep 23 fraction bits: 20 from hi, 3 from lo; the 29 bits below decide the rounding
        const unsigned int m23 = (mhi << 3) | (lo >> 29);
        const unsigned int rest = lo & 0x1fffffffu;
        const unsigned int up = (rest > 0x10000000u || (rest == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
        // a carry out of the fraction moves into the exponent (and 254 -> 255 gives infinity)
        return __uint_as_float(sign | ((((unsigned int)e32 << 23) | m23) + up));
    }
    // below the binary32 normal range: the significand 1.f (53 bits) shifted
    // right by 30 - e32 places (>= 30) lands on the 2^-149 grid
    if (e == 0) return __uint_as_float(sign);  // binary64 zeros and subnormals round to zero
    const int sh = 30 - e32;                    // 30 .. 925
    if (sh > 54) return __uint_as_float(sign);  // below a quarter of the smallest subnormal
    const unsigned long long sig = (1ull << 52) | ((unsigned long long)mhi << 32) | lo;
    const unsigned long long q = sig >> sh;
    const unsigned long long rem = sig & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    const unsigned long long up = (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
    return __uint_as_float(sign | (unsigned int)(q + up));  // q + up <= 2^23: at most the smallest normal
}

BITCONV_FN double to_f64(float x) {
    const unsigned int b = __float_as_uint(x);
    const unsigned int sign = b & 0x80000000u;
    unsigned int e = (b >> 23) & 0xffu;
    unsigned int m = b & 0x7fffffu;
    if (e == 0xffu) {
        if (m) m |= 0x400000u;  // quiet
        return __hiloint2double((int)(sign | 0x7ff00000u | (m >> 3)), (int)(m << 29));
    }
    if (e == 0) {
        if (m == 0) return __hiloint2double((int)sign, 0);
        // subnormal: shift the leading one into the implicit position
        const unsigned int lz = (unsigned int)__clz((int)m) - 8u;  // m < 2^23: lz >= 1
        m = (m << lz) & 0x7fffffu;
        e = 1u - lz;  // may wrap below zero: the rebias below adds it back as a signed value
        const unsigned int e64 = (unsigned int)((int)e + 896);
        return __hiloint2double((int)(sign | (e64 << 20) | (m >> 3)), (int)(m << 29));
    }
    return __hiloint2double((int)(sign | ((e + 896u) << 20) | (m >> 3)), (int)(m << 29));
}

}  // namespace bitconv
