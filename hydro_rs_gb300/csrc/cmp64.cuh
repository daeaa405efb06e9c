// IEEE comparisons of doubles evaluated on the integer pipe.
//
// On GB300 FP64 instructions issue at 1/64 of the FP32 rate, comparisons
// (DSETP) included, and the exact solver's searches spend about a quarter of
// their FP64 issue on them.  These helpers give the same truth values as the
// floating-point comparisons, for every pair of doubles: NaN is unordered
// (every ordered comparison false, != true), -0.0 equals +0.0, the infinities
// order as values.  They work on the bit patterns: a double's order key is its
// bit pattern read as a signed integer where it is non-negative and the
// negated magnitude where it is negative (so both zeros map to 0).
//
// Compiled for the device by nvcc and for the host by any C++ compiler (the
// unit test compares them with the hardware comparisons on special and random
// values).
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define CMP64_FN __host__ __device__ __forceinline__
#else
#define CMP64_FN inline
#endif

namespace cmp64 {

CMP64_FN int64_t bits(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    int64_t b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}
constexpr int64_t kMag = 0x7fffffffffffffffLL;
constexpr int64_t kInf = 0x7ff0000000000000LL;
CMP64_FN bool nan(double x) { return (bits(x) & kMag) > kInf; }
CMP64_FN int64_t key(double x) {
    const int64_t b = bits(x);
    return b >= 0 ? b : -(b & kMag);
}
// a < b, a <= b, a > b, a >= b, a == b, a != b
CMP64_FN bool lt(double a, double b) { return !nan(a) && !nan(b) && key(a) < key(b); }
CMP64_FN bool le(double a, double b) { return !nan(a) && !nan(b) && key(a) <= key(b); }
CMP64_FN bool gt(double a, double b) { return lt(b, a); }
CMP64_FN bool ge(double a, double b) { return le(b, a); }
CMP64_FN bool eq(double a, double b) { return !nan(a) && !nan(b) && key(a) == key(b); }
CMP64_FN bool ne(double a, double b) { return !eq(a, b); }
// fabs(a) < fabs(b), fabs(a) >= fabs(b): magnitudes order as unsigned integers
CMP64_FN bool abs_lt(double a, double b) { return !nan(a) && !nan(b) && (bits(a) & kMag) < (bits(b) & kMag); }
CMP64_FN bool abs_ge(double a, double b) { return !nan(a) && !nan(b) && (bits(a) & kMag) >= (bits(b) & kMag); }

}  // namespace cmp64
