// Host check of hydro_rs_gb300/csrc/bitconv.cuh against the C++ casts (IEEE
// round to nearest even on every host this builds on).  Built and run by
// tests/test_bitconv.py.  NaN results are compared as "both NaN".
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

static inline int __double2hiint(double x) { uint64_t b; std::memcpy(&b, &x, 8); return (int)(uint32_t)(b >> 32); }
static inline int __double2loint(double x) { uint64_t b; std::memcpy(&b, &x, 8); return (int)(uint32_t)b; }
static inline float __uint_as_float(unsigned int u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline unsigned int __float_as_uint(float f) { unsigned int u; std::memcpy(&u, &f, 4); return u; }
static inline double __hiloint2double(int hi, int lo) {
    uint64_t b = ((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}
static inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((unsigned)x); }
#define BITCONV_FN static inline
#include "../hydro_rs_gb300/csrc/bitconv.cuh"

static uint64_t s = 0x9e3779b97f4a7c15ull;
static inline uint64_t rnd() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
}
static long bad = 0, n = 0;
static void check_d(uint64_t bits) {
    double x;
    std::memcpy(&x, &bits, 8);
    const float want = (float)x, got = bitconv::to_f32_rn(x);
    n++;
    if (std::isnan(want) ? !std::isnan(got) : __float_as_uint(want) != __float_as_uint(got)) {
        if (bad++ < 10) std::printf("to_f32_rn(%016llx) = %08x, want %08x\n", (unsigned long long)bits,
                                    __float_as_uint(got), __float_as_uint(want));
    }
}
static void check_f(uint32_t bits) {
    const float x = __uint_as_float(bits);
    const double want = (double)x, got = bitconv::to_f64(x);
    uint64_t a, b;
    std::memcpy(&a, &want, 8);
    std::memcpy(&b, &got, 8);
    n++;
    if (std::isnan(want) ? !std::isnan(got) : a != b) {
        if (bad++ < 10) std::printf("to_f64(%08x) = %016llx, want %016llx\n", bits, (unsigned long long)b,
                                    (unsigned long long)a);
    }
}

int main() {
    const uint64_t special[] = {0, 1ull << 63, 0x7ff0000000000000ull, 0xfff0000000000000ull, 0x7ff8000000000000ull,
                                0x7ff0000000000001ull, 0xfff8000000000001ull, 1, 0x000fffffffffffffull,
                                0x47efffffe0000000ull /* max float + half ulp */, 0x47efffffdfffffffull,
                                0x47efffffffffffffull, 0x3690000000000000ull /* 2^-150 */, 0x3690000000000001ull,
                                0x36a0000000000000ull /* 2^-149 */, 0x380fffffffffffffull, 0x3810000000000000ull};
    for (uint64_t b : special) check_d(b);
    for (int i = 0; i < 20000000; i++) check_d(rnd());
    // exponents around the binary32 range, random fractions, halfway patterns
    for (int i = 0; i < 20000000; i++) {
        uint64_t e = 850 + rnd() % 300;  // 2^-173 .. 2^126
        uint64_t f = rnd() & 0xfffffffffffffull;
        if (i & 1) f = (f & ~0x1fffffffull) | 0x10000000ull;  // exactly half an ulp of a normal result
        if ((i & 3) == 2) f = f & ~((1ull << (rnd() % 53)) - 1ull);
        check_d(((rnd() & 1) << 63) | (e << 52) | f);
    }
    // ties at subnormal results
    for (int sh = 30; sh <= 54; sh++)
        for (int k = 0; k < 4000; k++) {
            uint64_t e = 896 - (sh - 30);
            uint64_t f = rnd() & 0xfffffffffffffull;
            f &= ~((1ull << sh) - 1ull);           // clear everything below the result's last bit
            if (k & 1) f |= 1ull << (sh - 1);      // and make it exactly half an ulp
            check_d((e << 52) | f);
        }
    for (uint32_t b = 0; b < (1u << 23); b++) {  // every subnormal, both signs
        check_f(b);
        check_f(b | 0x80000000u);
    }
    for (int i = 0; i < 30000000; i++) check_f((uint32_t)rnd());
    const uint32_t fs[] = {0x7f800000u, 0xff800000u, 0x7fc00000u, 0x7f800001u, 0xffffffffu, 0x00800000u, 0x7f7fffffu};
    for (uint32_t b : fs) check_f(b);
    std::printf("checked %ld conversions, %ld mismatches\n", n, bad);
    return bad != 0;
}
