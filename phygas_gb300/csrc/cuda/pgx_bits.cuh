// pgx_bits.cuh -- integer-to-FP32 conversion done with integer operations, and the FP64 reciprocal / reciprocal
// square root refinement of the force (internal header; also compiles as plain host C++, so its results can be
// checked on the CPU against the compiler's own conversion and against extended-precision values).
//
// A conversion whose source is a 64-bit integer issues, on this GPU, to the FP64 unit, which retires 1/64 of the
// FP32 pipes' rate; the FP32 draws of the finish stage need six of them per draw and were limited by that unit.
// The function below reaches the same bits through the integer pipes.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PGX_HD __host__ __device__ __forceinline__
#else
#define PGX_HD inline
#endif

namespace pgx {

PGX_HD int clz64_nz(uint64_t k) {       // k != 0
#ifdef __CUDA_ARCH__
    return __clzll((long long)k);
#else
    return __builtin_clzll(k);
#endif
}

// round-to-nearest-even(k) * 2^-sh in FP32, for 0 <= k < 2^63 and 2^-sh * k a normal number (k = 0 gives +0).
// Bit-identical to (float)(int64_t)k * 2^-sh: the significand is the top 24 bits of k rounded by the bits below
// them (ties to even), the exponent is the position of k's leading bit; a rounding carry out of the 24 bits moves
// into the exponent field by itself, because the significand is added to the exponent word with its implicit bit.
PGX_HD float u64_to_f32_scaled(uint64_t k, int sh) {
    if (k == 0) return 0.f;
    const int e = 63 - clz64_nz(k);                 // k in [2^e, 2^(e+1))
    uint32_t m;                                     // significand with its implicit bit, in [2^23, 2^24]
    if (e <= 23) {
        m = (uint32_t)k << (23 - e);
    } else {
        const int s = e - 23;
        const uint64_t q = k >> s, rem = k & ((1ull << s) - 1), half = 1ull << (s - 1);
        m = (uint32_t)q + (uint32_t)(rem > half || (rem == half && (q & 1u)));
    }
    const uint32_t bits = ((uint32_t)(e + 126 - sh) << 23) + m;
#ifdef __CUDA_ARCH__
    return __uint_as_float(bits);
#else
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
#endif
}

// ---- FP64 reciprocal and reciprocal square root from an FP32 seed ---------------------------------------------
// The seed is the FP32 unit's result on a float carrying the argument's exponent and the top 20 bits of its
// significand; integer operations move the values between the formats (on the GPU a conversion instruction would
// issue to the FP64 unit).  With the FP32 result within 2^-22 relative, the widened seed y is within 2^-19.2 of the
// true value (truncations 2^-20 of the argument, halved by the square root, and 2^-20 of the result), so
// e = 1 - x y^2 (an exact product: y has 20 significant bits) or e = 1 - d y is below 2^-18.2 in magnitude, and one
// third-order Householder step,
//   x^-1/2 = y (1 - e)^-1/2 ~ y (1 + e/2 + 3 e^2 / 8),   1/d = y / (1 - e) ~ y (1 + e + e^2),
// leaves a truncation error below 2^-56 (5 e^3 / 16, e^3) before the last rounding: within an ulp or two of the
// correctly rounded value, in 5 and 3 FP64 operations.  Valid for arguments in [2^-125, 2^125) (seed_ok).
constexpr uint32_t kSeedLo = 898u << 20, kSeedSpan = (1148u - 898u) << 20;

PGX_HD uint32_t f64_hi(double x) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2hiint(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return (uint32_t)(b >> 32);
#endif
}

PGX_HD uint32_t f64_lo(double x) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2loint(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return (uint32_t)b;
#endif
}

// x in FP32 with its significand truncated (toward zero), by integer operations: |f| <= |x| < |f| (1 + 2^-23) for
// 2^-126 <= |x| < 2^128; +-0 below that range and +-FLT_MAX above it (NaN included)
PGX_HD float f32_trunc(double x) {
    const uint32_t hi = f64_hi(x), lo = f64_lo(x);
    const uint32_t e = (hi >> 20) & 0x7ffu, sign = hi & 0x80000000u;
    uint32_t b;
    if (e < 897u) b = sign;
    else if (e > 1150u) b = sign | 0x7f7fffffu;
    else b = sign | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, 4);
    return f;
#endif
}

PGX_HD bool seed_ok(uint32_t hi) { return hi - kSeedLo < kSeedSpan; }

// the float with the argument's exponent and top 20 significand bits (seed_ok(hi) holds)
PGX_HD float seed_arg(uint32_t hi) {
    const uint32_t b = (hi - (896u << 20)) << 3;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, 4);
    return f;
#endif
}

// an FP32 result widened to FP64, keeping the top 20 bits of its significand
PGX_HD double widen_seed(float y) {
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)((__float_as_uint(y) >> 3) + (896u << 20)), 0);
#else
    uint32_t b;
    std::memcpy(&b, &y, 4);
    const uint64_t d = (uint64_t)((b >> 3) + (896u << 20)) << 32;
    double r;
    std::memcpy(&r, &d, 8);
    return r;
#endif
}

PGX_HD double rsqrt_refine(double x, double y) {
    const double e = fma(-x, y * y, 1.0);
    return fma(y, e * fma(e, 0.375, 0.5), y);
}

PGX_HD double rcp_refine(double d, double y) {
    const double e = fma(-d, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

}  // namespace pgx
