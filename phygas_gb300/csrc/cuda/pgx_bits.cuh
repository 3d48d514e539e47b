// pgx_bits.cuh -- integer-to-FP32 conversion done with integer operations (internal header; also compiles as plain
// host C++, so its results can be checked on the CPU against the compiler's own conversion).
//
// A conversion whose source is a 64-bit integer issues, on this GPU, to the FP64 unit, which retires 1/64 of the
// FP32 pipes' rate; the FP32 draws of the finish stage need six of them per draw and were limited by that unit.
// The function below reaches the same bits through the integer pipes.
#pragma once
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

}  // namespace pgx
