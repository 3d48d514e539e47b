// pgx_fmt.cuh -- printf("%.Nf") for doubles, exact, with integer arithmetic only (internal header; also compiles as
// plain host C++, so the CPU can check it against the C library's printf).
//
// x = m 2^e exactly (m the 53-bit significand as an integer).  x 10^N = m 10^N 2^e: with P = m 10^N (< 2^67, held in
// two 64-bit words) the value is P 2^e; for e < 0 it is rounded to an integer q = round(P / 2^-e), the tie going to
// the even q (the C library's round-to-nearest on the exact binary value), and for e >= 0 it is the integer P 2^e.
// The text is q's decimal digits with a point before the last N: the C library's result byte for byte, including
// "-0.000" for a negative value that rounds to zero and "nan" / "-nan" / "inf" / "-inf".
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PGX_FMT __host__ __device__ __forceinline__
#else
#define PGX_FMT inline
#endif

namespace pgx {

constexpr int kFmtMaxNumber = 330;      // the longest "%.4f" of a double: sign, 309 integer digits, point, 4 decimals

PGX_FMT uint64_t fmt_mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// decimal digits of a little-endian array of 32-bit limbs (destroyed), least significant first into rev; returns
// the count (at least one digit)
PGX_FMT int fmt_big_digits(uint32_t *limb, int nl, char *rev) {
    int nd = 0;
    while (nl > 0 && limb[nl - 1] == 0) nl--;
    while (nl > 0) {
        uint64_t r = 0;
        for (int i = nl - 1; i >= 0; i--) {                  // divide by 10^9
            const uint64_t cur = (r << 32) | limb[i];
            limb[i] = (uint32_t)(cur / 1000000000u);
            r = cur % 1000000000u;
        }
        while (nl > 0 && limb[nl - 1] == 0) nl--;
        for (int j = 0; j < 9; j++) {
            rev[nd++] = (char)('0' + r % 10);
            r /= 10;
            if (nl == 0 && r == 0) break;                     // no leading zeros in the top group
        }
    }
    if (nd == 0) rev[nd++] = '0';
    return nd;
}

// printf("%.<nd>f", x) into o (room for kFmtMaxNumber bytes, or nullptr to count only); returns the length.
// nd in 0..9.
PGX_FMT int fmt_fixed(char *o, double x, int nd) {
    uint64_t b;
    memcpy(&b, &x, 8);
    const bool neg = (b >> 63) != 0;
    const int ex = (int)((b >> 52) & 0x7ff);
    uint64_t m = b & 0xfffffffffffffull;
    int len = 0;
    auto put = [&](char c) {
        if (o) o[len] = c;
        len++;
    };
    if (neg) put('-');
    if (ex == 0x7ff) {
        const char *s = m ? "nan" : "inf";
        for (int i = 0; i < 3; i++) put(s[i]);
        return len;
    }
    int e;
    if (ex == 0) {
        e = -1074;
    } else {
        m |= 1ull << 52;
        e = ex - 1075;
    }
    uint64_t p10 = 1;
    for (int i = 0; i < nd; i++) p10 *= 10;
    // P = m p10 as (hi, lo)
    const uint64_t lo = m * p10, hi = fmt_mulhi(m, p10);
    char rev[kFmtMaxNumber];
    int n = 0;
    if (e < 0) {
        const int s = -e;
        uint64_t qh = 0, ql = 0;
        if (s < 128) {
            // q = P >> s, rem = P mod 2^s, compared with half = 2^(s-1)
            uint64_t rh, rl, hh, hl;
            if (s >= 64) {
                ql = s == 64 ? hi : (s < 128 ? hi >> (s - 64) : 0);
                qh = 0;
                rl = lo;
                rh = s == 64 ? 0 : hi & ((1ull << (s - 64)) - 1);
                hh = s == 64 ? 0 : 1ull << (s - 65);
                hl = s == 64 ? 1ull << 63 : 0;
            } else {
                ql = (lo >> s) | (hi << (64 - s));
                qh = hi >> s;
                rl = lo & ((1ull << s) - 1);
                rh = 0;
                hl = 1ull << (s - 1);
                hh = 0;
            }
            const bool above = rh > hh || (rh == hh && rl > hl), tie = rh == hh && rl == hl;
            if (above || (tie && (ql & 1))) {
                ql++;
                if (ql == 0) qh++;
            }
        }
        if (qh == 0) {
            uint64_t q = ql;
            do {
                rev[n++] = (char)('0' + q % 10);
                q /= 10;
            } while (q);
        } else {
            uint32_t limb[4] = {(uint32_t)ql, (uint32_t)(ql >> 32), (uint32_t)qh, (uint32_t)(qh >> 32)};
            n = fmt_big_digits(limb, 4, rev);
        }
    } else {
        // the integer P 2^e, up to 67 + 971 bits
        uint32_t limb[34] = {};
        const int w = e >> 5, sh = e & 31;
        const uint32_t v[3] = {(uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi};
        for (int i = 0; i < 3; i++) {
            const uint64_t t = (uint64_t)v[i] << sh;
            limb[w + i] |= (uint32_t)t;
            limb[w + i + 1] |= (uint32_t)(t >> 32);
        }
        n = fmt_big_digits(limb, 34, rev);
    }
    while (n < nd + 1) rev[n++] = '0';                     // at least one integer digit
    for (int i = n - 1; i >= nd; i--) put(rev[i]);
    if (nd > 0) {
        put('.');
        for (int i = nd - 1; i >= 0; i--) put(rev[i]);
    }
    return len;
}

// a NUL-terminated string of at most cap bytes
PGX_FMT int fmt_str(char *o, const char *s, int cap) {
    int len = 0;
    while (len < cap && s[len]) {
        if (o) o[len] = s[len];
        len++;
    }
    return len;
}

}  // namespace pgx
