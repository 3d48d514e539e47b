"""The integer-only FP32 conversion the FP32 draws use (phygas_gb300/csrc/cuda/pgx_bits.cuh) gives the bits of the
compiler's own int64 -> float conversion, checked on the CPU: the header also compiles as host C++."""
import os
import subprocess
import tempfile

from tests import oracle_tools as ot

PROBE = r"""
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include "pgx_bits.cuh"
static uint64_t sm = 12345;
static uint64_t next() {                       // splitmix64
    uint64_t z = (sm += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static long bad = 0, tested = 0;
static void check(uint64_t k, int sh) {
    const float want = (float)(int64_t)k * (sh == 53 ? 1.1102230246251565e-16f : 2.220446049250313e-16f);
    const float got = pgx::u64_to_f32_scaled(k, sh);
    uint32_t a, b;
    std::memcpy(&a, &want, 4);
    std::memcpy(&b, &got, 4);
    tested++;
    if (a != b && bad++ < 5) std::printf("k=%llu sh=%d want %a got %a\n", (unsigned long long)k, sh, want, got);
}
int main() {
    for (int sh : {52, 53}) {
        check(0, sh);
        for (int e = 0; e < 54; e++) {                 // around every power of two up to 2^53
            const uint64_t p = 1ull << e;
            for (int d = -40; d <= 40; d++)
                if ((int64_t)p + d >= 0 && p + d <= (1ull << 53)) check(p + d, sh);
        }
        for (int s = 1; s < 30; s++)                   // exact ties and their neighbours, even and odd significands
            for (uint64_t q : {0x800000ull, 0x800001ull, 0xABCDEFull, 0xFFFFFEull, 0xFFFFFFull})
                for (int d = -1; d <= 1; d++) check(((q << s) | (1ull << (s - 1))) + d, sh);
        for (long i = 0; i < 4000000; i++) {
            const uint64_t r = next();
            check(r >> 11, sh);                        // uniform 53-bit, as the draws use
            check((r >> 11) >> (r & 63) % 53, sh);      // every magnitude
        }
    }
    std::printf("tested %ld bad %ld\n", tested, bad);
    return bad != 0;
}
"""


def test_u64_to_f32_scaled_matches_the_cast():
    inc = os.path.join(ot.REPO, "phygas_gb300", "csrc", "cuda")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "probe.cpp"), os.path.join(d, "probe")
        open(src, "w").write(PROBE)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe], check=True)
        r = subprocess.run([exe], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stdout
    assert "bad 0" in r.stdout


REFINE = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "pgx_bits.cuh"
static uint64_t sm = 777;
static uint64_t next() {
    uint64_t z = (sm += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double uni() { return (double)(next() >> 11) * 0x1p-53; }
// the FP32 unit's result, anywhere within 2 ulp of the correctly rounded value
static float f32_result(double exact, int ulps) {
    float f = (float)exact;
    for (int i = 0; i < ulps; i++) f = std::nextafter(f, 0.f);
    for (int i = 0; i < -ulps; i++) f = std::nextafter(f, 1e30f);
    return f;
}
static double worst_rs = 0, worst_rc = 0;
static double ulps(double got, long double want) {
    const double w = (double)want;
    const double u = std::nextafter(std::fabs(w), 1e300) - std::fabs(w);
    return (double)(std::fabs((long double)got - want) / u);
}
static void one(double x) {
    const uint32_t hi = pgx::f64_hi(x);
    if (!pgx::seed_ok(hi)) return;
    const float a = pgx::seed_arg(hi);
    for (int k = -2; k <= 2; k++) {
        const double rs = pgx::rsqrt_refine(x, pgx::widen_seed(f32_result(1.0 / std::sqrt((double)a), k)));
        const double rc = pgx::rcp_refine(x, pgx::widen_seed(f32_result(1.0 / (double)a, k)));
        const double e1 = ulps(rs, 1.0L / std::sqrt((long double)x)), e2 = ulps(rc, 1.0L / (long double)x);
        if (e1 > worst_rs) worst_rs = e1;
        if (e2 > worst_rc) worst_rc = e2;
    }
}
int main() {
    for (long i = 0; i < 2000000; i++) {
        one(std::ldexp(1.0 + uni(), (int)(next() % 250) - 125));    // every binade of the valid range
        one(1.0 + 9.0 * uni());                                     // 1 + p of the halo
        one(std::exp(std::log(1e-3) + uni() * std::log(1e9)));      // squared radii of the force, kpc^2
    }
    for (int e = -125; e < 125; e++)                                 // binade edges
        for (int d = -3; d <= 3; d++) one(std::nextafter(std::ldexp(1.0, e), d < 0 ? 0.0 : 1e300) * (1.0 + d * 1e-16));
    std::printf("worst rsqrt %.3f ulp, worst rcp %.3f ulp\n", worst_rs, worst_rc);
    return !(worst_rs <= 2.0 && worst_rc <= 2.0);
}
"""


def test_force_reciprocals_within_two_ulp():
    """The FP64 reciprocal square root and reciprocal of the force (pgx_bits.cuh: seed from an FP32 result anywhere
    within 2 ulp, one third-order step) stay within 2 ulp of the exact values (80-bit host arithmetic) over every
    binade of their range, the force's radii and the halo's 1 + p."""
    inc = os.path.join(ot.REPO, "phygas_gb300", "csrc", "cuda")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "refine.cpp"), os.path.join(d, "refine")
        open(src, "w").write(REFINE)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe], check=True)
        r = subprocess.run([exe], stdout=subprocess.PIPE, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout


FMT = r"""
#include <cmath>
#include <cfloat>
#include <initializer_list>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "pgx_fmt.cuh"
static uint64_t sm = 99;
static uint64_t next() {
    uint64_t z = (sm += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static long bad = 0, tested = 0;
static void check(double x, int nd) {
    char want[400], got[400];
    snprintf(want, sizeof want, "%.*f", nd, x);
    const int n = pgx::fmt_fixed(got, x, nd);
    got[n] = 0;
    tested++;
    if (strcmp(want, got) || pgx::fmt_fixed(nullptr, x, nd) != n)
        if (bad++ < 10) printf("x=%a nd=%d want %s got %s\n", x, nd, want, got);
}
static double from_bits(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
int main() {
    for (int nd : {0, 1, 2, 3, 4, 6, 9}) {
        for (double x : {0.0, -0.0, 0.5, 1.5, 2.5, 0.125, 0.375, 0.0625, 1e-4, 5e-5, 9.9995, 99.995, -0.0004,
                         -0.0005, DBL_MAX, -DBL_MAX, DBL_MIN, 4.9e-324, (double)INFINITY, -(double)INFINITY,
                         (double)NAN, -(double)NAN, 9.2e14, 1e20, 1.8446744073709552e19})
            check(x, nd);
        for (int e = -1074; e <= 1023; e++) {          // every binade, and its neighbours
            const double p = ldexp(1.0, e);
            check(p, nd); check(-p, nd); check(nextafter(p, 0.0), nd); check(nextafter(p, 1e300), nd);
        }
        for (int k = 0; k < 20000; k++) {              // exact ties: odd multiples of 2^-j
            const double x = ldexp((double)(2 * (next() % 100000) + 1), -(int)(1 + next() % 20));
            check(x, nd); check(-x, nd);
        }
        for (long i = 0; i < 150000; i++) {
            check(from_bits(next()), nd);              // any bit pattern
            const double u = (double)(next() >> 11) * 0x1p-53;
            check(u * 1000.0, nd);                      // the rows' magnitudes
            check(ldexp(u, (int)(next() % 80) - 40), nd);
            check(std::round(u * 1e6) / 1e4, nd);       // near decimal boundaries
        }
    }
    printf("tested %ld bad %ld\n", tested, bad);
    return bad != 0;
}
"""


def test_fixed_point_text_matches_printf():
    """The row writer's %.Nf (pgx_fmt.cuh, integer arithmetic only, the same code the GPU runs) gives the C
    library's printf text byte for byte: every binade from subnormals to DBL_MAX, exact ties (round half to even),
    negative values that round to zero, infinities and NaNs, random bit patterns and row-sized values."""
    inc = os.path.join(ot.REPO, "phygas_gb300", "csrc", "cuda")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "fmt.cpp"), os.path.join(d, "fmt")
        open(src, "w").write(FMT)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe], check=True)
        r = subprocess.run([exe], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stdout
    assert "bad 0" in r.stdout


TRUNC = r"""
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include "pgx_bits.cuh"
static uint64_t sm = 777;
static uint64_t next() {
    uint64_t z = (sm += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static long bad = 0, tested = 0;
static void check(double x) {
    const float f = pgx::f32_trunc(x);
    const double a = std::fabs(x), g = std::fabs((double)f);
    bool ok;
    if (std::isnan(x)) ok = g == (double)FLT_MAX;
    else if (a < 0x1p-126) ok = f == 0.f && std::signbit(f) == std::signbit(x);
    else if (a >= 0x1p128) ok = g == (double)FLT_MAX && std::signbit(f) == std::signbit(x);
    else ok = g <= a && a < g * (1.0 + 0x1p-23) && std::signbit(f) == std::signbit(x) && std::isnormal(f);
    if (std::isfinite(x) && a >= 0x1p-126 && a < 0x1p128) {     // the truncation itself: the nearest float toward zero
        const float n = (float)x;
        const float t = std::fabs((double)n) > a ? std::nextafter(n, 0.f) : n;
        ok = ok && t == f;
    }
    tested++;
    if (!ok && bad++ < 5) std::printf("x=%a got %a\n", x, (double)f);
}
int main() {
    const double sp[] = {0.0, -0.0, 0x1p-1074, 0x1p-127, 0x1.fffffffffffffp-127, 0x1p-126, 0x1.ffffffp-126,
                         1.0, -1.0, 0x1.fffffep127, 0x1.ffffffp127, 0x1.fffffffffffffp127, 0x1p128, -0x1p128,
                         INFINITY, -INFINITY, NAN, -NAN, DBL_MAX};
    for (double x : sp) check(x);
    for (int e = -130; e <= 130; e++)
        for (int d = -3; d <= 3; d++) {
            const double p = std::ldexp(1.0, e);
            double x = p;
            for (int k = 0; k < (d < 0 ? -d : d); k++) x = std::nextafter(x, d < 0 ? 0.0 : INFINITY);
            check(x);
            check(-x);
        }
    for (long i = 0; i < 4000000; i++) {
        const uint64_t r = next();
        double x;
        std::memcpy(&x, &r, 8);
        check(x);                                       // any bit pattern
        check(std::ldexp((double)(r >> 11), -53 + (int)(r % 40) - 20) * ((r >> 7) & 1 ? -1 : 1));   // kpc-sized
    }
    std::printf("tested %ld bad %ld\n", tested, bad);
    return bad != 0;
}
"""


def test_f32_truncation_bounds():
    """The clone kernel's FP32 pre-test (pgx_orbit.cu) rests on f32_trunc (pgx_bits.cuh): the float nearest x toward
    zero, so |f| <= |x| < |f| (1 + 2^-23) in the normal range, +-0 below it and +-FLT_MAX above it and for NaN."""
    inc = os.path.join(ot.REPO, "phygas_gb300", "csrc", "cuda")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "trunc.cpp"), os.path.join(d, "trunc")
        open(src, "w").write(TRUNC)
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", inc, src, "-o", exe], check=True)
        r = subprocess.run([exe], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stdout
    assert "bad 0" in r.stdout
