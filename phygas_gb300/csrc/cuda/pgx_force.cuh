// pgx_force.cuh -- the Allen & Santillan (1991) Milky Way force and the kick-drift-kick step, FP64 (internal header
// of pgx_orbit.cu, which owns the halo power tables and fills them once per device).
#pragma once
#include "pgx_bits.cuh"
#include "pgx_internal.cuh"

namespace pgx {

// x^(gamma - 1) of the halo term as x * x^a, a = (gamma - 1) - 1 = 0.02: x = 2^e m, m in [1, 2); m in sub-interval
// j of 1024 with centre c_j, m = c_j (1 + t), |t| <= 2^-11; x^a = 2^(a e) c_j^a (1 + t)^a with the first two from
// tables and (1 + t)^a by its binomial series to t^4 (the next term, |C(a, 5)| t^5 <= 0.0039 2^-55, is below 2^-63
// relative).  Eight FP64 operations and a few integer ones, in place of a log and an exp (about 50 FP64-pipe slots
// on this GPU), and closer: each table entry and the series are within a few ulp, where exp(a' ln x) inherits the
// log's absolute error times |a' ln x|.
constexpr int kPow2Bias = 80, kPow2N = 96, kPowSubLog = 10, kPowSub = 1 << kPowSubLog, kPowTerms = 4;
static __device__ double g_halo_pow2[kPow2N];      // 2^(a e), e = i - kPow2Bias
static __device__ double g_halo_powc[kPowSub];     // c_j^a, c_j = 1 + (2 j + 1) / 2048
static __device__ double g_halo_invc[kPowSub];     // 1 / c_j
static __device__ double g_halo_coef[kPowTerms + 1];   // binomial coefficients C(a, n)

// the tables (one thread per entry; launched once per device, before any kernel that integrates an orbit)
__global__ void k_halo_tables() {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double a = kHaloG1 - 1.0;
    if (i < kPow2N) g_halo_pow2[i] = exp2(a * (double)(i - kPow2Bias));
    if (i < kPowSub) {
        const double c = 1.0 + (double)(2 * i + 1) / (2.0 * kPowSub);
        g_halo_powc[i] = pow(c, a);
        g_halo_invc[i] = 1.0 / c;
    }
    if (i == 0) {
        double c = 1.0;
        for (int n = 0; n <= kPowTerms; n++) {
            g_halo_coef[n] = c;
            c = c * (a - (double)n) / (double)(n + 1);
        }
    }
}
constexpr int kHaloTableThreads = kPowSub > kPow2N ? kPowSub : kPow2N;

// x^a for x > 0 normal (here x in [8e-14, 8.4])
__device__ __forceinline__ double halo_pow_a(double x) {
    const long long bits = __double_as_longlong(x);
    int e = (int)((bits >> 52) & 0x7ff) - 1023;
    e = e < -kPow2Bias ? -kPow2Bias : (e > kPow2N - 1 - kPow2Bias ? kPow2N - 1 - kPow2Bias : e);
    const int j = (int)((bits >> (52 - kPowSubLog)) & (kPowSub - 1));
    const double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    const double t = fma(m, __ldg(&g_halo_invc[j]), -1.0);
    double s = __ldg(&g_halo_coef[kPowTerms]);
#pragma unroll
    for (int n = kPowTerms - 1; n >= 0; n--) s = fma(s, t, __ldg(&g_halo_coef[n]));
    return __ldg(&g_halo_pow2[e + kPow2Bias]) * __ldg(&g_halo_powc[j]) * s;
}

// x^-1/2 and 1/d in FP64 from the FP32 unit's seed and one third-order step (pgx_bits.cuh: within an ulp or two,
// 5 and 3 FP64 operations); an argument outside [2^-125, 2^125) -- none in a force evaluation of a bound orbit --
// takes the library's function instead.
__device__ __forceinline__ double rsqrt_h3(double x) {
    const uint32_t hi = f64_hi(x);
    if (!seed_ok(hi)) return rsqrt(x);
    return rsqrt_refine(x, widen_seed(rsqrtf(seed_arg(hi))));
}
__device__ __forceinline__ double rcp_h3(double d) {
    const uint32_t hi = f64_hi(d);
    if (!seed_ok(hi)) return 1.0 / d;
    return rcp_refine(d, widen_seed(__frcp_rn(seed_arg(hi))));
}

// Acceleration of the Milky Way model at (x, y, z), FP64.
//
// Same model as the reference's milkyway_accel (src/potential.c:60-101), written for a GPU whose FP64 pipe is the
// scarce resource: the three pow() and the divisions become the reciprocal square roots and reciprocal above and the
// table power, using
//   (r^2+b^2)^-3/2 = rsqrt(r^2+b^2)^3          (bulge)
//   aR * x / R     = -GM x / D^3                 (disk, the R of the radial force cancels)
//   az(disk)       = -GM z (a + s) / (s D^3), s = sqrt(z^2 + b^2): (a + s) / s = 1 + a / s
//   x^g / (1 + x^(g-1)) = x p / (1 + p), p = x^(g-1) = x * x^(g-2)   (halo)
// Mathematically identical; the last bits differ from glibc's as any libm's do.  59 FP64 operations.
__device__ __forceinline__ void mw_accel(double x, double y, double z, double &ax, double &ay, double &az) {
    const double R2 = fma(x, x, y * y);
    const double r2 = fma(z, z, R2);
    const double ib = rsqrt_h3(r2 + kBulgeB2);
    const double zb2 = fma(z, z, kDiskB2);
    const double iz = rsqrt_h3(zb2);
    const double s = fma(zb2, iz, kDiskA);                      // a + sqrt(z^2 + b^2)
    const double iD = rsqrt_h3(fma(s, s, R2));
    const double fd = -kDiskGM * (iD * iD * iD);
    // r2 > kTinyR2 and min(r, cut) as integer compares of the bit patterns (for doubles >= 0 they order as the values
    // do; a compare or min of doubles would take an FP64-pipe slot): the same selections for every r2 >= 0
    double r, ir;
    if (__double_as_longlong(r2) > kTinyR2Bits) {
        ir = rsqrt_h3(r2);
        r = r2 * ir;
    } else {
        r = 1e-12;
        ir = 1e12;
    }
    const double xh = (__double_as_longlong(r) < kHaloCutBits ? r : kHaloCut) * kHaloInvA;
    const double p = xh * halo_pow_a(xh);              // xh^(gamma - 1)
    const double q = p * rcp_h3(1.0 + p);
    const double fh = -kHaloGM * xh * q * ((ir * ir) * ir);
    const double fr = fma(-kBulgeGM * ib, ib * ib, fh);       // bulge + halo radial terms
    const double g = fr + fd;
    ax = g * x;
    ay = g * y;
    az = z * fma(fd * kDiskA, iz, g);
}

// One orbit: position, velocity and the acceleration carried over (one force evaluation per step).
struct Orbit {
    double x, y, z, vx, vy, vz, ax, ay, az;
    __device__ __forceinline__ void init() { mw_accel(x, y, z, ax, ay, az); }
    // kick-drift-kick leapfrog (reference body_step, src/phygas.c:91-96).  Two half kicks per step, as the reference
    // rounds them: merging a step's closing kick with the next one's opening kick would save three FP64 operations
    // but moves the last bits of the orbits enough to change printed digits of the reference's published rows.
    __device__ __forceinline__ void kdk(double dt, double h) {
        vx = fma(ax, h, vx); vy = fma(ay, h, vy); vz = fma(az, h, vz);
        x = fma(vx, dt, x); y = fma(vy, dt, y); z = fma(vz, dt, z);
        mw_accel(x, y, z, ax, ay, az);
        vx = fma(ax, h, vx); vy = fma(ay, h, vy); vz = fma(az, h, vz);
    }
};

}  // namespace pgx
