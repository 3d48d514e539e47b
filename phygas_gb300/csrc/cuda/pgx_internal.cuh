// pgx_internal.cuh -- device-side building blocks shared by the kernels of libphygas_gb300 (internal header).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pgx {

// ---- Allen & Santillan (1991) parameters, in kpc / Myr / kpc^3 Myr^-2 (reference src/potential.c:34-45) --------
constexpr double kKms = 977.7922216807892;                      // km/s per kpc/Myr (reference src/units.h:14)
constexpr double kG = 4.30091e-6 / (kKms * kKms);
constexpr double kBulgeGM = kG * (606.0 * 2.325e7);
constexpr double kBulgeB2 = 0.3873 * 0.3873;
constexpr double kDiskGM = kG * (3690.0 * 2.325e7);
constexpr double kDiskA = 5.3178;
constexpr double kDiskB2 = 0.25 * 0.25;
constexpr double kHaloGM = kG * (4615.0 * 2.325e7);
constexpr double kHaloInvA = 1.0 / 12.0;
constexpr double kHaloCut = 100.0;
constexpr double kHaloG1 = 2.02 - 1.0;                          // gamma - 1, as the reference forms it
constexpr double kStepMyr = 0.5;                                // PH_PRE_STEP_MYR
constexpr int kSub = 10;                                        // PH_LIN_SUB
constexpr double kEps = 1e-5;                                   // PH_LIN_EPS_POS == PH_LIN_EPS_VEL

// Acceleration of the Milky Way model at (x, y, z), FP64.
//
// Same model as the reference's milkyway_accel (src/potential.c:60-101), written for a GPU whose FP64 pipe is the
// scarce resource: the three pow() and the divisions become reciprocal square roots and one log/exp pair, using
//   (r^2+b^2)^-3/2 = rsqrt(r^2+b^2)^3          (bulge)
//   aR * x / R     = -GM x / D^3                 (disk, the R of the radial force cancels)
//   x^g / (1 + x^(g-1)) = x p / (1 + p), p = x^(g-1) = exp((g-1) ln x)   (halo)
// Mathematically identical; the last bits differ from glibc's as any libm's do.
__device__ __forceinline__ void mw_accel(double x, double y, double z, double &ax, double &ay, double &az) {
    const double R2 = fma(x, x, y * y);
    const double r2 = fma(z, z, R2);
    const double ib = rsqrt(r2 + kBulgeB2);
    const double fb = -kBulgeGM * (ib * ib * ib);
    const double zb2 = fma(z, z, kDiskB2);
    const double iz = rsqrt(zb2);
    const double s = fma(zb2, iz, kDiskA);                      // a + sqrt(z^2 + b^2)
    const double iD = rsqrt(fma(s, s, R2));
    const double fd = -kDiskGM * (iD * iD * iD);
    double ir = rsqrt(r2);
    double r = r2 * ir;
    if (!(r > 1e-12)) { r = 1e-12; ir = 1e12; }
    const double xh = fmin(r, kHaloCut) * kHaloInvA;
    const double p = exp(kHaloG1 * log(xh));
    const double fh = -(kHaloGM * xh * p / (1.0 + p)) * (ir * ir * ir);
    const double fr = fb + fh;
    ax = (fr + fd) * x;
    ay = (fr + fd) * y;
    az = fma(fr, z, fd * z * s * iz);
}

// One orbit: position, velocity and the acceleration carried over (one force evaluation per step).
struct Orbit {
    double x, y, z, vx, vy, vz, ax, ay, az;
    __device__ __forceinline__ void init() { mw_accel(x, y, z, ax, ay, az); }
    // kick-drift-kick leapfrog (reference body_step, src/phygas.c:91-96)
    __device__ __forceinline__ void kdk(double dt, double h) {
        vx = fma(ax, h, vx); vy = fma(ay, h, vy); vz = fma(az, h, vz);
        x = fma(vx, dt, x); y = fma(vy, dt, y); z = fma(vz, dt, z);
        mw_accel(x, y, z, ax, ay, az);
        vx = fma(ax, h, vx); vy = fma(ay, h, vy); vz = fma(az, h, vz);
    }
};

// A lower bound on the smallest eigenvalue of a symmetric positive semi-definite 3x3 matrix (xx xy xz yy yz zz),
// FP64, by the trigonometric solution of the characteristic cubic (Smith, Comm. ACM 4, 168, 1961).  The margin covers
// the rounding of q + 2p cos(phi + 2 pi/3) (a few ulps of the trace) and the sensitivity of acos near r = 1 (the
// eigenvalue moves by <= 1.8 p dphi, dphi <= sqrt(2 dr) / 3 with dr ~ 1e-15).
// The bound is not clamped at zero: a matrix rounded to slightly indefinite keeps a valid (negative) bound.
__device__ __forceinline__ double sym3_min_eig_lb(double a, double b, double c, double d, double e, double f) {
    const double p1 = b * b + c * c + e * e;
    const double tiny = 4.0 * 1.1102230246251565e-16 * (fabs(a) + fabs(d) + fabs(f));
    if (p1 == 0.0) return fmin(a, fmin(d, f)) - tiny;
    const double q = (a + d + f) * (1.0 / 3.0);
    const double A = a - q, D = d - q, F = f - q;
    const double p = sqrt((A * A + D * D + F * F + 2.0 * p1) * (1.0 / 6.0));
    if (!(p > 0.0)) return q - tiny;
    const double ip = 1.0 / p;
    const double detB = (A * (D * F - e * e) - b * (b * F - e * c) + c * (b * e - D * c)) * (ip * ip * ip);
    const double r = fmin(fmax(0.5 * detB, -1.0), 1.0);
    const double phi = acos(r) * (1.0 / 3.0);
    const double lmin = q + 2.0 * p * cos(phi + 2.0943951023931957);
    const double margin = 4e-8 * p + 32.0 * 1.1102230246251565e-16 * (fabs(q) + 2.0 * p);
    return lmin - margin;
}

// splitmix64 output for call n (n >= 1) of a generator seeded with `seed`: its state is a Weyl sequence,
// state_n = seed + n * golden, so any draw of a pair's stream is reachable without the ones before it.
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ULL;
__device__ __forceinline__ uint64_t splitmix_mix(uint64_t z) {      // output for state z
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t splitmix_at(uint64_t seed, uint64_t n) { return splitmix_mix(seed + n * kGolden); }

}  // namespace pgx
