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
constexpr long long kHaloCutBits = 0x4059000000000000LL;       // the bit pattern of kHaloCut (checked in orbit_setup)
constexpr double kTinyR2 = 1e-24;                               // below it the force's r is taken as 1e-12
constexpr long long kTinyR2Bits = 0x3af357c299a88ea7LL;        // the bit pattern of kTinyR2 (checked in orbit_setup)
constexpr double kHaloG1 = 2.02 - 1.0;                          // gamma - 1, as the reference forms it
constexpr double kStepMyr = 0.5;                                // PH_PRE_STEP_MYR
constexpr int kSub = 10;                                        // PH_LIN_SUB
constexpr double kEps = 1e-5;                                   // PH_LIN_EPS_POS == PH_LIN_EPS_VEL

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
