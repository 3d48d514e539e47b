// pgx_screen_math.cuh -- FP64 per-point and per-pair arithmetic of the screen (internal header).
//
// Included only by translation units built with --fmad=false, so every expression below is evaluated as written:
// the reference's association and no fused multiply-add.  The FP64 screen and the FP64 rechecks of the
// mixed-precision screen call these same functions, which is what makes their results identical.
#pragma once
#include "pgx_internal.cuh"
#include "pgx_kernels.h"

namespace pgx {

constexpr double kInf = __builtin_huge_val();

// m^T M^-1 m for symmetric M = (xx xy xz yy yz zz) by the adjugate; -1 when det <= 0 (reference quad_inv,
// src/phygas.c:348-356).  The cofactors and the determinant are computed once per matrix and shared by the forms of
// a point (the same operations on the same operands as evaluating quad_inv for each, so the same bits).
struct Adj64 {
    double i00, i01, i02, i11, i12, i22, det;
    __device__ __forceinline__ explicit Adj64(const double (&M)[6]) {
        const double a = M[0], b = M[1], c = M[2], d = M[3], e = M[4], f = M[5];
        i00 = d * f - e * e; i01 = c * e - b * f; i02 = b * e - c * d;
        det = a * i00 + b * i01 + c * i02;
        i11 = a * f - c * c; i12 = b * c - a * e; i22 = a * d - b * b;
    }
    __device__ __forceinline__ double form(double mx, double my, double mz) const {
        if (!(det > 0)) return -1.0;
        return (mx * (i00 * mx + i01 * my + i02 * mz) + my * (i01 * mx + i11 * my + i12 * mz) +
                mz * (i02 * mx + i12 * my + i22 * mz)) / det;
    }
};
__device__ __forceinline__ double quad_inv64(const double (&M)[6], double mx, double my, double mz) {
    return Adj64(M).form(mx, my, mz);
}

// chi2 at one track point k of a pair: the form at the point's separation m0 and at the closest point of the step's
// segment m0 -> m1, with the reference's rule for which one counts and its trace bound (src/phygas.c:379-405).
// M holds S_target + S_cluster on entry.  Returns the point's chi2 (or -1: singular, or +inf: rejected by the
// bound) and the segment fraction s.
__device__ __forceinline__ double point_chi2_64(double (&M)[6], double R2, const double (&m0)[3],
                                                const double (&m1)[3], bool more, double cut, double &s_out) {
    M[0] += R2; M[3] += R2; M[5] += R2;
    s_out = 0.0;
    const double thr = 2.0 * cut * (M[0] + M[3] + M[5]);
    if (thr < kInf) {
        const double dx = m1[0] - m0[0], dy = m1[1] - m0[1], dz = m1[2] - m0[2];
        const double a = m0[0] * dx + m0[1] * dy + m0[2] * dz, dd = dx * dx + dy * dy + dz * dz;
        bool far;
        if (a >= 0) far = m0[0] * m0[0] + m0[1] * m0[1] + m0[2] * m0[2] > thr;
        else if (-a >= dd) far = m1[0] * m1[0] + m1[1] * m1[1] + m1[2] * m1[2] > thr;
        else far = (m0[0] * m0[0] + m0[1] * m0[1] + m0[2] * m0[2]) * dd - a * a > thr * dd;
        if (far) return kInf;
    }
    const Adj64 adj(M);
    double q = adj.form(m0[0], m0[1], m0[2]), s = 0.0;
    if (more) {
        const double dx = m1[0] - m0[0], dy = m1[1] - m0[1], dz = m1[2] - m0[2];
        const double dd = dx * dx + dy * dy + dz * dz;
        if (dd > 0) {
            s = -(m0[0] * dx + m0[1] * dy + m0[2] * dz) / dd;
            if (s < 0) s = 0; else if (s > 1) s = 1;
        }
        const double qs = adj.form(m0[0] + dx * s, m0[1] + dy * s, m0[2] + dz * s);
        if (qs >= 0 && qs < q) q = qs; else s = 0.0;
    }
    s_out = s;
    return q;
}

// running minimum over a pair's points, strict < in point order (the first of equal minima wins)
struct ScanState {
    double best, sb;
    int kb;
    __device__ __forceinline__ void begin() { best = kInf; sb = 0.0; kb = 0; }
    __device__ __forceinline__ void point(int k, double (&M)[6], double R2, const double (&m0)[3],
                                          const double (&m1)[3], bool more, double cut) {
        double s;
        const double q = point_chi2_64(M, R2, m0, m1, more, cut, s);
        if (q >= 0 && q < best) { best = q; kb = k; sb = s; }
    }
};

// the rest of a kept pair's row, and what its draws need (reference ph_screen_finish, src/phygas.c:413-431)
__device__ __forceinline__ void finish_prep_pair(const ScreenTables &T, const KeptPair &p, FinishIn &f,
                                                 ScreenRowDev &r) {
    const size_t NT = T.nt, NC = T.nc;
    const int n = T.ns < T.cn[p.c] ? T.ns : T.cn[p.c];
    const int kb = p.kb, k1 = kb + 1 < n ? kb + 1 : kb;
    const double sb = p.sb;
    const double *ta = T.t64 + (size_t)kb * 12 * NT + p.s, *ca = T.c64 + (size_t)kb * 12 * NC + p.c;
    const double *tb = T.t64 + (size_t)k1 * 12 * NT + p.s, *cb = T.c64 + (size_t)k1 * 12 * NC + p.c;
    const double ax = ta[0] - ca[0], ay = ta[NT] - ca[NC], az = ta[2 * NT] - ca[2 * NC];
    const double bx = tb[0] - cb[0], by = tb[NT] - cb[NC], bz = tb[2 * NT] - cb[2 * NC];
    const double mx = ax + (bx - ax) * sb, my = ay + (by - ay) * sb, mz = az + (bz - az) * sb;
    const double vx = ta[3 * NT] - ca[3 * NC], vy = ta[4 * NT] - ca[4 * NC], vz = ta[5 * NT] - ca[5 * NC];
    double C[6];
#pragma unroll
    for (int i = 0; i < 6; i++) C[i] = ta[(6 + i) * NT] + ca[(6 + i) * NC];
    r.star = p.s + T.s_off; r.cluster = p.c; r.kb = kb; r.pad = 0; r.sb = sb; r.chi2 = p.chi2;
    r.t_myr = ((double)kb + sb) * kStepMyr;
    r.d_nom_pc = sqrt(mx * mx + my * my + mz * mz) * 1000.0;
    r.vrel_kms = sqrt(vx * vx + vy * vy + vz * vz) * kKms;
    r.sig_pc = sqrt((C[0] + C[3] + C[5]) / 3.0) * 1000.0;
    r.p_r50 = r.p_rtot = 0.0;
    const double l00 = sqrt(fmax(C[0], 0.0)), l10 = l00 > 0 ? C[1] / l00 : 0.0, l20 = l00 > 0 ? C[2] / l00 : 0.0;
    const double l11 = sqrt(fmax(C[3] - l10 * l10, 0.0)), l21 = l11 > 0 ? (C[4] - l20 * l10) / l11 : 0.0;
    const double l22 = sqrt(fmax(C[5] - l20 * l20 - l21 * l21, 0.0));
    f.mx = mx; f.my = my; f.mz = mz;
    f.l00 = l00; f.l10 = l10; f.l20 = l20; f.l11 = l11; f.l21 = l21; f.l22 = l22;
    f.r50 = T.r50[p.c];
    f.rt = T.rtot[p.c];
    uint64_t h = T.seed_prefix[p.s];                       // ph_seed(id, name), FNV-1a continued over the name
    const unsigned char *nm = reinterpret_cast<const unsigned char *>(T.cname + (size_t)p.c * 40);
    for (int i = 0; i < 40 && nm[i]; i++) h = (h ^ nm[i]) * 1099511628211ULL;
    f.seed = h;
}

// one standard normal from two splitmix64 outputs (reference mc_gaussian, src/montecarlo.c:4-17), FP64
__device__ __forceinline__ double gauss64(uint64_t a, uint64_t b) {
    double u1 = (double)(a >> 11) * (1.0 / 9007199254740992.0);
    if (u1 <= 0.0) u1 = 1.0 / 18446744073709551616.0;
    const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
}

// position of draw i of a kept pair (its Gaussians are calls 6i+1 .. 6i+6 of the pair's stream)
__device__ __forceinline__ void draw_xyz64(const FinishIn &f, int i, double &x, double &y, double &z) {
    const uint64_t n = 6ull * (uint64_t)i;
    const double z0 = gauss64(splitmix_at(f.seed, n + 1), splitmix_at(f.seed, n + 2));
    const double z1 = gauss64(splitmix_at(f.seed, n + 3), splitmix_at(f.seed, n + 4));
    const double z2 = gauss64(splitmix_at(f.seed, n + 5), splitmix_at(f.seed, n + 6));
    x = f.mx + f.l00 * z0;
    y = f.my + f.l10 * z0 + f.l11 * z1;
    z = f.mz + f.l20 * z0 + f.l21 * z1 + f.l22 * z2;
}

// draw i of a kept pair: bit 0 = inside r50, bit 1 = inside rtot
__device__ __forceinline__ int draw_inside64(const FinishIn &f, int i) {
    double x, y, z;
    draw_xyz64(f, i, x, y, z);
    const double r = sqrt(x * x + y * y + z * z);
    return (r < f.r50 ? 1 : 0) | (r < f.rt ? 2 : 0);
}

}  // namespace pgx
