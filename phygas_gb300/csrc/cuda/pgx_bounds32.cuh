// pgx_bounds32.cuh -- the FP32 point evaluation of the mixed-precision screen with its error bounds (internal
// header; also compiles as plain host C++ with FP contraction off, which gives the device's results bit for bit --
// every fused multiply-add below is an explicit fmaf, and the file that includes it on the device is compiled with
// --fmad=false).
#pragma once
#include <cmath>
#include "pgx_bits.cuh"

namespace pgx {

// ---- the FP32 point evaluation with its error bounds ------------------------------------------------------------
constexpr float kEps32 = 5.9604645e-8f;      // 2^-24
// The FP32 LDL^T form is exact for a matrix M' with |M'_ij - M_ij| <= 14 eps sqrt(M_ii M_jj) (eps = 2^-24): 3 for
// storing S_t, S_c, R^2 in FP32 and adding them, 7 for the factorization (the (2,2) entry; |l_ik| D_k |l_jk| sums to
// at most sqrt(M_ii M_jj) for positive pivots), 4 for the two-row forward substitution (twice its 2 eps
// componentwise backward error).  The matrix sqrt(M_ii M_jj) has spectral norm tr(M), so ||M' - M|| <= kC1 eps tr(M)
// with kC1 = 16 (14 plus second-order terms); then (1 - rho) M <= M' <= (1 + rho) M, rho = kC1 eps tr(M) / lam, and
// the exact form lies within rho of the form of M', which the rounding of squares, reciprocals and sums (5 eps)
// separates from the computed one: kC2 = 16 covers it with margin.
constexpr float kC1 = 16.f, kC2 = 16.f;
// relative error of the FP64 path's adjugate form m^T adj(M) m / det(M) (pgx_screen_math.cuh): cofactors, det
// and numerator each lose at most a few hundred ulps of T^3 / det, T = trace(M) (all |M_ij| <= T); 256 eps_64
constexpr float kAdj64 = 2.85e-14f;

struct Bound {
    float lb, ub;          // lb <= the FP64 path's point chi2 <= ub (ub = +inf: no upper bound)
};

// m^T (L D L^T)^-1 m with the factors of one point
PGX_HD float ldl_form(float l10, float l20, float l21, float i1, float i2, float i3, float x,
                                          float y, float z) {
    const float y1 = fmaf(-l10, x, y);
    const float y2 = fmaf(-l21, y1, fmaf(-l20, x, z));
    return fmaf(y2 * y2, i3, fmaf(y1 * y1, i2, x * x * i1));
}

// The reference's trace bound (chi2 >= dist^2 / trace M over the step's segment) with FP32 margins: the exact
// dist^2 > 1.5 cut tr (factor 2, cancellation limited by the m00 guard), so the exact chi2 > 1.5 cut, and the FP64
// path's value -- rejected by its own test, or evaluated with relative error < 1/3 (the tr / lam guard, see
// kAdj64) -- is above the cut.  a = m0.dr, dd = |dr|^2, m00 = |m0|^2, m11 = |m1|^2.
PGX_HD bool trace_far32(float a, float dd, float m00, float m11, float tr, float lam, float cut) {
    const float thr = 2.f * cut * tr;
    const float thr_m = thr * (1.f + 1e-5f);
    bool far;
    if (a >= 0.f) far = m00 > thr_m;
    else if (-a >= dd) far = m11 > thr_m;
    else far = (fmaf(m00, dd, -a * a) > thr_m * dd) && (m00 * (8.f * kEps32) < cut * tr);
    return far && tr < 1.8e6f * lam;
}

// Reciprocal and reciprocal square root on the GPU's fast units: within 2 ulp (4 eps relative) by their documented
// worst case (PTX rcp.approx.f32: 1 ulp; rsqrt.approx.f32: relative error 2^-22.9; both over the full range).  The
// .ftz forms flush subnormal arguments and results, which never occur here: every argument is checked or clamped to
// be at least 1e-30, and a reciprocal's argument at most 1e30, so arguments and results are normal -- and they issue
// as one special-function instruction, without the subnormal scaling around it.  Host builds use the exact operations,
// which the same margins cover, scaled by (1 + host_fast_err): a host test sets it to put the results at either end
// of the device units' error band (it is 0 otherwise, and does not exist in device code).
#ifndef __CUDA_ARCH__
inline float host_fast_err = 0.f;
#endif
PGX_HD float fast_rcp(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.f / x * (1.f + host_fast_err);
#endif
}
PGX_HD float fast_rsqrt(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.f / sqrtf(x) * (1.f + host_fast_err);
#endif
}

// A cheap test, run before the full bounds, that the FP64 path's point chi2 v is >= cut: then the point can be
// neither a kept pair's minimum nor under the cut, and needs no bounds.  The trace bound is not tried first: on the
// screen's workload it never settles all 32 lanes of a warp at once, so it would only add instructions, and this
// test settles all but 0.05 % of the points it rejects (those go to the full bounds, which apply it).
// True by the triangle inequality in the M^-1 norm: the points the FP64 path evaluates (m0 and its nearest point u) lie
// on the FP64 segment m0 -> m1, within dx = 3 eps max(|m0|, |m1|) of the FP32 segment, whose points all have
// |x| >= |m0| - |dr|.  With q0 = m0^T M^-1 m0 and c = dr^T M^-1 dr as FP32 LDL^T forms and lam <= lambda_min(M):
// v >= (1 - r64) (sqrt(q0 (1 - r)) - sqrt(c (1 + r)) - dx / sqrt(lam))^2, r64 <= 3 kAdj64 (tr / lam)^2 the FP64
// adjugate's rounding (det(M) >= lam^2 tr / 3).
// The reciprocals and square roots run on the fast units (4 eps each), so the error terms of point_bound32 grow:
// the factorization's backward error becomes 13 eps sqrt(M_ii M_jj) (5 eps in each l, 6 in the pivots), with the
// storage's 3 and the substitution's 4 at most 20 eps tr(M) -- kSkipC1 = 24 -- and the form's own rounding 8 eps
// (12 below); each square root via x rsqrtf(x) is within 5 eps.
constexpr float kSkipC1 = 24.f;
PGX_HD bool point_skip32(const float (&St)[6], const float (&Sc)[6], float lmt, float lmc,
                         const float (&m0)[3], const float (&m1)[3], float cut) {
    const float M0 = St[0] + Sc[0], M1 = St[1] + Sc[1], M2 = St[2] + Sc[2];
    const float M3 = St[3] + Sc[3], M4 = St[4] + Sc[4], M5 = St[5] + Sc[5];
    const float tr = M0 + M3 + M5;
    const float lam = (lmt + lmc) * (1.f - 16.f * kEps32);
    const float dx = m1[0] - m0[0], dy = m1[1] - m0[1], dz = m1[2] - m0[2];
    const float m00 = fmaf(m0[0], m0[0], fmaf(m0[1], m0[1], m0[2] * m0[2]));
    const float m11 = fmaf(m1[0], m1[0], fmaf(m1[1], m1[1], m1[2] * m1[2]));
    if (!(lam > 1e-30f && M0 > 1e-30f && tr < 1e30f)) return false;
    const float i1 = fast_rcp(M0);
    const float l10 = M1 * i1, l20 = M2 * i1;
    const float D2 = fmaf(-l10, M1, M3);
    if (!(D2 > 1e-30f)) return false;
    const float i2 = fast_rcp(D2);
    const float uu = fmaf(-l20, M1, M4);
    const float l21 = uu * i2;
    const float D3 = fmaf(-l21, uu, fmaf(-l20, M2, M5));
    if (!(D3 > 1e-30f)) return false;
    const float i3 = fast_rcp(D3);
    const float il = fast_rcp(lam);
    const float tl = tr * il * (1.f + 8.f * kEps32);
    const float rho = kSkipC1 * kEps32 * tl;
    if (!(rho <= 0.25f)) return false;
    const float q0 = ldl_form(l10, l20, l21, i1, i2, i3, m0[0], m0[1], m0[2]);
    const float c = ldl_form(l10, l20, l21, i1, i2, i3, dx, dy, dz);
    const float r = rho + 12.f * kEps32;
    const float big2 = fmaxf(fmaxf(m00, m11), 1e-30f);
    const float big = big2 * fast_rsqrt(big2) * (1.f + 8.f * kEps32);
    const float qa = fmaxf(q0 * (1.f - r), 1e-30f), ca = fmaxf(c * (1.f + r), 1e-30f);
    const float d = qa * fast_rsqrt(qa) * (1.f - 8.f * kEps32) - ca * fast_rsqrt(ca) * (1.f + 8.f * kEps32) -
                    (3.f * kEps32 * big + 1e-12f) * fast_rsqrt(lam) * (1.f + 8.f * kEps32);
    if (!(d > 0.f)) return false;
    const float r64 = kAdj64 * 3.f * (1.f + 16.f * kEps32) * tl * tl;
    return d * d * (1.f - r64) * (1.f - 8.f * kEps32) >= cut;
}

// ---- block culling: eight points of a pair settled by one test ---------------------------------------------------
// A block is track points [8b, 8b + 8) of a pair with the segment end 8b + 8 (those that exist: k < n).  Per object
// (star or cluster) and block, computed in FP64 from its track (k_block_tables), with km = 8b + 4 the position
// reference and ke = min(8b + 8, n_obj - 1) the last point of the block's range:
//   v, a     FP32 velocity and acceleration at km, and eps >= |p(k) - p(km) - v tau_k - a tau_k^2 / 2| over the range
//            (tau_k = (km - k) h, h = 0.5 Myr: the track runs back in time) plus a h^2 / 8 for the chords between
//            points, so every point the FP64 path evaluates for the block -- m0 at a track point, or its nearest
//            point on a chord -- lies in the tube p(km) + v tau + a tau^2 / 2 + e, |e| <= eps, |tau| <= 4 h;
//   S        an FP32 matrix that dominates S(k) (+ R^2 I for a cluster) at every point of the range: S(ke) + delta I,
//            delta >= the largest eigenvalue of S(k) - S(ke) over the range, or -- the covariances are needle-thin
//            and turn along the track, so S(k) - S(ke) is positive mostly along one direction u and delta is often
//            many times the thin axis -- S(ke) + alpha u u^T + beta I with beta covering the plane orthogonal to u
//            (k_block_tables derives both); the FP32 rounding absorbed;
//   lam      <= lambda_min(S) (the point's FP64 lower bound at ke, plus delta or beta, rounded down);
//   lam_lo   <= lambda_min(S(k)) at every point of the range (the point bounds' minimum), for the adjugate's error.
// For a pair, M(k) = S_t(k) + S_c(k) + R^2 I <= N = S_t + S_c (Loewner order), so x^T M(k)^-1 x >= x^T N^-1 x, and
// every evaluated x = m_ref + dv tau + da tau^2 / 2 + e (m_ref = the separation at km, dv and da the differences)
// has, by the triangle inequality in the N^-1 norm,
//   |x|_N >= |m_ref|_N - 4h |dv|_N - 8h^2 |da|_N - (eps_t + eps_c + 3 eps |m_ref|) / sqrt(lam_t + lam_c).
// The N^-1 forms come from one FP32 LDL^T with point_skip32's margins.  When the square of the bound, less the FP64
// adjugate's rounding at M(k) (tr M(k) <= tr N, lambda_min M(k) >= lam_lo_t + lam_lo_c), is >= cut, every point of
// the block has v >= cut: none can be a kept pair's minimum or bring the pair under the cut.
constexpr int kBlk = 8;                       // points per block
#ifndef PGX_BLK_TAU
#define PGX_BLK_TAU 2.0f                      // (a host test of the bound may build it with another value)
#endif
constexpr float kBlkTau = PGX_BLK_TAU;        // Myr: the largest |tau| in a block's tube (4 steps of 0.5 Myr)

// The point test against a block's dominating matrix N = S_t + S_c (the block tables of the point's block) in place of
// the point's own M(k): M(k) <= N, so every form in M(k)^-1 is at least the form in N^-1; lam <= lambda_min(N), and
// the FP64 adjugate's rounding at M(k) from tr(N) / lam_lo as in the block test.  Otherwise point_skip32's triangle
// test on the step's segment.
PGX_HD bool point_skip32_blk(const float4 (&bt)[4], const float4 (&bc)[4], const float (&m0)[3], const float (&m1)[3],
                             float cut) {
    const float N0 = bt[2].x + bc[2].x, N1 = bt[2].y + bc[2].y, N2 = bt[2].z + bc[2].z;
    const float N3 = bt[2].w + bc[2].w, N4 = bt[3].x + bc[3].x, N5 = bt[3].y + bc[3].y;
    const float tr = N0 + N3 + N5;
    const float lam = (bt[1].w + bc[1].w) * (1.f - 16.f * kEps32);
    const float lam_lo = (bt[3].z + bc[3].z) * (1.f - 16.f * kEps32);
    if (!(lam > 1e-30f && lam_lo > 1e-30f && N0 > 1e-30f && tr < 1e30f)) return false;
    const float i1 = fast_rcp(N0);
    const float l10 = N1 * i1, l20 = N2 * i1;
    const float D2 = fmaf(-l10, N1, N3);
    if (!(D2 > 1e-30f)) return false;
    const float i2 = fast_rcp(D2);
    const float uu = fmaf(-l20, N1, N4);
    const float l21 = uu * i2;
    const float D3 = fmaf(-l21, uu, fmaf(-l20, N2, N5));
    if (!(D3 > 1e-30f)) return false;
    const float i3 = fast_rcp(D3);
    const float tl = tr * fast_rcp(lam) * (1.f + 8.f * kEps32);
    const float rho = kSkipC1 * kEps32 * tl;
    if (!(rho <= 0.25f)) return false;
    const float dx = m1[0] - m0[0], dy = m1[1] - m0[1], dz = m1[2] - m0[2];
    const float m00 = fmaf(m0[0], m0[0], fmaf(m0[1], m0[1], m0[2] * m0[2]));
    const float m11 = fmaf(m1[0], m1[0], fmaf(m1[1], m1[1], m1[2] * m1[2]));
    const float q0 = ldl_form(l10, l20, l21, i1, i2, i3, m0[0], m0[1], m0[2]);
    const float c = ldl_form(l10, l20, l21, i1, i2, i3, dx, dy, dz);
    const float r = rho + 12.f * kEps32;
    const float big2 = fmaxf(fmaxf(m00, m11), 1e-30f);
    const float big = big2 * fast_rsqrt(big2) * (1.f + 8.f * kEps32);
    const float qa = fmaxf(q0 * (1.f - r), 1e-30f), ca = fmaxf(c * (1.f + r), 1e-30f);
    const float d = qa * fast_rsqrt(qa) * (1.f - 8.f * kEps32) - ca * fast_rsqrt(ca) * (1.f + 8.f * kEps32) -
                    (3.f * kEps32 * big + 1e-12f) * fast_rsqrt(lam) * (1.f + 8.f * kEps32);
    if (!(d > 0.f)) return false;
    const float tlo = tr * fast_rcp(lam_lo) * (1.f + 8.f * kEps32);
    const float r64 = kAdj64 * 3.f * (1.f + 16.f * kEps32) * tlo * tlo;
    return d * d * (1.f - r64) * (1.f - 8.f * kEps32) >= cut;
}

PGX_HD bool block_skip32(const float4 (&bt)[4], const float4 (&bc)[4], const float (&mref)[3], float cut) {
    const float N0 = bt[2].x + bc[2].x, N1 = bt[2].y + bc[2].y, N2 = bt[2].z + bc[2].z;
    const float N3 = bt[2].w + bc[2].w, N4 = bt[3].x + bc[3].x, N5 = bt[3].y + bc[3].y;
    const float tr = N0 + N3 + N5;
    const float lam = (bt[1].w + bc[1].w) * (1.f - 16.f * kEps32);
    const float lam_lo = (bt[3].z + bc[3].z) * (1.f - 16.f * kEps32);
    if (!(lam > 1e-30f && lam_lo > 1e-30f && N0 > 1e-30f && tr < 1e30f)) return false;
    const float i1 = fast_rcp(N0);
    const float l10 = N1 * i1, l20 = N2 * i1;
    const float D2 = fmaf(-l10, N1, N3);
    if (!(D2 > 1e-30f)) return false;
    const float i2 = fast_rcp(D2);
    const float uu = fmaf(-l20, N1, N4);
    const float l21 = uu * i2;
    const float D3 = fmaf(-l21, uu, fmaf(-l20, N2, N5));
    if (!(D3 > 1e-30f)) return false;
    const float i3 = fast_rcp(D3);
    const float il = fast_rcp(lam);
    const float tl = tr * il * (1.f + 8.f * kEps32);
    const float rho = kSkipC1 * kEps32 * tl;
    if (!(rho <= 0.25f)) return false;
    const float dvx = bt[0].x - bc[0].x, dvy = bt[0].y - bc[0].y, dvz = bt[0].z - bc[0].z;
    const float dax = bt[1].x - bc[1].x, day = bt[1].y - bc[1].y, daz = bt[1].z - bc[1].z;
    const float qa = ldl_form(l10, l20, l21, i1, i2, i3, mref[0], mref[1], mref[2]);
    const float qv = ldl_form(l10, l20, l21, i1, i2, i3, dvx, dvy, dvz);
    const float qc = ldl_form(l10, l20, l21, i1, i2, i3, dax, day, daz);
    // the differences dv, da are FP32 subtractions of the stored values (relative 1 eps each): 2 eps more
    const float r = rho + 12.f * kEps32, rs = r + 2.f * kEps32;
    const float m2 = fmaxf(fmaf(mref[0], mref[0], fmaf(mref[1], mref[1], mref[2] * mref[2])), 1e-30f);
    const float mn = m2 * fast_rsqrt(m2) * (1.f + 8.f * kEps32);
    const float sa = fmaxf(qa * (1.f - r), 1e-30f), sv = fmaxf(qv * (1.f + rs), 1e-30f),
                sc = fmaxf(qc * (1.f + rs), 1e-30f);
    const float e = (bt[0].w + bc[0].w) * (1.f + 4.f * kEps32) + 3.f * kEps32 * mn + 1e-12f;
    const float d = sa * fast_rsqrt(sa) * (1.f - 8.f * kEps32) -
                    kBlkTau * (sv * fast_rsqrt(sv)) * (1.f + 8.f * kEps32) -
                    (0.5f * kBlkTau * kBlkTau) * (sc * fast_rsqrt(sc)) * (1.f + 8.f * kEps32) -
                    e * fast_rsqrt(lam) * (1.f + 8.f * kEps32);
    if (!(d > 0.f)) return false;
    const float tlo = tr * fast_rcp(lam_lo) * (1.f + 8.f * kEps32);
    const float r64 = kAdj64 * 3.f * (1.f + 16.f * kEps32) * tlo * tlo;
    if (!(r64 < 0.5f)) return false;
    return d * d * (1.f - r64) * (1.f - 12.f * kEps32) >= cut;
}

// Bounds on the FP64 path's point chi2 v = min(q(m0), q(ms)) -- the forms at the step's start and at the segment's
// nearest point to the origin, pgx_screen_math.cuh point_chi2_64 -- from FP32 data.  Returns false when the point is
// rejected by the reference's trace bound with margins (see below): then v, if the FP64 path evaluates it at all,
// is above the cut, and the point can neither be the minimum of a kept pair nor bring a pair under the cut.
//
// The cluster side carries the kernel radius: Sc = S_c + R^2 I, each entry the FP32 rounding of the FP64 sum (one
// rounding, where St + S_c + R^2 in FP32 took three), and lmc <= lmin(S_c) + R^2, so M = St + Sc.
// lam = lmt + lmc <= lambda_min(M) (Weyl; the lmin are FP64 lower bounds from the covariance kernel, rounded down).
// Bounds on the exact forms, then the FP64 path's own rounding on top:
//  * Rayleigh, robust to any conditioning: for any vector w, x^T M^-1 x >= (w.x)^2 / w^T M w (Cauchy-Schwarz), and
//    on the segment w.x >= min(w.m0, w.m1); with w = m0, m1 and the FP32 nearest point u this bounds the whole
//    segment from below (w^T M w needs no inversion: error <= 10 eps (sum sqrt(M_ii) |w_i|)^2).
//  * LDL^T in FP32 where it is well conditioned: the computed form is exact for a matrix within kC1 eps tr(M) of M
//    (storage, two additions, the factorization's and the substitution's backward errors), so the exact form is
//    within rho relative of it, rho = kC1 eps tr(M) / lam; kC2 eps more for squares and sums.  A point that differs from the FP64 path's by
//    <= d moves a form by <= 2 sqrt(q / lam) d + d^2 / lam in any direction: d0 = 3 eps |m0| for the start (hi/lo
//    rounding), du for the nearest point.  Locating that point is ill-conditioned for a short step nearly
//    tangent to the sphere through m0 (s = -m0.dr / |dr|^2), so du comes from the errors of m0.dr and |dr|^2, and is
//    never more than the segment's own length (both points lie on it).
//  * The FP64 adjugate evaluation adds relative error <= kAdj64 T^3 / det(M), det(M) >= lam^2 tr(M) / 3.
// lb <= v <= ub: lb = max(Rayleigh, min(lb(q0), lb(qs))), ub = min(ub(q0), ub(qs)) (+inf without LDL^T).
PGX_HD bool point_bound32(const float (&St)[6], const float (&Sc)[6], float lmt, float lmc,
                                              const float (&m0)[3], const float (&m1)[3], bool more, float cut,
                                              Bound &b) {
    const float inf = __builtin_huge_valf();
    const float M0 = St[0] + Sc[0], M1 = St[1] + Sc[1], M2 = St[2] + Sc[2];
    const float M3 = St[3] + Sc[3], M4 = St[4] + Sc[4], M5 = St[5] + Sc[5];
    const float tr = M0 + M3 + M5;
    const float lam = (lmt + lmc) * (1.f - 16.f * kEps32);
    const float dx = m1[0] - m0[0], dy = m1[1] - m0[1], dz = m1[2] - m0[2];
    const float a = fmaf(m0[0], dx, fmaf(m0[1], dy, m0[2] * dz));
    const float dd = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float m00 = fmaf(m0[0], m0[0], fmaf(m0[1], m0[1], m0[2] * m0[2]));
    const float m11 = fmaf(m1[0], m1[0], fmaf(m1[1], m1[1], m1[2] * m1[2]));
    if (trace_far32(a, dd, m00, m11, tr, lam, cut)) return false;
    if (!(lam > 0.f)) {
        b.lb = 0.f;
        b.ub = inf;
        return true;
    }
    const float big = sqrtf(fmaxf(m00, m11));
    const float n0 = sqrtf(m00);
    const float dr_err = 8.f * kEps32 * big + 1e-12f;   // |FP32 dr - FP64 dr|: the rounding of m0 and m1
    float s = 0.f;
    if (more && dd > 0.f) s = fminf(fmaxf(-a / dd, 0.f), 1.f);
    const float ux = fmaf(dx, s, m0[0]), uy = fmaf(dy, s, m0[1]), uz = fmaf(dz, s, m0[2]);
    float du = 3.f * kEps32 * n0 + 1e-12f;
    if (more) {
        const float dn = sqrtf(dd);
        float dv = 2.f * dn + dr_err + 3.f * kEps32 * big;      // both points lie on the segment
        if (dn > 2.f * dr_err) {
            const float dd_lo = (dn - dr_err) * (dn - dr_err), dr_hi = dn + dr_err;
            const float a_err = big * dr_err * (1.f + 4.f * kEps32) + 6.f * kEps32 * big * dn;
            const float dd_err = 2.f * dn * dr_err + dr_err * dr_err + 4.f * kEps32 * dd;
            const float ds = a_err / dd_lo + fabsf(a) * dd_err / (dd * dd_lo);
            dv = fminf(dv, 3.f * kEps32 * big + dr_err + ds * dr_hi);
        }
        du = dv * (1.f + 8.f * kEps32);
    }
    // Rayleigh lower bound over the segment, w = m0, m1, u
    float lb = 0.f;
    {
        const float sq0 = sqrtf(M0), sq3 = sqrtf(M3), sq5 = sqrtf(M5);
        const float W[3][3] = {{m0[0], m0[1], m0[2]}, {m1[0], m1[1], m1[2]}, {ux, uy, uz}};
#pragma unroll
        for (int w = 0; w < 3; w++) {
            if (w > 0 && !more) break;
            const float wx = W[w][0], wy = W[w][1], wz = W[w][2];
            const float wn = sqrtf(fmaf(wx, wx, fmaf(wy, wy, wz * wz)));
            const float e0 = fmaf(wx, m0[0], fmaf(wy, m0[1], wz * m0[2]));
            const float e1 = more ? fmaf(wx, m1[0], fmaf(wy, m1[1], wz * m1[2])) : e0;
            const float t = fminf(e0, e1) - 9.f * kEps32 * wn * big;
            const float wMw = fmaf(M0, wx * wx, fmaf(M3, wy * wy, fmaf(M5, wz * wz,
                              2.f * fmaf(M1, wx * wy, fmaf(M2, wx * wz, M4 * wy * wz)))));
            const float sw = fmaf(sq0, fabsf(wx), fmaf(sq3, fabsf(wy), sq5 * fabsf(wz)));
            const float wMw_ub = fmaxf(wMw, 0.f) + 10.f * kEps32 * sw * sw;
            if (t > 0.f && wMw_ub > 0.f) lb = fmaxf(lb, t * t / wMw_ub * (1.f - 8.f * kEps32));
        }
    }
    float ub = inf;
    // LDL^T
    const float D1 = M0;
    const float i1 = 1.f / D1;
    const float l10 = M1 * i1, l20 = M2 * i1;
    const float D2 = fmaf(-l10, M1, M3);
    const float i2 = 1.f / D2;
    const float uu = fmaf(-l20, M1, M4);
    const float l21 = uu * i2;
    const float D3 = fmaf(-l21, uu, fmaf(-l20, M2, M5));
    const float i3 = 1.f / D3;
    const bool pos = D1 > 0.f && D2 > 0.f && D3 > 0.f;
    // A second lower bound on lambda_min(M): det(M) / c2(M), c2 = the sum of the 2x2 principal minors
    // (= l1 l2 + l1 l3 + l2 l3 >= l1 l2), much closer than the Weyl sum when S_t and S_c are thin in different
    // directions.  det(M) >= D1 D2 D3 / (1 + rho)^3: the factors are exact for M' with |M' - M| <= rho lam, so every
    // eigenvalue of M is >= its eigenvalue of M' / (1 + rho).  c2 from FP32 data is within 16 eps of
    // (M0 M3 + M0 M5 + M3 M5) of the exact value (storage and the products).
    float lamx = lam;
    if (pos) {
        const float g = 1.f + kC1 * kEps32 * tr / lam;
        const float det_lo = D1 * D2 * D3 * (1.f - 8.f * kEps32) / (g * g * g);
        const float P = fmaf(M0, M3, fmaf(M0, M5, M3 * M5));
        const float c2 = fmaf(M0, M3, -(M1 * M1)) + fmaf(M0, M5, -(M2 * M2)) + fmaf(M3, M5, -(M4 * M4));
        const float c2_ub = fmaf(16.f * kEps32, P, c2) * (1.f + 4.f * kEps32);
        if (c2_ub > 0.f) lamx = fmaxf(lam, det_lo / c2_ub * (1.f - 4.f * kEps32));
    }
    const float rho = kC1 * kEps32 * tr / lamx;
    const bool ldl = pos && rho <= 0.25f;
    const float T = tr * (1.f + 4.f * kEps32);
    float det_lb = lamx * lamx * tr * (1.f / 3.f) * (1.f - 8.f * kEps32);
    if (ldl) {
        const float rel = rho + kC2 * kEps32;
        const float il = 1.f / lamx;
        const float q0 = ldl_form(l10, l20, l21, i1, i2, i3, m0[0], m0[1], m0[2]);
        const float d0 = 3.f * kEps32 * n0 + 1e-12f;
        const float e0 = 2.f * sqrtf(q0 * (1.f + rel) * il) * d0 + d0 * d0 * il;
        float lo = fmaf(q0, -rel, q0) - e0;
        ub = fmaf(q0, rel, q0) + e0;
        if (more) {
            const float qs = ldl_form(l10, l20, l21, i1, i2, i3, ux, uy, uz);
            const float es = 2.f * sqrtf(qs * (1.f + rel) * il) * du + du * du * il;
            lo = fminf(lo, fmaf(qs, -rel, qs) - es);
            ub = fminf(ub, fmaf(qs, rel, qs) + es);
        }
        lb = fmaxf(lb, lo);
        const float g = 1.f + rho;
        det_lb = fmaxf(det_lb, D1 * D2 * D3 * (1.f - 8.f * kEps32) / (g * g * g));
    }
    const float r64 = det_lb > 0.f ? kAdj64 * (T * T) * (T / det_lb) : inf;
    if (!(r64 < 0.5f)) {
        b.lb = 0.f;
        b.ub = inf;
        return true;
    }
    b.lb = fmaxf(lb * (1.f - r64), 0.f);
    b.ub = ub < inf ? ub * (1.f + r64) * (1.f + 4.f * kEps32) : inf;
    return true;
}

}  // namespace pgx
