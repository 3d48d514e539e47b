// pgx_mixed.cu -- the mixed-precision screen of libphygas_gb300, and the cluster-table column gather.
//
// The orbits and state-transition matrices stay FP64 (pgx_orbit.cu).  The scan over every (star, cluster, point)
// and the 512 draws per kept pair run in FP32 on cluster-relative coordinates (star and cluster positions carried
// as FP32 hi + lo pairs, so m = (t_hi - c_hi) + (t_lo - c_lo) keeps FP64-level accuracy of the separation), each
// FP32 value with a rigorous error bound.  Only what the bound cannot decide is recomputed with the FP64 path's own
// functions (pgx_screen_math.cuh), so the rows are the FP64 path's rows bit for bit:
//
//   k_block_tables   per star and per cluster and block of 8 track points: the data of the block test
//   k_mx_scan32_blocks  the filter below with a first level: one test per (pair, block of 8 points) settles the
//                    block's points at once (most blocks); the blocks it cannot settle are walked point by point
//                    as below, 32 blocks at a time on full warps.  The default (PHYGAS_SCAN_BLOCKS=0: k_mx_scan32)
//   k_mx_scan32      FP32 filter, one thread per pair (warp = 32 stars x one cluster).  Per point: a cheap skip
//                    test (triangle inequality in the M^-1 norm, one FP32 LDL^T) that settles most points; the rest
//                    are queued per warp for the bounds LB <= chi2_64 <= UB on the FP64 path's value (the
//                    reference's trace bound, a Rayleigh lower bound that needs no inversion, and an LDL^T solve
//                    where it is well conditioned), 32 at a time on full warps.
//                    Per pair: its candidate points -- those that can be the FP64 minimum of a kept pair
//                    (LB_k < cut, LB_k <= min UB) -- in four slots, or "more than four".
//   k_mx_count / k_mx_emit   stable compaction of the pairs that may be kept, a thread per (star, range of 1/16 of
//                            the clusters)
//   k_mx_list_*      the listed candidates written out; k_mx_cand walks the overflowed pairs again for theirs,
//                    keeping up to 64 per pair for k_mx_cand_copy (k_mx_cand_big walks a pair with more a third time)
//   k_mx_eval64      one thread per candidate point: the FP64 point chi2 (full warps on the scarce FP64 pipe)
//   k_mx_best        per possible pair: FP64 argmin over its candidates (smallest value, first point of equals)
//   k_mx_kept_*      stable compaction of the pairs under the cut
//   k_mx_finish32    one warp per kept pair: the 512 draws in FP32 with a per-draw error bound, in two phases (the
//                    first Gaussian settles the draws far outside both radii; the rest are completed from a
//                    per-warp queue); a draw whose distance is within the bound of r50 or rtot is redone in FP64
#include <algorithm>
#include <vector>
#include "pgx_bits.cuh"
#include "pgx_bounds32.cuh"
#include "pgx_internal.cuh"
#include "pgx_mixed.h"
#include "pgx_screen_math.cuh"

namespace pgx {

static_assert(kBlk == kBlockPoints, "the block tables and the filter's block test agree on the block size");

int grow(DevBuf &b, size_t bytes, std::string &err) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return 0;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes + bytes / 4);
    if (e != cudaSuccess) {
        err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGX_E_NOMEM : PGX_E_CUDA;
    }
    b.cap = bytes + bytes / 4;
    return 0;
}
int check(cudaError_t e, std::string &err, const char *what) {
    if (e == cudaSuccess) return 0;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return PGX_E_CUDA;
}

namespace {
template <class T> T *Pb(DevBuf &b) { return reinterpret_cast<T *>(b.p); }
}  // namespace

void mixed_free(MixedBufs &m) {
    DevBuf *all[] = {&m.order, &m.ub, &m.kmin, &m.flag, &m.cnt, &m.off, &m.total, &m.kept, &m.cand, &m.cand_off,
                     &m.ent, &m.entq, &m.aux, &m.ovf};
    for (DevBuf *b : all)
        if (b->p) { cudaFree(b->p); b->p = nullptr; b->cap = 0; }
}

// ---- cluster table: slot order (longest track first) -> cluster order ------------------------------------------
__global__ void k_gather_cols(int nc, int nmax, const int *__restrict__ order, const double *__restrict__ s64,
                              const float4 *__restrict__ s32, const float *__restrict__ slm, double *__restrict__ d64,
                              float4 *__restrict__ d32, float *__restrict__ dlm) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)nc * nmax) return;
    const int slot = (int)(idx % nc), k = (int)(idx / nc), col = order[slot];
    const size_t NC = nc;
    for (int f = 0; f < 12; f++) d64[((size_t)k * 12 + f) * NC + col] = s64[((size_t)k * 12 + f) * NC + slot];
    for (int q = 0; q < 3; q++) d32[((size_t)k * NC + col) * 3 + q] = s32[((size_t)k * NC + slot) * 3 + q];
    dlm[(size_t)k * NC + col] = slm[(size_t)k * NC + slot];
}

int gather_columns(cudaStream_t st, int nc, int nmax, const int *order_host, const double *t64_slot,
                   const float4 *t32_slot, const float *lm_slot, double *c64, float4 *c32, float *clm, MixedBufs &m) {
    int rc = grow(m.order, (size_t)nc * 4, m.err);
    if (rc) return rc;
    if ((rc = check(cudaMemcpyAsync(m.order.p, order_host, (size_t)nc * 4, cudaMemcpyHostToDevice, st), m.err, "order")))
        return rc;
    if ((rc = check(cudaMemsetAsync(c64, 0, (size_t)nmax * 12 * nc * 8, st), m.err, "memset"))) return rc;
    if ((rc = check(cudaMemsetAsync(c32, 0, (size_t)nmax * 3 * nc * 16, st), m.err, "memset"))) return rc;
    if ((rc = check(cudaMemsetAsync(clm, 0, (size_t)nmax * nc * 4, st), m.err, "memset"))) return rc;
    const size_t work = (size_t)nc * nmax;
    k_gather_cols<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(nc, nmax, Pb<int>(m.order), t64_slot, t32_slot,
                                                                   lm_slot, c64, c32, clm);
    if ((rc = check(cudaGetLastError(), m.err, "k_gather_cols"))) return rc;
    return check(cudaStreamSynchronize(st), m.err, "gather sync");
}

// The FP32 cluster table carries the kernel radius: S + R^2 I rounded once from FP64, and lmin + R^2 rounded down
// (point_skip32 / point_bound32 read M = St + Sc and lam = lmt + lmc).  The FP64 table is left as it is.
__global__ void k_fold_r2(int nc, int nmax, const int *__restrict__ cn, const double *__restrict__ c64,
                          const double *__restrict__ R2, float4 *__restrict__ c32, float *__restrict__ clm) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)nc * nmax) return;
    const int c = (int)(idx % nc), k = (int)(idx / nc);
    if (k >= cn[c]) return;
    const size_t NC = nc;
    const double r2 = R2[c];
    const double *S = c64 + ((size_t)k * 12 + 6) * NC + c;      // xx xy xz yy yz zz
    float4 *q = c32 + ((size_t)k * NC + c) * 3;
    q[1].z = (float)(S[0] + r2);
    q[2].y = (float)(S[3 * NC] + r2);
    q[2].w = (float)(S[5 * NC] + r2);
    clm[(size_t)k * NC + c] = __double2float_rd((double)clm[(size_t)k * NC + c] + r2);
}

int mixed_cluster_aux(cudaStream_t st, int nc, int nmax, const int *cn, const double *c64, const double *R2,
                      float4 *c32, float *clm, MixedBufs &m) {
    const size_t work = (size_t)nc * nmax;
    k_fold_r2<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(nc, nmax, cn, c64, R2, c32, clm);
    return check(cudaGetLastError(), m.err, "k_fold_r2");
}

// ---- block tables: per object (star or cluster) and block of kBlk points, the data block_skip32 reads --------------
// t64 [k][12][N] (pos, vel, S), lm [k][N] (FP32 lower bounds on lambda_min(S), with R^2 for the clusters), npts[i]
// points (nullptr: nmax for every object), R2[i] on the diagonal of S (clusters; nullptr for stars).  Out: blk
// [b][N][4] float4 = (v, eps) (a, lam) (S0 S1 S2 S3) (S4 S5 lam_lo 0), as pgx_bounds32.cuh describes; a block whose
// position reference km = kBlk b + kBlk/2 lies past the object's track is zeroed (no pair tests it: a pair tests
// block b only when km < its point count, which is at most the object's).
__global__ void k_block_tables(int N, int nmax, const int *__restrict__ npts, const double *__restrict__ t64,
                               const float *__restrict__ lm, const double *__restrict__ R2,
                               float4 *__restrict__ blk) {
    const int nblk = (nmax + kBlk - 1) / kBlk;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)N * nblk) return;
    const size_t NN = N;
    const int i = (int)(idx % NN), b = (int)(idx / NN);
    const int n = npts ? npts[i] : nmax;
    float4 *o = blk + ((size_t)b * NN + i) * 4;
    const int km = b * kBlk + kBlk / 2;
    if (km >= n) {
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        o[0] = z; o[1] = z; o[2] = z; o[3] = z;
        return;
    }
    const int k0 = b * kBlk, ke = min(b * kBlk + kBlk, n - 1);
    auto at = [&](int k, int f) { return t64[((size_t)k * 12 + f) * NN + i]; };
    const double h = kStepMyr;
    // velocity and acceleration at km in FP32: the tube is measured against the stored values themselves
    const int kp = min(km + 1, n - 1), kq = km - 1;
    float v32[3], a32[3];
    for (int c = 0; c < 3; c++) {
        v32[c] = (float)at(km, 3 + c);
        a32[c] = (float)((at(kq, 3 + c) - at(kp, 3 + c)) / ((double)(kp - kq) * h));
    }
    const double pm[3] = {at(km, 0), at(km, 1), at(km, 2)};
    double e2 = 0.0;
    for (int k = k0; k <= ke; k++) {
        const double tau = (double)(km - k) * h;
        double s = 0.0;
        for (int c = 0; c < 3; c++) {
            const double d = at(k, c) - pm[c] - (double)v32[c] * tau - 0.5 * (double)a32[c] * tau * tau;
            s += d * d;
        }
        e2 = fmax(e2, s);
    }
    const double an = sqrt((double)a32[0] * a32[0] + (double)a32[1] * a32[1] + (double)a32[2] * a32[2]);
    // the residual (FP64: rounding far below the margins), and the chords between points, a h^2 / 8
    const double eps = sqrt(e2) * (1.0 + 1e-12) + 1e-13 + 0.125 * an * h * h * (1.0 + 1e-12);
    // covariance: S(ke) dominates the range after delta >= the largest eigenvalue of S(k) - S(ke) is added
    const double r2 = R2 ? R2[i] : 0.0;
    double Se[6];
    for (int q = 0; q < 6; q++) Se[q] = at(ke, 6 + q);
    Se[0] += r2; Se[3] += r2; Se[5] += r2;
    // delta: a bound on the largest eigenvalue of S(k) - S(ke) over the range (Gershgorin: the largest diagonal entry
    // plus its row's off-diagonal magnitudes, rounding included), and k*, the point where it is largest
    double delta = 0.0;
    int kstar = -1;
    float lam_lo = __int_as_float(0x7f800000);
    for (int k = k0; k <= ke; k++) {
        if (k < ke) {
            double D[6];
            for (int q = 0; q < 6; q++) D[q] = at(k, 6 + q) - at(ke, 6 + q);
            const double g0 = D[0] + fabs(D[1]) + fabs(D[2]), g1 = D[3] + fabs(D[1]) + fabs(D[4]),
                         g2 = D[5] + fabs(D[2]) + fabs(D[4]);
            const double up = fmax(g0, fmax(g1, g2)) * (1.0 + 1e-12);
            if (up > delta) { delta = up; kstar = k; }
        }
        lam_lo = fminf(lam_lo, lm[(size_t)k * NN + i]);
    }
    double mxe = 0.0;
    for (int q = 0; q < 6; q++) mxe = fmax(mxe, fabs(Se[q]));
    // or S(ke) + alpha u u^T + beta I: the needle-thin covariances turn and shrink along the track, so S(k) - S(ke)
    // is positive mostly along one direction u (where the needle was), and delta I inflates the thin axes by many
    // times their size.  With u the top eigenvector of S(k*) - S(ke) and (u, w1, w2) an orthonormal basis, each
    // D = S(k) - S(ke) rotated into it: beta >= the largest eigenvalue of its (w1, w2) block over the range, and then
    // alpha >= the Schur complement's need, b^T C^-1 b - a for B = beta' I - D written as [a b^T; b C], makes
    // alpha u u^T + B positive semidefinite at every k, so S(ke) + alpha u u^T + beta' I dominates S(k).  Kept when
    // beta is under half of delta (the thin axes grow by beta instead of delta).  Its FP64 roundings are relative to
    // the entries, far below the FP32 storage margin r below.
    bool rank1 = false;
    double al = 0.0, be = 0.0, u[3] = {0.0, 0.0, 0.0};
    if (kstar >= 0) {
        double D[6];
        for (int q = 0; q < 6; q++) D[q] = at(kstar, 6 + q) - at(ke, 6 + q);
        const double lt = -sym3_min_eig_lb(-D[0], -D[1], -D[2], -D[3], -D[4], -D[5]);   // ~ its top eigenvalue
        // the eigenvector: the largest cross product of two rows of D - lt I
        const double R0[3] = {D[0] - lt, D[1], D[2]}, R1[3] = {D[1], D[3] - lt, D[4]}, R2r[3] = {D[2], D[4], D[5] - lt};
        auto cross = [](const double *x, const double *y, double *z) {
            z[0] = x[1] * y[2] - x[2] * y[1]; z[1] = x[2] * y[0] - x[0] * y[2]; z[2] = x[0] * y[1] - x[1] * y[0];
        };
        double c0[3], c1[3], c2[3];
        cross(R0, R1, c0); cross(R0, R2r, c1); cross(R1, R2r, c2);
        const double n0 = c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2];
        const double n1 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
        const double n2 = c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2];
        const double *cb = n0 >= n1 && n0 >= n2 ? c0 : (n1 >= n2 ? c1 : c2);
        const double nb = fmax(n0, fmax(n1, n2));
        if (lt > 0.0 && nb > 0.0) {
            const double inv = 1.0 / sqrt(nb);
            u[0] = cb[0] * inv; u[1] = cb[1] * inv; u[2] = cb[2] * inv;
            const double e0[3] = {1.0, 0.0, 0.0}, e1[3] = {0.0, 1.0, 0.0};
            double w1[3], w2[3];
            cross(u, fabs(u[0]) < 0.9 ? e0 : e1, w1);
            const double iw = 1.0 / sqrt(w1[0] * w1[0] + w1[1] * w1[1] + w1[2] * w1[2]);
            w1[0] *= iw; w1[1] *= iw; w1[2] *= iw;
            cross(u, w1, w2);
            // each D rotated into (u, w1, w2): its entries x^T D y
            double du_[kBlk], dw11[kBlk], dw12[kBlk], dw22[kBlk], duw1[kBlk], duw2[kBlk];
            const int nk = ke - k0;                       // <= kBlk: ke <= k0 + kBlk
            for (int j = 0; j < nk; j++) {
                double Dk[6];
                for (int q = 0; q < 6; q++) Dk[q] = at(k0 + j, 6 + q) - at(ke, 6 + q);
                double Du[3], Dw1[3];                     // D u, D w1
                Du[0] = Dk[0] * u[0] + Dk[1] * u[1] + Dk[2] * u[2];
                Du[1] = Dk[1] * u[0] + Dk[3] * u[1] + Dk[4] * u[2];
                Du[2] = Dk[2] * u[0] + Dk[4] * u[1] + Dk[5] * u[2];
                Dw1[0] = Dk[0] * w1[0] + Dk[1] * w1[1] + Dk[2] * w1[2];
                Dw1[1] = Dk[1] * w1[0] + Dk[3] * w1[1] + Dk[4] * w1[2];
                Dw1[2] = Dk[2] * w1[0] + Dk[4] * w1[1] + Dk[5] * w1[2];
                const double Dw2_2 = Dk[2] * w2[0] + Dk[4] * w2[1] + Dk[5] * w2[2];
                const double Dw2_0 = Dk[0] * w2[0] + Dk[1] * w2[1] + Dk[2] * w2[2];
                const double Dw2_1 = Dk[1] * w2[0] + Dk[3] * w2[1] + Dk[4] * w2[2];
                du_[j] = u[0] * Du[0] + u[1] * Du[1] + u[2] * Du[2];
                duw1[j] = w1[0] * Du[0] + w1[1] * Du[1] + w1[2] * Du[2];
                duw2[j] = w2[0] * Du[0] + w2[1] * Du[1] + w2[2] * Du[2];
                dw11[j] = w1[0] * Dw1[0] + w1[1] * Dw1[1] + w1[2] * Dw1[2];
                dw12[j] = w2[0] * Dw1[0] + w2[1] * Dw1[1] + w2[2] * Dw1[2];
                dw22[j] = w2[0] * Dw2_0 + w2[1] * Dw2_1 + w2[2] * Dw2_2;
                const double h = 0.5 * (dw11[j] - dw22[j]);
                be = fmax(be, 0.5 * (dw11[j] + dw22[j]) + sqrt(h * h + dw12[j] * dw12[j]));
            }
            be = be * (1.0 + 1e-6) + 1e-9 * mxe;
            bool ok = true;
            for (int j = 0; j < nk; j++) {
                // B = be I - D in the basis: a = be - D_uu, b = -D_uw, C = be I - D_ww
                const double a = be - du_[j], b1 = -duw1[j], b2 = -duw2[j];
                const double c11 = be - dw11[j], c12 = -dw12[j], c22 = be - dw22[j];
                const double det = c11 * c22 - c12 * c12;
                if (!(c11 > 0.0 && det > 0.0)) { ok = false; break; }
                al = fmax(al, (c22 * b1 * b1 - 2.0 * c12 * b1 * b2 + c11 * b2 * b2) / det - a);
            }
            if (ok) {
                al = al * (1.0 + 1e-6) + 1e-9 * mxe;
                rank1 = be < 0.5 * delta;
            }
        }
    }
    // the chosen matrix plus r I, rounded to FP32: each entry's rounding is within 2^-24 of its magnitude, so the
    // rounding error E has ||E|| <= 3 * 2^-24 (mx + r) < r: the stored matrix still dominates it
    double Sd[6];
    if (rank1) {
        Sd[0] = Se[0] + al * u[0] * u[0] + be; Sd[1] = Se[1] + al * u[0] * u[1]; Sd[2] = Se[2] + al * u[0] * u[2];
        Sd[3] = Se[3] + al * u[1] * u[1] + be; Sd[4] = Se[4] + al * u[1] * u[2]; Sd[5] = Se[5] + al * u[2] * u[2] + be;
    } else {
        Sd[0] = Se[0] + delta; Sd[1] = Se[1]; Sd[2] = Se[2];
        Sd[3] = Se[3] + delta; Sd[4] = Se[4]; Sd[5] = Se[5] + delta;
    }
    double mx = 0.0;
    for (int q = 0; q < 6; q++) mx = fmax(mx, fabs(Sd[q]));
    const double r = 4.0 * 5.9604644775390625e-8 * mx;
    Sd[0] += r; Sd[3] += r; Sd[5] += r;
    const float lam = __double2float_rd((double)lm[(size_t)ke * NN + i] + (rank1 ? be : delta));
    o[0] = make_float4(v32[0], v32[1], v32[2], __double2float_ru(eps));
    o[1] = make_float4(a32[0], a32[1], a32[2], lam);
    o[2] = make_float4((float)Sd[0], (float)Sd[1], (float)Sd[2], (float)Sd[3]);
    o[3] = make_float4((float)Sd[4], (float)Sd[5], lam_lo, 0.f);
}

int block_tables(cudaStream_t st, int N, int nmax, const int *npts, const double *t64, const float *lm,
                 const double *R2, float4 *blk, std::string &err) {
    const size_t work = (size_t)N * ((nmax + kBlk - 1) / kBlk);
    if (work == 0) return 0;
    k_block_tables<<<(unsigned)((work + 127) / 128), 128, 0, st>>>(N, nmax, npts, t64, lm, R2, blk);
    return check(cudaGetLastError(), err, "k_block_tables");
}

// The cluster table cluster-major for the staged filter: one cluster's block-table column, FP32 track and lambda
// bounds each contiguous (the bulk copies move contiguous ranges), lambda rows padded to lm_pitch (a multiple of 4).
__global__ void k_cluster_major(int nc, int ncp, int nblk, int lm_pitch, const float4 *__restrict__ blk,
                                const float4 *__restrict__ c32, const float *__restrict__ lm, float4 *__restrict__ blk_cm,
                                float4 *__restrict__ c32_cm, float *__restrict__ lm_cm) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int rows = ncp > nblk ? ncp : nblk;
    if (idx >= (size_t)nc * rows) return;
    const int c = (int)(idx % nc), k = (int)(idx / nc);
    if (k < nblk)
        for (int q = 0; q < 4; q++) blk_cm[((size_t)c * nblk + k) * 4 + q] = blk[((size_t)k * nc + c) * 4 + q];
    if (k < ncp) {
        for (int q = 0; q < 3; q++) c32_cm[((size_t)c * ncp + k) * 3 + q] = c32[((size_t)k * nc + c) * 3 + q];
        lm_cm[(size_t)c * lm_pitch + k] = lm[(size_t)k * nc + c];
    }
}

int cluster_major(cudaStream_t st, int nc, int ncp, int nblk, int lm_pitch, const float4 *blk, const float4 *c32,
                  const float *lm, float4 *blk_cm, float4 *c32_cm, float *lm_cm, std::string &err) {
    const size_t work = (size_t)nc * (ncp > nblk ? ncp : nblk);
    k_cluster_major<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(nc, ncp, nblk, lm_pitch, blk, c32, lm, blk_cm,
                                                                    c32_cm, lm_cm);
    return check(cudaGetLastError(), err, "k_cluster_major");
}

// separation of star and cluster at one point from the split FP32 positions
__device__ __forceinline__ void sep32(const float4 &t0, const float4 &t1, const float4 &c0, const float4 &c1,
                                      float (&m)[3]) {
    m[0] = (t0.x - c0.x) + (t0.w - c0.w);
    m[1] = (t0.y - c0.y) + (t1.x - c1.x);
    m[2] = (t0.z - c0.z) + (t1.y - c1.y);
}

// ---- K1: FP32 filter over every pair -------------------------------------------------------------------------
// A point k can be the FP64 minimum of a kept pair only if lb_k < cut and lb_k <= min_j ub_j (otherwise some point
// is certainly lower, or none is under the cut): the pair's candidates.  The walk keeps them in kCandSlots slots:
// the running min ub only decreases, so a point that qualifies at the end qualified when it was walked, and a slot
// whose lb has risen above the running min ub is free again.  Per pair: flag[c][s] = 0 (no candidate: the pair
// cannot be kept), 1 (its candidates are in klist[c][s], kCandSlots 16-bit point numbers, 0xffff = empty) or 2 (more
// candidates than slots, or a point number that does not fit 16 bits: the candidates are found again by a second
// walk, which needs ubmin[c][s]).  A slot is taken while its lb is under the cut (empty slots hold +inf) and not
// above the running min ub.  ubmin and klist are written for flagged pairs only.
constexpr int kCandSlots = 4;
constexpr unsigned kNoPoint = 0xffffu;
constexpr int kScanStars = 128;         // stars per block (one per thread)
constexpr int kQueue = 64;              // per warp: points waiting for their full bounds

// The full bounds of point k of pair (s, c), for a point the skip test did not settle: false when rejected.
__device__ __forceinline__ bool point_at32(const ScreenTables &T, int s, int c, int k, float cut, Bound &b) {
    const size_t NT = T.nt, NC = T.nc;
    const int n = T.ns < T.cn[c] ? T.ns : T.cn[c];
    const bool more = k + 1 < n;
    const float4 *tp = T.t32 + ((size_t)k * NT + s) * 3, *cp = T.c32 + ((size_t)k * NC + c) * 3;
    const float4 t0 = tp[0], t1 = tp[1], t2 = tp[2];
    const float4 c0 = __ldg(cp), c1 = __ldg(cp + 1), c2 = __ldg(cp + 2);
    float m0[3], m1[3];
    sep32(t0, t1, c0, c1, m0);
    if (more) {
        const float4 *tn = tp + NT * 3, *cn = cp + NC * 3;
        sep32(tn[0], tn[1], __ldg(cn), __ldg(cn + 1), m1);
    } else {
        m1[0] = m0[0]; m1[1] = m0[1]; m1[2] = m0[2];
    }
    const float St[6] = {t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
    const float Sc[6] = {c1.z, c1.w, c2.x, c2.y, c2.z, c2.w};
    return point_bound32(St, Sc, T.lm_t[(size_t)k * NT + s], __ldg(T.lm_c + (size_t)k * NC + c), m0, m1,
                         more, cut, b);
}

// One block: kScanStars stars x one cluster; a warp walks its 32 pairs' points in step.  Clusters are the grid's fast
// axis, so the blocks resident at one time share one block of stars, whose track data stays in L2.
// Each lane runs the cheap test (point_skip32) on its point; the few points it cannot settle are queued per warp in
// shared memory and given their full bounds 32 at a time, one per lane, so the long evaluation runs on full warps
// instead of diverging on most steps; the owner lane then folds the results into its pair's state.  The state (min
// ub and the candidate slots) does not depend on the order the points are folded in.
// six resident blocks per SM asked of the compiler (80 registers, a 4-byte spill): 24 warps to issue from, where 95
// registers left 20; the kernel is issue-bound and runs 7 % faster so (5, 7 and 8 blocks measured slower)
__global__ void __launch_bounds__(kScanStars, 6) k_mx_scan32(ScreenTables T, float cut,
                                                             unsigned char *__restrict__ flag,
                                                             float *__restrict__ ubmin,
                                                             unsigned long long *__restrict__ klist) {
    __shared__ int s_q[kScanStars / 32][kQueue];
    __shared__ float s_lb[kScanStars / 32][32], s_ub[kScanStars / 32][32];
    __shared__ unsigned s_own[kScanStars / 32][32];                // per owner lane: its entries of the drain
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, c = blockIdx.x;
    const int s0 = blockIdx.y * kScanStars + w * 32;
    if (s0 >= T.nt) return;                                       // the whole warp: uniform
    const bool active = s0 + lane < T.nt;
    const int s = active ? s0 + lane : T.nt - 1;                  // lanes past the end shadow a valid star
    const float inf = __int_as_float(0x7f800000);
    float um = inf, ls[kCandSlots];
    unsigned kq[kCandSlots];
#pragma unroll
    for (int i = 0; i < kCandSlots; i++) { ls[i] = inf; kq[i] = kNoPoint; }
    bool over = false;
    auto fold = [&](int k, float lb, float ub) {
        um = fminf(um, ub);
        if (lb < cut && lb <= um) {
            bool placed = false;
#pragma unroll
            for (int i = 0; i < kCandSlots; i++)
                if (!placed && !(ls[i] < cut && ls[i] <= um)) { ls[i] = lb; kq[i] = (unsigned)k; placed = true; }
            over |= !placed || k >= (int)kNoPoint;
        }
    };
    // full bounds for queue entries [0, cnt) (an entry is owner lane | k << 5), one per lane; then each owner lane
    // folds its own entries, found from a bit mask per owner, in queue order (the order it queued them in)
    auto drain = [&](int cnt) {
        __syncwarp();
        s_own[w][lane] = 0u;
        __syncwarp();
        if (lane < cnt) {
            const int e = s_q[w][lane];
            Bound b;
            const bool keep = point_at32(T, s0 + (e & 31), c, e >> 5, cut, b);
            s_lb[w][lane] = keep ? b.lb : inf;
            s_ub[w][lane] = keep ? b.ub : inf;
            atomicOr(&s_own[w][e & 31], 1u << lane);
        }
        __syncwarp();
        for (unsigned mine = s_own[w][lane]; mine; mine &= mine - 1u) {
            const int j = __ffs(mine) - 1;
            fold(s_q[w][j] >> 5, s_lb[w][j], s_ub[w][j]);
        }
        __syncwarp();
    };
    const size_t NT = T.nt, NC = T.nc;
    const int n = T.ns < T.cn[c] ? T.ns : T.cn[c];
    const float4 *tp = T.t32 + (size_t)s * 3, *cp = T.c32 + (size_t)c * 3;
    float4 t0 = tp[0], t1 = tp[1], t2 = tp[2];
    float4 c0 = __ldg(cp), c1 = __ldg(cp + 1), c2 = __ldg(cp + 2);
    float mcur[3];
    sep32(t0, t1, c0, c1, mcur);
    int qn = 0;
    for (int k = 0; k < n; k++) {
        const float St[6] = {t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
        const float Sc[6] = {c1.z, c1.w, c2.x, c2.y, c2.z, c2.w};
        const float lmt = T.lm_t[(size_t)k * NT + s], lmc = __ldg(T.lm_c + (size_t)k * NC + c);
        float mnext[3] = {mcur[0], mcur[1], mcur[2]};
        if (k + 1 < n) {
            const float4 *tn = tp + (size_t)(k + 1) * NT * 3, *cn = cp + (size_t)(k + 1) * NC * 3;
            t0 = tn[0]; t1 = tn[1]; t2 = tn[2];
            c0 = __ldg(cn); c1 = __ldg(cn + 1); c2 = __ldg(cn + 2);
            sep32(t0, t1, c0, c1, mnext);
        }
        const bool need = active && !point_skip32(St, Sc, lmt, lmc, mcur, mnext, cut);
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        if (need) s_q[w][qn + __popc(mask & ((1u << lane) - 1u))] = lane | (k << 5);
        qn += __popc(mask);
        if (qn >= 32) {
            drain(32);
            const int rest = qn - 32;
            const int v = lane < rest ? s_q[w][32 + lane] : 0;
            __syncwarp();
            if (lane < rest) s_q[w][lane] = v;
            qn = rest;
        }
        mcur[0] = mnext[0]; mcur[1] = mnext[1]; mcur[2] = mnext[2];
    }
    if (qn > 0) drain(qn);
    if (!active) return;
    unsigned long long kl = 0;
    bool any = false;
#pragma unroll
    for (int i = 0; i < kCandSlots; i++) {
        const bool live = ls[i] < cut && ls[i] <= um;
        any |= live;
        kl |= (unsigned long long)(live ? kq[i] : kNoPoint) << (16 * i);
    }
    const size_t o = (size_t)c * NT + s;
    flag[o] = over ? 2 : (any ? 1 : 0);
    if (over || any) {
        ubmin[o] = um;
        klist[o] = kl;
    }
}

// a cluster value: from shared memory (staged) or through the read-only cache
template <bool STAGE, class V> __device__ __forceinline__ V ldc(const V *p) {
    if (STAGE) return *p;
    return __ldg(p);
}

// The bulk copies of one cluster's data into shared memory on an mbarrier, and the wait for them.  The wait is
// bounded: should it ever run out, the CTA records it in T.wait_err (the host turns that into an error), waits once
// more, bounded too, for its copies in flight, and reports false (the CTA then returns without output).
__device__ bool stage_cluster(const ScreenTables &T, int c, float4 *sb, float4 *sc, float *sl, uint64_t *bar) {
    const unsigned ab = (unsigned)__cvta_generic_to_shared(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ab) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int n = T.cn[c];
        const unsigned b1 = (unsigned)T.nblk * 64u, b2 = (unsigned)n * 48u, b3 = ((unsigned)n * 4u + 15u) & ~15u;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ab), "r"(b1 + b2 + b3)
                     : "memory");
        const void *g1 = T.blk_cm + (size_t)c * T.nblk * 4, *g2 = T.c32_cm + (size_t)c * T.ncp * 3;
        const void *g3 = T.lm_cm + (size_t)c * T.lm_pitch;
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"((unsigned)__cvta_generic_to_shared(sb)), "l"(g1), "r"(b1), "r"(ab) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"((unsigned)__cvta_generic_to_shared(sc)), "l"(g2), "r"(b2), "r"(ab) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"((unsigned)__cvta_generic_to_shared(sl)), "l"(g3), "r"(b3), "r"(ab) : "memory");
    }
    auto wait = [&]() {
        for (int it = 0; it < (1 << 22); it++) {
            unsigned ok;
            asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                         : "=r"(ok) : "r"(ab) : "memory");
            if (ok) return true;
        }
        return false;
    };
    if (wait()) return true;
    if (T.wait_err) atomicExch(T.wait_err, 1);
    wait();
    return false;
}

// the full bounds of a point, out of line (the block kernel's single copy of point_bound32)
__device__ __noinline__ bool point_at32_ol(const ScreenTables *T, int s, int c, int k, float cut, Bound *b) {
    return point_at32(*T, s, c, k, cut, *b);
}

// k_mx_scan32 with block culling.  One block: kScanStars stars x one cluster; a warp walks its 32 pairs in step.
// Clusters are the grid's fast axis, so the blocks resident at one time share one block of stars, whose track data
// stays in L2.
// The walk has two levels.  First a block test per lane (block_skip32, with the block tables): one test settles the
// eight points of a block -- most blocks of most pairs.  The blocks it cannot settle are queued per warp in shared
// memory and walked 32 at a time, one per lane (different pairs and blocks), point by point: each point gets the
// cheap point test (point_skip32), and the few points it cannot settle either are queued again, per warp, for their
// full bounds, 32 at a time on full warps.  The owner lane of each point then folds the results into its pair's state
// (min ub and the candidate slots), which does not depend on the order the points are folded in.  Points past the
// last testable block (fewer than five left) are walked by every lane in step, as are all points when the tables
// have no block data.  A settled block's points all have chi2 >= cut in the FP64 path: they can neither be a kept
// pair's minimum nor bring a pair under the cut, and they are left out of min ub, which only admits more candidates.
// Once a pair's min ub is below the cut, blocks and points are settled against it instead (strictly above another
// point's FP64 value: not the minimum), so a kept pair's points after its minimum mostly need no full bounds.
// six resident blocks per SM asked of the compiler: 24 warps to issue from; the kernel is issue-bound
template <int MINB, bool STAGE>
__global__ void __launch_bounds__(kScanStars, MINB) k_mx_scan32_blocks(const __grid_constant__ ScreenTables T,
                                                                      float cut, unsigned char *__restrict__ flag,
                                                                      float *__restrict__ ubmin,
                                                                      unsigned long long *__restrict__ klist) {
    // STAGE: this CTA's cluster -- its block-table column, its FP32 track and its lambda bounds, contiguous in the
    // cluster-major copies -- comes into shared memory by three bulk copies (TMA, cp.async.bulk) on one mbarrier;
    // the filter then reads the cluster from there instead of through the L1 cache
    extern __shared__ __align__(128) unsigned char s_dyn[];
    __shared__ __align__(8) uint64_t s_bar;
    const float4 *cblk = T.blk_c + (size_t)blockIdx.x * 4, *cc32 = T.c32 + (size_t)blockIdx.x * 3;
    const float *clm = T.lm_c + blockIdx.x;
    size_t cbs = (size_t)T.nc * 4, ccs = (size_t)T.nc * 3, cls = T.nc;         // strides between points / blocks
    if (STAGE) {
        float4 *sb = reinterpret_cast<float4 *>(s_dyn), *sc = sb + (size_t)T.nblk * 4;
        float *sl = reinterpret_cast<float *>(sc + (size_t)T.ncp * 3);
        if (!stage_cluster(T, blockIdx.x, sb, sc, sl, &s_bar)) return;
        cblk = sb; cc32 = sc; clm = sl;
        cbs = 4; ccs = 3; cls = 1;
    }
    __shared__ int s_q[kScanStars / 32][kQueue];                  // points waiting for their full bounds
    __shared__ int s_bq[kScanStars / 32][kQueue];                 // blocks waiting to be walked point by point
    __shared__ float s_lb[kScanStars / 32][32], s_ub[kScanStars / 32][32];
    __shared__ unsigned s_own[kScanStars / 32][32];                // per owner lane: its entries of the drain
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, c = blockIdx.x;
    const int s0 = blockIdx.y * kScanStars + w * 32;
    if (s0 >= T.nt) return;                                       // the whole warp: uniform
    const bool active = s0 + lane < T.nt;
    const int s = active ? s0 + lane : T.nt - 1;                  // lanes past the end shadow a valid star
    const float inf = __int_as_float(0x7f800000);
    float um = inf, ls[kCandSlots];
    unsigned kq[kCandSlots];
#pragma unroll
    for (int i = 0; i < kCandSlots; i++) { ls[i] = inf; kq[i] = kNoPoint; }
    bool over = false;
    auto fold = [&](int k, float lb, float ub) {
        um = fminf(um, ub);
        if (lb < cut && lb <= um) {
            bool placed = false;
#pragma unroll
            for (int i = 0; i < kCandSlots; i++)
                if (!placed && !(ls[i] < cut && ls[i] <= um)) { ls[i] = lb; kq[i] = (unsigned)k; placed = true; }
            over |= !placed || k >= (int)kNoPoint;
        }
    };
    // full bounds for queue entries [0, cnt) (an entry is owner lane | k << 5), one per lane; then each owner lane
    // folds its own entries, found from a bit mask per owner, in queue order (the order it queued them in)
    auto drain = [&](int cnt) {
        __syncwarp();
        s_own[w][lane] = 0u;
        __syncwarp();
        if (lane < cnt) {
            const int e = s_q[w][lane];
            Bound b;
            const bool keep = point_at32_ol(&T, s0 + (e & 31), c, e >> 5, cut, &b);
            s_lb[w][lane] = keep ? b.lb : inf;
            s_ub[w][lane] = keep ? b.ub : inf;
            atomicOr(&s_own[w][e & 31], 1u << lane);
        }
        __syncwarp();
        for (unsigned mine = s_own[w][lane]; mine; mine &= mine - 1u) {
            const int j = __ffs(mine) - 1;
            fold(s_q[w][j] >> 5, s_lb[w][j], s_ub[w][j]);
        }
        __syncwarp();
    };
    int qn = 0;
    // every lane in step: its entry (owner | k << 5) when `need`, draining 32 at a time
    auto push_point = [&](bool need, int entry) {
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        if (need) s_q[w][qn + __popc(mask & ((1u << lane) - 1u))] = entry;
        qn += __popc(mask);
        if (qn >= 32) {
            drain(32);
            const int rest = qn - 32;
            const int v = lane < rest ? s_q[w][32 + lane] : 0;
            __syncwarp();
            if (lane < rest) s_q[w][lane] = v;
            qn = rest;
        }
    };
    // A point or block whose lower bound is >= thr needs nothing more: thr = cut (it can be neither under the cut nor
    // the minimum of a kept pair), or just above the pair's min ub so far (its FP64 value is then strictly above
    // another point's: not the minimum, ties included).  Either way it is left out of min ub, which only admits more
    // candidates.  The pair's min ub falls as its points' full bounds are folded in, so blocks and points walked
    // after its minimum are mostly settled against it.
    auto pair_thr = [&]() { return fminf(cut, fmaxf(um * (1.f + 1e-6f), 1e-30f)); };
    const size_t NT = T.nt;
    const int n = T.ns < T.cn[c] ? T.ns : T.cn[c];
    // the point test of point k of star st's pair (its separations at k and k + 1 in mc / mn), as every walk runs it
    auto point_needs = [&](int st, int k, const float4 &t1, const float4 &t2, const float4 &c1, const float4 &c2,
                           const float (&mc)[3], const float (&mn)[3], float thr) {
        const float St[6] = {t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
        const float Sc[6] = {c1.z, c1.w, c2.x, c2.y, c2.z, c2.w};
        const float lmt = T.lm_t[(size_t)k * NT + st], lmc = ldc<STAGE>(clm + (size_t)k * cls);
        return !point_skip32(St, Sc, lmt, lmc, mc, mn, thr);
    };
    // ---- level 1: blocks of kBlk points whose position reference km = kBlk b + kBlk/2 lies on the pair's track
    const int nbt = n > kBlk / 2 ? (n - kBlk / 2 - 1) / kBlk + 1 : 0;
    {
        // walk the queued blocks [0, cnt) point by point, one block per lane
        auto walk_blocks = [&](int cnt) {
            __syncwarp();
            const int e = lane < cnt ? s_bq[w][lane] : 0;
            const int o = e & 31, b = e >> 5, st = s0 + o;
            const float thr = __shfl_sync(0xffffffffu, pair_thr(), o);    // the owner's threshold at this walk
            const int k0 = b * kBlk, k1 = min(k0 + kBlk, n);
            const float4 *tp = T.t32 + (size_t)st * 3;
            float4 t0, t1, t2, c0, c1, c2;
            float mc[3] = {0.f, 0.f, 0.f};
            if (lane < cnt) {
                const float4 *a = tp + (size_t)k0 * NT * 3, *q = cc32 + (size_t)k0 * ccs;
                t0 = a[0]; t1 = a[1]; t2 = a[2];
                c0 = ldc<STAGE>(q); c1 = ldc<STAGE>(q + 1); c2 = ldc<STAGE>(q + 2);
                sep32(t0, t1, c0, c1, mc);
            }
            for (int j = 0; j < kBlk; j++) {
                const int k = k0 + j;
                const bool valid = lane < cnt && k < k1;
                bool need = false;
                if (valid) {
                    const float4 T1 = t1, T2 = t2, C1 = c1, C2 = c2;
                    float mn[3] = {mc[0], mc[1], mc[2]};
                    if (k + 1 < n) {
                        const float4 *a = tp + (size_t)(k + 1) * NT * 3, *q = cc32 + (size_t)(k + 1) * ccs;
                        t0 = a[0]; t1 = a[1]; t2 = a[2];
                        c0 = ldc<STAGE>(q); c1 = ldc<STAGE>(q + 1); c2 = ldc<STAGE>(q + 2);
                        sep32(t0, t1, c0, c1, mn);
                    }
                    need = point_needs(st, k, T1, T2, C1, C2, mc, mn, thr);
                    mc[0] = mn[0]; mc[1] = mn[1]; mc[2] = mn[2];
                }
                push_point(need, o | (k << 5));
            }
        };
        int bn = 0;
        const float4 *bt = T.blk_t + (size_t)s * 4;
        // blocks 0 .. nbt-1 get the test; block nbt, the points after them (fewer than five), is walked untested;
        // the last pass tests nothing and walks what is left (one call site keeps the kernel's code small)
        const int kt = nbt * kBlk, nball = nbt + (kt < n ? 1 : 0);
        for (int b = 0; b <= nball; b++) {
            bool need = false;
            if (b < nbt && active) {
                const int km = b * kBlk + kBlk / 2;
                const float4 *a = bt + (size_t)b * NT * 4, *q = cblk + (size_t)b * cbs;
                const float4 BT[4] = {a[0], a[1], a[2], a[3]};
                const float4 BC[4] = {ldc<STAGE>(q), ldc<STAGE>(q + 1), ldc<STAGE>(q + 2), ldc<STAGE>(q + 3)};
                const float4 *tm = T.t32 + ((size_t)km * NT + s) * 3, *cm = cc32 + (size_t)km * ccs;
                float mref[3];
                sep32(tm[0], tm[1], ldc<STAGE>(cm), ldc<STAGE>(cm + 1), mref);
                need = !block_skip32(BT, BC, mref, pair_thr());
            } else if (b < nball) {
                need = active;
            }
            const unsigned mask = __ballot_sync(0xffffffffu, need);
            if (need) s_bq[w][bn + __popc(mask & ((1u << lane) - 1u))] = lane | (b << 5);
            bn += __popc(mask);
            if (bn >= 32 || (b == nball && bn > 0)) {
                const int cnt = min(bn, 32);
                walk_blocks(cnt);
                const int rest = bn - cnt;
                const int v = lane < rest ? s_bq[w][cnt + lane] : 0;
                __syncwarp();
                if (lane < rest) s_bq[w][lane] = v;
                bn = rest;
            }
        }
    }
    if (qn > 0) drain(qn);
    if (!active) return;
    unsigned long long kl = 0;
    bool any = false;
#pragma unroll
    for (int i = 0; i < kCandSlots; i++) {
        const bool live = ls[i] < cut && ls[i] <= um;
        any |= live;
        kl |= (unsigned long long)(live ? kq[i] : kNoPoint) << (16 * i);
    }
    const size_t o = (size_t)c * NT + s;
    flag[o] = over ? 2 : (any ? 1 : 0);
    if (over || any) {
        ubmin[o] = um;
        klist[o] = kl;
    }
}

// ---- multi-block exclusive scan of int counts --------------------------------------------------------------------
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int block_incl_scan(int v, int *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += t;
    }
    if (lane == 31) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        int x = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += t;
        }
        sh[lane] = x;
    }
    __syncthreads();
    if (w > 0) v += sh[w - 1];
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_partials(int n, const int *__restrict__ in, int *__restrict__ part) {
    __shared__ int sh[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    const int incl = block_incl_scan(v, sh);
    if (threadIdx.x == kScanBlock - 1) part[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_top(int nb, int *__restrict__ part, int *__restrict__ total) {
    __shared__ int sh[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? part[i] : 0;
        const int incl = block_incl_scan(v, sh);
        if (i < nb) part[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_apply(int n, const int *__restrict__ in,
                                                           const int *__restrict__ part, int *__restrict__ out) {
    __shared__ int sh[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    const int incl = block_incl_scan(v, sh);
    if (i < n) out[i] = part[blockIdx.x] + incl - v;
}

// exclusive scan of n ints into out, total into *total (device); part: ceil(n / 1024) ints of scratch
int exclusive_scan(cudaStream_t st, int n, const int *in, int *out, int *part, int *total, std::string &err) {
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    if (n <= 0) return check(cudaMemsetAsync(total, 0, 4, st), err, "scan total");
    k_scan_partials<<<nb, kScanBlock, 0, st>>>(n, in, part);
    k_scan_top<<<1, kScanBlock, 0, st>>>(nb, part, total);
    k_scan_apply<<<nb, kScanBlock, 0, st>>>(n, in, part, out);
    return check(cudaGetLastError(), err, "scan");
}

// ---- K2: possible pairs in (star, cluster) order --------------------------------------------------------------
struct PossPair {
    int s, c;
    float ubmin;
    int over;                     // 1: more candidates than slots (found again by a walk)
    unsigned long long klist;     // the candidate slots, as k_mx_scan32 left them
};

// A star's clusters are split into kEmitGroups contiguous ranges, one thread per (star, range) (grid y = range), so
// that a part of a few thousand stars still fills the GPU.  Counts and offsets are indexed s * kEmitGroups + g: the
// scan over them is in (star, cluster) order.
constexpr int kEmitGroups = 16;

__device__ __forceinline__ void emit_range(int nc, int g, int &c0, int &c1) {
    const int len = (nc + kEmitGroups - 1) / kEmitGroups;
    c0 = min(nc, g * len);
    c1 = min(nc, c0 + len);
}

__global__ void k_mx_count(int nt, int nc, const unsigned char *__restrict__ flag, int *__restrict__ npair) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
    if (s >= nt) return;
    int c0, c1;
    emit_range(nc, g, c0, c1);
    int a = 0;
    for (int c = c0; c < c1; c++) a += flag[(size_t)c * nt + s] != 0;
    npair[(size_t)s * kEmitGroups + g] = a;
}

__global__ void k_mx_emit(int nt, int nc, const unsigned char *__restrict__ flag, const float *__restrict__ ubmin,
                          const unsigned long long *__restrict__ klist, const int *__restrict__ opair,
                          PossPair *__restrict__ P) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
    if (s >= nt) return;
    int c0, c1;
    emit_range(nc, g, c0, c1);
    int p = opair[(size_t)s * kEmitGroups + g];
    for (int c = c0; c < c1; c++) {
        const size_t o = (size_t)c * nt + s;
        const int f = flag[o];
        if (!f) continue;
        PossPair r;
        r.s = s; r.c = c; r.ubmin = ubmin[o]; r.over = f == 2; r.klist = klist[o];
        P[p++] = r;
    }
}

// per possible pair: its number of listed candidates (0 for an overflowed pair, counted by its walk) and whether it
// overflowed
__global__ void k_mx_list_count(int np, const PossPair *__restrict__ P, int *__restrict__ cnt, int *__restrict__ ovf) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const PossPair r = P[p];
    int n = 0;
#pragma unroll
    for (int i = 0; i < kCandSlots; i++) n += ((r.klist >> (16 * i)) & 0xffffu) != kNoPoint;
    cnt[p] = r.over ? 0 : n;
    ovf[p] = r.over;
}

__global__ void k_mx_list_emit(int np, const PossPair *__restrict__ P, const int *__restrict__ off,
                               int2 *__restrict__ E) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const PossPair r = P[p];
    if (r.over) return;
    int e = off[p];
#pragma unroll
    for (int i = 0; i < kCandSlots; i++) {
        const unsigned k = (unsigned)(r.klist >> (16 * i)) & 0xffffu;
        if (k != kNoPoint) E[e++] = make_int2(p, (int)k);
    }
}

__global__ void k_mx_ovf_emit(int np, const int *__restrict__ ovf, const int *__restrict__ off, int *__restrict__ A) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np && ovf[p]) A[off[p]] = p;
}

// ---- K3: the overflowed pairs walked again for their candidate points, once -------------------------------------
// One warp per pair, lane j taking points j, j + 32, ...: each point gets the scan's tests (the cheap skip test, then
// the full bounds) and is a candidate when lb < cut and lb <= the pair's min ub.  A ballot numbers the candidates of
// each 32 points, so they are written in point order.
__device__ __forceinline__ bool point_cand32(const ScreenTables &T, int s, int c, int k, int n, float cut, float um) {
    const size_t NT = T.nt, NC = T.nc;
    const bool more = k + 1 < n;
    const float4 *tp = T.t32 + ((size_t)k * NT + s) * 3, *cp = T.c32 + ((size_t)k * NC + c) * 3;
    const float4 t0 = tp[0], t1 = tp[1], t2 = tp[2];
    const float4 c0 = __ldg(cp), c1 = __ldg(cp + 1), c2 = __ldg(cp + 2);
    float m0[3], m1[3];
    sep32(t0, t1, c0, c1, m0);
    if (more) {
        const float4 *tn = tp + NT * 3, *cn = cp + NC * 3;
        sep32(tn[0], tn[1], __ldg(cn), __ldg(cn + 1), m1);
    } else {
        m1[0] = m0[0]; m1[1] = m0[1]; m1[2] = m0[2];
    }
    const float St[6] = {t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
    const float Sc[6] = {c1.z, c1.w, c2.x, c2.y, c2.z, c2.w};
    const float lmt = T.lm_t[(size_t)k * NT + s], lmc = __ldg(T.lm_c + (size_t)k * NC + c);
    Bound b;
    // a point whose FP64 value is surely above the pair's min ub (strictly) is not its minimum: no candidate
    const float thr = fminf(cut, fmaxf(um * (1.f + 1e-6f), 1e-30f));
    return !point_skip32(St, Sc, lmt, lmc, m0, m1, thr) &&
           point_bound32(St, Sc, lmt, lmc, m0, m1, more, cut, b) && b.lb < cut && b.lb <= um;
}

constexpr int kCandWarps = 4;
constexpr int kCandCap = 64;            // candidates an overflowed pair keeps from its single walk

// The walk: the candidates' point numbers into X[i][0, kCandCap), their count into cnt[p]; a pair with more is
// listed in big[0, *nbig) (in any order) and walked again by k_mx_cand_big
__global__ void __launch_bounds__(kCandWarps * 32) k_mx_cand(ScreenTables T, float cut, int na,
                                                             const int *__restrict__ A,
                                                             const PossPair *__restrict__ P, int *__restrict__ cnt,
                                                             int *__restrict__ X, int *__restrict__ big,
                                                             int *__restrict__ nbig) {
    const int i = blockIdx.x * kCandWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= na) return;                                          // the whole warp: uniform
    const int p = A[i];
    const PossPair r = P[p];
    const int n = T.ns < T.cn[r.c] ? T.ns : T.cn[r.c];
    int e = 0;
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int k = k0 + lane;
        const bool hit = k < n && point_cand32(T, r.s, r.c, k, n, cut, r.ubmin);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        const int at = e + __popc(m & ((1u << lane) - 1u));
        if (hit && at < kCandCap) X[(size_t)i * kCandCap + at] = k;
        e += __popc(m);
    }
    if (lane == 0) {
        cnt[p] = e;
        if (e > kCandCap) big[atomicAdd(nbig, 1)] = i;
    }
}

// the kept candidates of the overflowed pairs into their places in E
__global__ void k_mx_cand_copy(int na, const int *__restrict__ A, const int *__restrict__ cnt,
                               const int *__restrict__ off, const int *__restrict__ X, int2 *__restrict__ E) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t / kCandCap), j = (int)(t % kCandCap);
    if (i >= na) return;
    const int p = A[i], n = cnt[p];
    if (n <= kCandCap && j < n) E[off[p] + j] = make_int2(p, X[(size_t)i * kCandCap + j]);
}

// the listed pairs with more than kCandCap candidates: walked again, writing all of them (each into its own place,
// so the list's order does not matter)
__global__ void __launch_bounds__(kCandWarps * 32) k_mx_cand_big(ScreenTables T, float cut, int nbig,
                                                                 const int *__restrict__ big,
                                                                 const int *__restrict__ A,
                                                                 const PossPair *__restrict__ P,
                                                                 const int *__restrict__ off, int2 *__restrict__ E) {
    const int b = blockIdx.x * kCandWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (b >= nbig) return;                                        // the whole warp: uniform
    const int p = A[big[b]];
    const PossPair r = P[p];
    const int n = T.ns < T.cn[r.c] ? T.ns : T.cn[r.c];
    int e = off[p];
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int k = k0 + lane;
        const bool hit = k < n && point_cand32(T, r.s, r.c, k, n, cut, r.ubmin);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) E[e + __popc(m & ((1u << lane) - 1u))] = make_int2(p, k);
        e += __popc(m);
    }
}

// ---- K4..K6: FP64 rechecks --------------------------------------------------------------------------------------
__device__ __forceinline__ double point64_at(const ScreenTables &T, int s, int c, int k, double cut, double &sv) {
    const size_t NT = T.nt, NC = T.nc;
    const int n = T.ns < T.cn[c] ? T.ns : T.cn[c];
    const double *tk = T.t64 + (size_t)k * 12 * NT + s, *ck = T.c64 + (size_t)k * 12 * NC + c;
    double M[6], m0[3], m1[3];
#pragma unroll
    for (int i = 0; i < 6; i++) M[i] = tk[(6 + i) * NT] + ck[(6 + i) * NC];
#pragma unroll
    for (int i = 0; i < 3; i++) m0[i] = tk[i * NT] - ck[i * NC];
    const bool more = k + 1 < n;
    if (more) {
#pragma unroll
        for (int i = 0; i < 3; i++) m1[i] = tk[(12 + i) * NT] - ck[(12 + i) * NC];
    } else {
        m1[0] = m0[0]; m1[1] = m0[1]; m1[2] = m0[2];
    }
    return point_chi2_64(M, T.R2[c], m0, m1, more, cut, sv);
}

__global__ void k_mx_eval64(ScreenTables T, double cut, int ne, const PossPair *__restrict__ P,
                            const int2 *__restrict__ E, double *__restrict__ ev, double *__restrict__ es) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int2 pk = E[e];
    const PossPair p = P[pk.x];
    double sv;
    ev[e] = point64_at(T, p.s, p.c, pk.y, cut, sv);
    es[e] = sv;
}

struct PairBest {
    double chi2, sb;
    int kb, pad;
};

// FP64 argmin over a pair's candidates: the smallest value, the first point of equal ones (as the strict < of a
// walk in point order) -- the candidates need not be in point order
__global__ void k_mx_best(int np, const int *__restrict__ off, const int *__restrict__ cnt,
                          const int2 *__restrict__ E, const double *__restrict__ ev, const double *__restrict__ es,
                          PairBest *__restrict__ B) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double best = kInf, sb = 0.0;
    int kb = 0x7fffffff;
    const int e0 = off[p], n = cnt[p];
    for (int q = 0; q < n; q++) {
        const double v = ev[e0 + q];
        const int k = E[e0 + q].y;
        if (v >= 0 && (v < best || (v == best && k < kb))) { best = v; kb = k; sb = es[e0 + q]; }
    }
    PairBest o;
    o.chi2 = best; o.sb = best < kInf ? sb : 0.0; o.kb = best < kInf ? kb : 0; o.pad = 0;
    B[p] = o;
}

__global__ void k_mx_kept_flags(int np, const PairBest *__restrict__ B, double cut, int *__restrict__ f) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) f[p] = B[p].chi2 < cut;
}

__global__ void k_mx_kept_emit(int np, const PossPair *__restrict__ P, const PairBest *__restrict__ B, double cut,
                               const int *__restrict__ off, KeptPair *__restrict__ K) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const PairBest b = B[p];
    if (!(b.chi2 < cut)) return;
    KeptPair k;
    k.s = P[p].s; k.c = P[p].c; k.kb = b.kb; k.pad = 0; k.sb = b.sb; k.chi2 = b.chi2;
    K[off[p]] = k;
}

// entries beyond this are screened by the FP64 selection instead (identical rows; bounds the work buffers)
constexpr long long kMaxEntries = 400000000LL;

// the block filter's launch shapes: resident blocks per SM asked of the compiler (its register cap), in the order
// pgx_screen_shapes lists them; the screen autotuner picks one per context
constexpr int kScanVariants = 4;
constexpr int kScanShapes[kScanVariants] = {6, 5, 7, 8};
int scan_shapes() { return kScanVariants; }
int scan_shape(int v) { return kScanShapes[v % kScanVariants]; }

int mixed_select(cudaStream_t st, const ScreenTables &T, double cut, MixedBufs &m, cudaEvent_t ev_scan, int *total,
                 PgxStats *stats) {
    std::string &err = m.err;
    const int nt = T.nt, nc = T.nc;
    const size_t pairs = (size_t)nt * nc;
    int rc, launches = 0;
    const size_t ng = (size_t)nt * kEmitGroups;         // (star, cluster range) counts
    const int nbs = (int)(ng / kScanBlock) + 2;
    if ((rc = grow(m.flag, pairs, err)) || (rc = grow(m.ub, pairs * 4, err)) || (rc = grow(m.kmin, pairs * 8, err)) ||
        (rc = grow(m.cnt, ng * 4, err)) || (rc = grow(m.off, ng * 4, err)) ||
        (rc = grow(m.total, 64, err)) || (rc = grow(m.aux, (size_t)nbs * 4 + 64, err)))
        return rc;
    int *cnt = Pb<int>(m.cnt), *off = Pb<int>(m.off), *tot = Pb<int>(m.total), *part = Pb<int>(m.aux);
    if ((size_t)(nt + kScanStars - 1) / kScanStars > 65535) {
        err = "mixed precision: too many stars in one call";
        return PGX_E_LIMIT;
    }
    dim3 g(nc, (nt + kScanStars - 1) / kScanStars);
    const float cutf = (float)cut;
    if (T.blk_t && T.blk_c) {
        auto *fl = Pb<unsigned char>(m.flag);
        auto *ub = Pb<float>(m.ub);
        auto *km = Pb<unsigned long long>(m.kmin);
        if (T.blk_cm && T.c32_cm && T.lm_cm) {
            const size_t dyn = (size_t)T.nblk * 64 + (size_t)T.ncp * 48 + (size_t)T.lm_pitch * 4;
            k_mx_scan32_blocks<6, true><<<g, kScanStars, dyn, st>>>(T, cutf, fl, ub, km);
        } else {
            switch (kScanShapes[m.scan_variant % kScanVariants]) {
                case 5: k_mx_scan32_blocks<5, false><<<g, kScanStars, 0, st>>>(T, cutf, fl, ub, km); break;
                case 7: k_mx_scan32_blocks<7, false><<<g, kScanStars, 0, st>>>(T, cutf, fl, ub, km); break;
                case 8: k_mx_scan32_blocks<8, false><<<g, kScanStars, 0, st>>>(T, cutf, fl, ub, km); break;
                default: k_mx_scan32_blocks<6, false><<<g, kScanStars, 0, st>>>(T, cutf, fl, ub, km); break;
            }
        }
    } else
        k_mx_scan32<<<g, kScanStars, 0, st>>>(T, cutf, Pb<unsigned char>(m.flag), Pb<float>(m.ub),
                                              Pb<unsigned long long>(m.kmin));
    if ((rc = check(cudaGetLastError(), err, "k_mx_scan32"))) return rc;
    if ((rc = check(cudaEventRecord(ev_scan, st), err, "event"))) return rc;
    const dim3 ge((nt + 127) / 128, kEmitGroups);
    k_mx_count<<<ge, 128, 0, st>>>(nt, nc, Pb<unsigned char>(m.flag), cnt);
    if ((rc = exclusive_scan(st, (int)ng, cnt, off, part, tot, err))) return rc;
    launches += 2 + 3;
    int np = 0;
    if ((rc = check(cudaMemcpyAsync(&np, tot, 4, cudaMemcpyDeviceToHost, st), err, "counts")) ||
        (rc = check(cudaStreamSynchronize(st), err, "counts sync")))
        return rc;
    // per possible pair p: PossPair P[p], PairBest B[p]; int arrays A (overflowed pairs), pc / po (candidate
    // counts and offsets), flags / offsets (overflowed, then kept), and the scan's block partials
    const int nbp = np / kScanBlock + 2;
    if ((rc = grow(m.cand, (size_t)np * sizeof(PossPair) + 64, err)) ||
        (rc = grow(m.cand_off, ((size_t)np * 3 + nbp) * 4 + 64, err)) ||
        (rc = grow(m.entq, (size_t)np * (sizeof(PairBest) + 8) + 64, err)))
        return rc;
    PossPair *P = Pb<PossPair>(m.cand);
    int *A = Pb<int>(m.cand_off), *pc = A + np, *po = pc + np, *ppart = po + np;
    PairBest *B = Pb<PairBest>(m.entq);
    int *kf = reinterpret_cast<int *>(B + np), *ko = kf + np;
    k_mx_emit<<<ge, 128, 0, st>>>(nt, nc, Pb<unsigned char>(m.flag), Pb<float>(m.ub),
                                  Pb<unsigned long long>(m.kmin), off, P);
    launches += 1;
    int na = 0, ne = 0, nk = 0;
    if (np > 0) {
        // candidate counts: from the slots, or by walking the overflowed pairs again
        k_mx_list_count<<<(np + 255) / 256, 256, 0, st>>>(np, P, pc, kf);
        if ((rc = exclusive_scan(st, np, kf, ko, ppart, tot + 2, err))) return rc;
        k_mx_ovf_emit<<<(np + 255) / 256, 256, 0, st>>>(np, kf, ko, A);
        if ((rc = check(cudaMemcpyAsync(&na, tot + 2, 4, cudaMemcpyDeviceToHost, st), err, "overflowed")) ||
            (rc = check(cudaStreamSynchronize(st), err, "overflowed sync")))
            return rc;
        launches += 2 + 3;
        int *X = nullptr, *big = nullptr, *nbig = tot + 4;
        if (na > 0) {
            if ((rc = grow(m.ovf, (size_t)na * (kCandCap + 1) * 4, err))) return rc;
            X = Pb<int>(m.ovf);
            big = X + (size_t)na * kCandCap;
            if ((rc = check(cudaMemsetAsync(nbig, 0, 4, st), err, "memset"))) return rc;
            k_mx_cand<<<(na + kCandWarps - 1) / kCandWarps, kCandWarps * 32, 0, st>>>(T, cutf, na, A, P, pc, X, big,
                                                                                     nbig);
            launches += 1;
        }
        if ((rc = exclusive_scan(st, np, pc, po, ppart, tot + 1, err))) return rc;
        int counts[4] = {0, 0, 0, 0};                            // entries, -, -, pairs with > kCandCap candidates
        if ((rc = check(cudaMemcpyAsync(counts, tot + 1, 16, cudaMemcpyDeviceToHost, st), err, "entries")) ||
            (rc = check(cudaStreamSynchronize(st), err, "entries sync")))
            return rc;
        ne = counts[0];
        const int n_big = na > 0 ? counts[3] : 0;
        launches += 3;
        if ((long long)ne > kMaxEntries) {
            err = "mixed precision: too many candidate points for the work buffers";
            return PGX_E_LIMIT;
        }
        if ((rc = grow(m.ent, (size_t)ne * (sizeof(int2) + 16) + 64, err))) return rc;
        int2 *E = Pb<int2>(m.ent);
        double *ev = reinterpret_cast<double *>(E + ne), *es = ev + ne;
        k_mx_list_emit<<<(np + 255) / 256, 256, 0, st>>>(np, P, po, E);
        launches += 1;
        if (na > 0) {
            k_mx_cand_copy<<<(unsigned)(((long)na * kCandCap + 255) / 256), 256, 0, st>>>(na, A, pc, po, X, E);
            launches += 1;
            if (n_big > 0) {
                k_mx_cand_big<<<(n_big + kCandWarps - 1) / kCandWarps, kCandWarps * 32, 0, st>>>(T, cutf, n_big, big,
                                                                                                A, P, po, E);
                launches += 1;
            }
        }
        if (ne > 0) {
            k_mx_eval64<<<(ne + 127) / 128, 128, 0, st>>>(T, cut, ne, P, E, ev, es);
            launches += 1;
        }
        k_mx_best<<<(np + 127) / 128, 128, 0, st>>>(np, po, pc, E, ev, es, B);
        k_mx_kept_flags<<<(np + 255) / 256, 256, 0, st>>>(np, B, cut, kf);
        if ((rc = exclusive_scan(st, np, kf, ko, ppart, tot + 3, err))) return rc;
        if ((rc = check(cudaMemcpyAsync(&nk, tot + 3, 4, cudaMemcpyDeviceToHost, st), err, "kept")) ||
            (rc = check(cudaStreamSynchronize(st), err, "kept sync")))
            return rc;
        if ((rc = grow(m.kept, (size_t)nk * sizeof(KeptPair) + 16, err))) return rc;
        if (nk > 0) k_mx_kept_emit<<<(np + 255) / 256, 256, 0, st>>>(np, P, B, cut, ko, Pb<KeptPair>(m.kept));
        if ((rc = check(cudaGetLastError(), err, "k_mx_kept_emit"))) return rc;
        launches += 2 + 3 + (nk > 0);
    } else if ((rc = grow(m.kept, 16, err))) {
        return rc;
    }
    *total = nk;
    if (stats) {
        stats->candidates = np;
        stats->ambiguous = na;
        stats->rechecked_points = ne;
        stats->kernels += launches;
    }
    return 0;
}

const KeptPair *mixed_kept(MixedBufs &m) { return (const KeptPair *)m.kept.p; }

// ---- the 512 draws in FP32 --------------------------------------------------------------------------------------
// Box-Muller with the GPU's fast transcendental units, each with its documented worst-case error, and a bound per
// draw on the distance to the FP64 path's draw (gauss64, draw_xyz64):
//  * u = k 2^-53 from the 53-bit integer k in FP32 within 2^-23 relative (two 32-bit conversions and a fused
//    multiply-add), so |ln U - ln u| <= 1.2e-7;
//  * __logf: absolute error <= 2^-21.41 on [0.5, 2], else 3 ulp, so r^2 = -2 ln u1 is within
//    D = 9.6e-7 + 3.6e-7 r^2;  radius = r^2 rsqrt(r^2) (fast_rsqrt: 2 ulp) within 3e-7 relative of sqrt(r^2), and
//    |sqrt(r^2) - sqrt(r^2_64)| <= min(D / sqrt(r^2), sqrt(D)) <= min(D rsqrt 1.000001, 1e-3 + 6e-4 radius);
//  * cos(2 pi u2) = -cos(theta), theta = (U2 - 1/2) 6.283185f in [-pi, pi] (6.283185f < 2 pi), with U2 from the top
//    32 bits of u2's generator output alone (|U2 - u2| <= 2^-32 + 2^-24 u2 < 2^-23, within the absolute error the
//    bound allows the conversion): the angle, one fused multiply-add, is within 1.19e-6 of 2 pi (u2 - 1/2)
//    (conversion 7.5e-7, the constant 1.6e-7, one rounding 1.9e-7) and __cosf adds <= 2^-21.19 absolute, so the
//    cosine is within 1.61e-6;
//  * z = -radius cos: |z - z_64| <= 1.000003 e_radius + 1.68e-6 radius.
// x = m + L z by three fused multiply-adds from FP32 m and L: every component within
// 4 eps (|m| + |L| max|z|) + |L| max|z - z_64| of the FP64 path's.
__device__ __forceinline__ float u53_unit(uint64_t k) {
    return fmaf((float)(uint32_t)(k >> 21), 0x1p-32f, (float)(uint32_t)(k & 0x1fffffu) * 0x1p-53f);
}

// The bound of one Gaussian, err = 1.000003 e_radius + 1.68e-6 radius with
// e_radius = 3e-7 radius + min(1.000001 D rs, 1e-3 + 6e-4 radius), is evaluated with the factors folded into the
// constants: err = kG1 radius + min(D' rs, kG3 radius + kG4), D' = kG5 r^2 + kG6.  Each folded constant is rounded
// up and carries a further 1 + 1e-6 for the roundings of the fused evaluation (five operations, 2^-24 each).
constexpr float kG1 = (3e-7f * 1.000003f + 1.68e-6f) * 1.000001f, kG3 = 6e-4f * 1.000003f * 1.000001f,
                kG4 = 1e-3f * 1.000003f * 1.000001f, kG5 = 3.6e-7f * 1.000001f * 1.000003f * 1.000001f,
                kG6 = 9.6e-7f * 1.000001f * 1.000003f * 1.000001f;
// angle theta = (U2 - 1/2) 6.283185f as one fused multiply-add on the converted top 32 bits: 6.283185f 2^-32 is
// exact and 3.1415925f is half of 6.283185f, so one rounding replaces the subtraction's and the product's
constexpr float kAngleScale = 6.283185f * 0x1p-32f, kAngleShift = 3.1415925f;

__device__ __forceinline__ void gauss32(uint64_t a, uint64_t b, float &z, float &rad, float &err) {
    const float u1 = fmaxf(u53_unit(a >> 11), 0x1p-64f);       // the reference's floor for u1 = 0
    const float r2 = fmaxf(-2.f * __logf(u1), 0.f);
    const float rs = fast_rsqrt(fmaxf(r2, 1e-30f));
    rad = r2 * rs;
    z = -rad * __cosf(fmaf((float)(uint32_t)(b >> 32), kAngleScale, -kAngleShift));
    err = fmaf(kG1, rad, fminf(fmaf(kG5, r2, kG6) * rs, fmaf(kG3, rad, kG4)));
}

struct Fin32 {
    float mx, my, mz, l00, l10, l20, l11, l21, l22, r50s, rts, e50, etot;
    float eA, eE, eM;          // ex = eA max(radius) + eE max(err) + eM (draw32)
};

// the pair's FP32 constants: lane j converts field j of fin, the warp shares them (one conversion per warp)
__device__ __forceinline__ Fin32 fin32(const FinishIn &fin, int lane) {
    const double *fd = reinterpret_cast<const double *>(&fin);
    double v = fd[lane < 11 ? lane : (lane < 13 ? lane - 2 : 0)];
    if (lane == 11 || lane == 12) v = v * v;                 // r50^2, rtot^2
    const float fv = (float)v;
    Fin32 g;
    g.mx = __shfl_sync(0xffffffffu, fv, 0); g.my = __shfl_sync(0xffffffffu, fv, 1);
    g.mz = __shfl_sync(0xffffffffu, fv, 2);
    g.l00 = __shfl_sync(0xffffffffu, fv, 3); g.l10 = __shfl_sync(0xffffffffu, fv, 4);
    g.l20 = __shfl_sync(0xffffffffu, fv, 5); g.l11 = __shfl_sync(0xffffffffu, fv, 6);
    g.l21 = __shfl_sync(0xffffffffu, fv, 7); g.l22 = __shfl_sync(0xffffffffu, fv, 8);
    g.r50s = __shfl_sync(0xffffffffu, fv, 11); g.rts = __shfl_sync(0xffffffffu, fv, 12);
    const float mabs = fabsf(g.mx) + fabsf(g.my) + fabsf(g.mz);
    const float lsum = fabsf(g.l00) + fabsf(g.l10) + fabsf(g.l20) + fabsf(g.l11) + fabsf(g.l21) + fabsf(g.l22);
    // ex = 4 eps mabs + lsum (4 eps amax + emax (1 + 2 eps)), amax = 1.000001 max(radius) + emax, expanded; the
    // factor 1.000001 on each covers the roundings here and of the two fused multiply-adds in draw32
    g.eA = lsum * (4.f * kEps32 * 1.000001f) * 1.000001f;
    g.eE = lsum * (1.f + 6.f * kEps32) * 1.000001f;
    g.eM = mabs * (4.f * kEps32) * 1.000001f;
    g.e50 = 8.f * kEps32 * g.r50s;                 // rounding of r50^2 and of the comparison
    g.etot = 8.f * kEps32 * g.rts;
    return g;
}

// FP32 draw whose splitmix64 state before its first call is w: position and ex >= |x_j - x_j,64| for each j
__device__ __forceinline__ void draw32(const Fin32 &g, uint64_t w, float &x, float &y, float &z, float &ex) {
    float z0, z1, z2, a0, a1, a2, e0, e1, e2;
    gauss32(splitmix_mix(w + kGolden), splitmix_mix(w + 2 * kGolden), z0, a0, e0);
    gauss32(splitmix_mix(w + 3 * kGolden), splitmix_mix(w + 4 * kGolden), z1, a1, e1);
    gauss32(splitmix_mix(w + 5 * kGolden), splitmix_mix(w + 6 * kGolden), z2, a2, e2);
    x = fmaf(g.l00, z0, g.mx);
    y = fmaf(g.l11, z1, fmaf(g.l10, z0, g.my));
    z = fmaf(g.l22, z2, fmaf(g.l21, z1, fmaf(g.l20, z0, g.mz)));
    ex = fmaf(g.eA, fmaxf(a0, fmaxf(a1, a2)), fmaf(g.eE, fmaxf(e0, fmaxf(e1, e2)), g.eM));
}

// The 512 draws of a kept pair, in two phases.  A draw's first coordinate x = mx + l00 z0 depends on its first
// Gaussian alone, and |x| >= max(r50, rtot) puts the draw outside both spheres whatever z1 and z2 are (r >= |x|, in
// the FP64 path's arithmetic as well).  Phase 1 draws z0 for all 512 and settles the draws whose x, less its error
// bound (4 eps |mx| + |l00| (4 eps |z0| + e0 (1 + 2 eps)), the x row of draw32's bound), clears the larger radius;
// with sigma of hundreds of pc against radii of tens, most do.  The rest are queued per warp in shared memory with
// z0 and its bound, and phase 2 completes them 32 at a time on full warps: z1, z2, the position and its bound as
// draw32 computes them, and the FP64 recheck of a draw within its bound of a radius -- the counts are the FP64
// path's, and the same as drawing every draw in full.
constexpr int kFinWarps = 8, kFinQueue = 64;

__global__ void __launch_bounds__(kFinWarps * 32) k_mx_finish32(int n, const FinishIn *__restrict__ fin,
                                                                ScreenRowDev *__restrict__ rows,
                                                                int *__restrict__ nrecheck) {
    __shared__ int s_i[kFinWarps][kFinQueue];
    __shared__ float s_z[kFinWarps][kFinQueue], s_a[kFinWarps][kFinQueue], s_e[kFinWarps][kFinQueue];
    const int h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    if (h >= n) return;                                           // the whole warp: uniform
    const Fin32 g = fin32(fin[h], lane);
    const uint64_t seed = fin[h].seed;
    // the x row of the bound, and the larger radius with a margin for its rounding to FP32
    const float eA0 = fabsf(g.l00) * (4.f * kEps32 * 1.000001f) * 1.000001f;
    const float eE0 = fabsf(g.l00) * (1.f + 6.f * kEps32) * 1.000001f;
    const float eM0 = fabsf(g.mx) * (4.f * kEps32) * 1.000001f;
    const float rout = sqrtf(fmaxf(g.r50s, g.rts)) * (1.f + 1e-6f);
    int in50 = 0, intot = 0, rechecks = 0;
    // phase 2 for queue entries [0, cnt), one per lane
    auto complete = [&](int cnt) {
        __syncwarp();
        if (lane < cnt) {
            const int i = s_i[wq][lane];
            const float z0 = s_z[wq][lane], a0 = s_a[wq][lane], e0 = s_e[wq][lane];
            const uint64_t w = seed + (uint64_t)(6 * i) * kGolden;
            float z1, z2, a1, a2, e1, e2;
            gauss32(splitmix_mix(w + 3 * kGolden), splitmix_mix(w + 4 * kGolden), z1, a1, e1);
            gauss32(splitmix_mix(w + 5 * kGolden), splitmix_mix(w + 6 * kGolden), z2, a2, e2);
            const float x = fmaf(g.l00, z0, g.mx);
            const float y = fmaf(g.l11, z1, fmaf(g.l10, z0, g.my));
            const float z = fmaf(g.l22, z2, fmaf(g.l21, z1, fmaf(g.l20, z0, g.mz)));
            const float ex = fmaf(g.eA, fmaxf(a0, fmaxf(a1, a2)), fmaf(g.eE, fmaxf(e0, fmaxf(e1, e2)), g.eM));
            const float r2 = fmaf(x, x, fmaf(y, y, z * z));
            const float x1 = fabsf(x) + fabsf(y) + fabsf(z);
            const float er = 3.f * kEps32 * r2 + 2.f * x1 * ex + 3.f * ex * ex;
            const float d50 = r2 - g.r50s, dt = r2 - g.rts;
            if (fabsf(d50) > er + g.e50 && fabsf(dt) > er + g.etot) {
                in50 += d50 < 0.f;
                intot += dt < 0.f;
            } else {
                const int v = draw_inside64(fin[h], i);             // the FP64 path's own draw
                in50 += v & 1;
                intot += v >> 1;
                rechecks++;
            }
        }
        __syncwarp();
    };
    // draw i uses calls 6i+1 .. 6i+6 of the pair's splitmix64 stream, whose state is seed + call * golden
    uint64_t w = seed + (uint64_t)(6 * lane) * kGolden;
    int qn = 0;
#pragma unroll 1
    for (int q = 0; q < 16; q++, w += 192 * kGolden) {
        float z0, a0, e0;
        gauss32(splitmix_mix(w + kGolden), splitmix_mix(w + 2 * kGolden), z0, a0, e0);
        const float x = fmaf(g.l00, z0, g.mx);
        const float ex0 = fmaf(eA0, a0, fmaf(eE0, e0, eM0));
        const bool open = !(fabsf(x) * (1.f - 4.f * kEps32) - ex0 >= rout);
        const unsigned m = __ballot_sync(0xffffffffu, open);
        if (open) {
            const int at = qn + __popc(m & ((1u << lane) - 1u));
            s_i[wq][at] = lane + 32 * q;
            s_z[wq][at] = z0;
            s_a[wq][at] = a0;
            s_e[wq][at] = e0;
        }
        qn += __popc(m);
        if (qn >= 32) {
            complete(32);
            const int rest = qn - 32;
            int vi = 0;
            float vz = 0.f, va = 0.f, ve = 0.f;
            if (lane < rest) {
                vi = s_i[wq][32 + lane]; vz = s_z[wq][32 + lane]; va = s_a[wq][32 + lane]; ve = s_e[wq][32 + lane];
            }
            __syncwarp();
            if (lane < rest) {
                s_i[wq][lane] = vi; s_z[wq][lane] = vz; s_a[wq][lane] = va; s_e[wq][lane] = ve;
            }
            qn = rest;
        }
    }
    if (qn > 0) complete(qn);
    in50 = __reduce_add_sync(0xffffffffu, in50);
    intot = __reduce_add_sync(0xffffffffu, intot);
    rechecks = __reduce_add_sync(0xffffffffu, rechecks);
    if (lane == 0) {
        rows[h].p_r50 = (double)in50 / 512.0;
        rows[h].p_rtot = (double)intot / 512.0;
        if (rechecks) atomicAdd(nrecheck, rechecks);
    }
}

// Self-check of the FP32 draws: per pair (one warp), the largest |x_j - x_j,64| / ex over its 512 draws and three
// components -- at most 1 when the per-draw bound holds.
__global__ void __launch_bounds__(256) k_mx_check_draws(int n, const FinishIn *__restrict__ fin,
                                                        double *__restrict__ ratio) {
    const int h = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (h >= n) return;
    const FinishIn f = fin[h];
    const Fin32 g = fin32(f, lane);
    double worst = 0.0;
    uint64_t w = f.seed + (uint64_t)(6 * lane) * kGolden;
    for (int q = 0; q < 16; q++, w += 192 * kGolden) {
        float x, y, z, ex;
        draw32(g, w, x, y, z, ex);
        double x64, y64, z64;
        draw_xyz64(f, lane + 32 * q, x64, y64, z64);
        const double d = fmax(fabs((double)x - x64), fmax(fabs((double)y - y64), fabs((double)z - z64)));
        worst = fmax(worst, d / (double)ex);
    }
    for (int o = 16; o > 0; o >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    if (lane == 0) ratio[h] = worst;
}

int mixed_check_draws(cudaStream_t st, int n, const FinishIn *fin, double *ratio, std::string &err) {
    k_mx_check_draws<<<(unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, st>>>(n, fin, ratio);
    return check(cudaGetLastError(), err, "k_mx_check_draws");
}

int mixed_finish(cudaStream_t st, int n, const FinishIn *fin, ScreenRowDev *rows, MixedBufs &m, PgxStats *stats) {
    int rc;
    if ((rc = grow(m.total, 64, m.err))) return rc;
    int *cnt = Pb<int>(m.total) + 8;
    if ((rc = check(cudaMemsetAsync(cnt, 0, 4, st), m.err, "memset"))) return rc;
    k_mx_finish32<<<(unsigned)(((size_t)n + kFinWarps - 1) / kFinWarps), kFinWarps * 32, 0, st>>>(n, fin, rows, cnt);
    if (stats) stats->kernels += 0;     // counted with the finish prep by the caller
    if ((rc = check(cudaGetLastError(), m.err, "k_mx_finish32"))) return rc;
    int h = 0;
    if ((rc = check(cudaMemcpyAsync(&h, cnt, 4, cudaMemcpyDeviceToHost, st), m.err, "rechecks"))) return rc;
    if ((rc = check(cudaStreamSynchronize(st), m.err, "finish sync"))) return rc;
    if (stats) stats->rechecked_draws = h;
    return 0;
}

}  // namespace pgx

namespace pgx {
// Self-check of point_bound32: n independent points given in FP64 (star and cluster positions at the point and at
// the next one, the two covariances, R^2), evaluated as the screen evaluates them -- the FP32 bounds from split
// positions and FP32 covariances, and the FP64 point chi2.  rej[i] = 1 when FP32 rejects the point by the trace
// bound, 2 when the cheap test (point_skip32) skips it (its bounds are returned all the same), else 0.
__global__ void k_mx_check_bounds(int n, const double *__restrict__ pos, const double *__restrict__ S,
                                  const double *__restrict__ R2, double cut, double *__restrict__ v64,
                                  float *__restrict__ lb, float *__restrict__ ub, int *__restrict__ rej) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *p = pos + (size_t)i * 12;          // t0 c0 t1 c1, 3 each
    const double *s = S + (size_t)i * 12;            // S_t, S_c
    float4 q[4][2];
    for (int a = 0; a < 4; a++) {
        const float hx = (float)p[3 * a], hy = (float)p[3 * a + 1], hz = (float)p[3 * a + 2];
        q[a][0] = make_float4(hx, hy, hz, (float)(p[3 * a] - (double)hx));
        q[a][1] = make_float4((float)(p[3 * a + 1] - (double)hy), (float)(p[3 * a + 2] - (double)hz), 0.f, 0.f);
    }
    float m0[3], m1[3], St[6], Sc[6];
    sep32(q[0][0], q[0][1], q[1][0], q[1][1], m0);
    sep32(q[2][0], q[2][1], q[3][0], q[3][1], m1);
    // the cluster side as the table holds it: S_c + R^2 I rounded once, lmin(S_c) + R^2 rounded down
    for (int j = 0; j < 6; j++) {
        St[j] = (float)s[j];
        Sc[j] = (float)(j == 0 || j == 3 || j == 5 ? s[6 + j] + R2[i] : s[6 + j]);
    }
    const double lt = sym3_min_eig_lb(s[0], s[1], s[2], s[3], s[4], s[5]);
    const double lc = sym3_min_eig_lb(s[6], s[7], s[8], s[9], s[10], s[11]);
    const float lmt = __double2float_rd(lt - 1e-12 * fabs(lt));
    const float lmc = __double2float_rd((double)__double2float_rd(lc - 1e-12 * fabs(lc)) + R2[i]);
    Bound b;
    const bool dec = point_bound32(St, Sc, lmt, lmc, m0, m1, true, (float)cut, b);
    double M[6], d0[3], d1[3], sv;
    for (int j = 0; j < 6; j++) M[j] = s[j] + s[6 + j];
    for (int j = 0; j < 3; j++) { d0[j] = p[j] - p[3 + j]; d1[j] = p[6 + j] - p[9 + j]; }
    v64[i] = point_chi2_64(M, R2[i], d0, d1, true, cut, sv);
    lb[i] = dec ? b.lb : 0.f;
    ub[i] = dec ? b.ub : 0.f;
    rej[i] = !dec ? 1 : (point_skip32(St, Sc, lmt, lmc, m0, m1, (float)cut) ? 2 : 0);
}

int mixed_check_bounds(cudaStream_t st, int n, const double *pos, const double *S, const double *R2, double cut,
                       double *v64, float *lb, float *ub, int *rej, std::string &err) {
    k_mx_check_bounds<<<(n + 127) / 128, 128, 0, st>>>(n, pos, S, R2, cut, v64, lb, ub, rej);
    return check(cudaGetLastError(), err, "k_mx_check_bounds");
}

// Self-check of the block test on a staged chunk: every (pair, testable block) gets block_skip32 as the filter runs
// it, and every point of a block it settles gets the FP64 path's point chi2 (pgx_screen_math.cuh): a point under the
// cut there is a violation.  cnt: blocks tested, blocks settled, points of settled blocks, violations.
// The block test against the FP64 path, per (pair, block): counts of blocks tested and settled, the points of the
// settled blocks and those under the cut (violations, 0 when the bound holds); the blocks whose points are all at or
// above the cut (what an exact block test would settle) and the blocks of pairs with a point under the cut; and over
// the points of the blocks the test leaves, those the point test settles, those at or above the cut (what an exact
// point test would settle), and the point test's violations (also of the point test against the block's dominating
// matrix, whose settled points and those the point test leaves follow).
__global__ void k_mx_check_blocks(ScreenTables T, double cut, unsigned long long *__restrict__ cnt) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t NT = T.nt, NC = T.nc;
    if (p >= NT * NC) return;
    const int s = (int)(p % NT), c = (int)(p / NT);
    const int n = T.ns < T.cn[c] ? T.ns : T.cn[c];
    const int nbt = n > kBlk / 2 ? (n - kBlk / 2 - 1) / kBlk + 1 : 0;
    unsigned long long k_[kCheckBlockCounts] = {};
    const double R2 = T.R2[c];
    bool kept = false;
    unsigned long long nb_pair = 0;
    for (int b = 0; b < nbt; b++) {
        const int km = b * kBlk + kBlk / 2;
        const float4 *a = T.blk_t + ((size_t)b * NT + s) * 4, *q = T.blk_c + ((size_t)b * NC + c) * 4;
        const float4 BT[4] = {a[0], a[1], a[2], a[3]};
        const float4 BC[4] = {q[0], q[1], q[2], q[3]};
        const float4 *tm = T.t32 + ((size_t)km * NT + s) * 3, *cm = T.c32 + ((size_t)km * NC + c) * 3;
        float mref[3];
        sep32(tm[0], tm[1], cm[0], cm[1], mref);
        k_[0]++;
        nb_pair++;
        const bool settled = block_skip32(BT, BC, mref, (float)cut);
        k_[1] += settled;
        bool all_above = true;
        for (int k = b * kBlk; k < min(b * kBlk + kBlk, n); k++) {
            const double *tk = T.t64 + (size_t)k * 12 * NT + s, *ck = T.c64 + (size_t)k * 12 * NC + c;
            double M[6], m0[3], m1[3], sv;
            for (int i = 0; i < 6; i++) M[i] = tk[(6 + i) * NT] + ck[(6 + i) * NC];
            for (int i = 0; i < 3; i++) m0[i] = tk[i * NT] - ck[i * NC];
            const bool more = k + 1 < n;
            for (int i = 0; i < 3; i++) m1[i] = more ? tk[(12 + i) * NT] - ck[(12 + i) * NC] : m0[i];
            const double v = point_chi2_64(M, R2, m0, m1, more, cut, sv);
            const bool under = v >= 0 && v < cut;
            all_above &= !under;
            kept |= under;
            if (settled) {
                k_[2]++;
                k_[3] += under;
            } else {
                const float4 *t = T.t32 + ((size_t)k * NT + s) * 3, *cc = T.c32 + ((size_t)k * NC + c) * 3;
                float mc[3], mn[3];
                sep32(t[0], t[1], cc[0], cc[1], mc);
                if (more) {
                    const float4 *t2 = t + NT * 3, *c2 = cc + NC * 3;
                    sep32(t2[0], t2[1], c2[0], c2[1], mn);
                } else {
                    mn[0] = mc[0]; mn[1] = mc[1]; mn[2] = mc[2];
                }
                const float St[6] = {t[1].z, t[1].w, t[2].x, t[2].y, t[2].z, t[2].w};
                const float Sc[6] = {cc[1].z, cc[1].w, cc[2].x, cc[2].y, cc[2].z, cc[2].w};
                const bool pskip = point_skip32(St, Sc, T.lm_t[(size_t)k * NT + s], T.lm_c[(size_t)k * NC + c], mc,
                                                mn, (float)cut);
                const bool nskip = point_skip32_blk(BT, BC, mc, mn, (float)cut);
                k_[6]++;
                k_[7] += pskip;
                k_[8] += !under;
                k_[9] += (pskip || nskip) && under;
                k_[10] += nskip;
                k_[11] += nskip && !pskip;
            }
        }
        k_[4] += all_above;
    }
    if (kept) k_[5] += nb_pair;
    for (int i = 0; i < kCheckBlockCounts; i++)
        if (k_[i]) atomicAdd(cnt + i, k_[i]);
}

int mixed_check_blocks(cudaStream_t st, const ScreenTables &T, double cut, unsigned long long *cnt,
                       std::string &err) {
    if (!T.blk_t || !T.blk_c) {
        err = "no block tables";
        return PGX_E_ARG;
    }
    int rc = check(cudaMemsetAsync(cnt, 0, kCheckBlockCounts * sizeof(unsigned long long), st), err, "memset");
    if (rc) return rc;
    const size_t pairs = (size_t)T.nt * T.nc;
    k_mx_check_blocks<<<(unsigned)((pairs + 127) / 128), 128, 0, st>>>(T, cut, cnt);
    return check(cudaGetLastError(), err, "k_mx_check_blocks");
}
}  // namespace pgx
