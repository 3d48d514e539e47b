// pgx_draws.cu -- the draws from the measurement errors on the GPU (the survey's "device-side draws"): the
// astrometric draws of ph_sample_target / ph_sample_cluster with their radial-velocity priors, the nominal state and
// 6-D covariance of a star's draws (ph_lin_target_init), and the clone start states of ph_pair_draw
// (reference src/phygas.c:21-82, 182-198, 256-284; coordinates src/coords.c:77-131; splitmix64 and Box-Muller
// src/montecarlo.h:26-41, src/montecarlo.c:4-17).
//
// The host versions (csrc/host/ph_host.c) are the reference's draws bit for bit and stay the default.  These run the
// same operations in the same order (this file is built without FP contraction), with the device's log, exp, cos,
// sin, sqrt and pow in place of the C library's: the results differ from the host's in the last bits where those
// functions do, and the screen and pair results made from them agree with the host-draw results within the hot
// path's tolerances.  The random streams are the host's: the same seeds, the same number of generator calls per draw
// (retries of non-physical draws included), so the same draws are taken.
//   k_draw_targets   one thread per object: its nominal state and its n_samp draws in turn (the stream is
//                    sequential: a retried draw shifts every later one), the covariance summed in the host's order
//   k_draw_pairs     one thread per pair: its clones in turn, target then cluster per clone, into the pair's slot
//   k_compact_pairs  the pairs' successful clones back to back (a warp per pair)
#include <cstdint>
#include "pgx_internal.cuh"
#include "pgx_mixed.h"

namespace pgx {
namespace {

constexpr double kKmsKpcMyr = 977.7922216807892;
constexpr double kGrav = 4.30091e-6 / (kKmsKpcMyr * kKmsKpcMyr);
constexpr double kMgalMsun = 2.325e7;
constexpr double kPi = 3.14159265358979323846;
constexpr double kRad = kPi / 180.0;
constexpr double kAuYr = 1.495978707e8 / 3.15576e7;
// the Milky Way model and the Sun (reference src/potential.c, src/coords.h:51), as the host file states them
constexpr double kBulgeGM = kGrav * (606.0 * kMgalMsun), kBulgeB = 0.3873;
constexpr double kDiskGM = kGrav * (3690.0 * kMgalMsun), kDiskA = 5.3178, kDiskB = 0.2500;
constexpr double kHaloGM = kGrav * (4615.0 * kMgalMsun), kHaloA = 12.0, kHaloCut = 100.0, kHaloGamma = 2.02;
constexpr double kR0 = 8.122, kZ0 = 0.0208, kVc = 229.0, kUpec = 11.1, kVpec = 12.24, kWpec = 7.25;
__constant__ double kIcrsToGal[3][3] = {
    {-0.0548755604162154, -0.8734370902348850, -0.4838350155487132},
    {0.4941094278755837, -0.4448296299600112, 0.7469822444972189},
    {-0.8676661490190047, -0.1980763734312015, 0.4559837761750669},
};

struct D3 { double x, y, z; };
__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 add(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 sub(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 mul(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct Rng {                     // splitmix64: state advanced by the golden ratio, one output per call
    uint64_t state;
    __device__ uint64_t next() { return splitmix_mix(state += kGolden); }
    __device__ double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    __device__ double gauss() {  // Box-Muller, the second value discarded
        double u1 = uniform();
        if (u1 <= 0.0) u1 = 1.0 / 18446744073709551616.0;
        const double u2 = uniform();
        return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
    }
};
__device__ __forceinline__ double g_or_zero(Rng *g) { return g ? g->gauss() : 0.0; }

__device__ D3 icrs_to_gal(D3 v) {
    return d3(kIcrsToGal[0][0] * v.x + kIcrsToGal[0][1] * v.y + kIcrsToGal[0][2] * v.z,
              kIcrsToGal[1][0] * v.x + kIcrsToGal[1][1] * v.y + kIcrsToGal[1][2] * v.z,
              kIcrsToGal[2][0] * v.x + kIcrsToGal[2][1] * v.y + kIcrsToGal[2][2] * v.z);
}
__device__ D3 sun_pos() { return d3(0.0 - kR0, 0.0, 0.0 + kZ0); }
__device__ D3 sun_vel() {
    return d3(0.0 + kUpec / kKmsKpcMyr, 0.0 + (kVc + kVpec) / kKmsKpcMyr, 0.0 + kWpec / kKmsKpcMyr);
}

// the force in the reference's form (the host's host_accel), for the circular-velocity RV prior
__device__ D3 accel_ref(D3 q) {
    const double R2 = q.x * q.x + q.y * q.y, R = sqrt(R2), r = sqrt(dot(q, q));
    D3 a = d3(0, 0, 0);
    const double pl = pow(r * r + kBulgeB * kBulgeB, 1.5);
    a = add(a, mul(q, -kBulgeGM / (pl > 0 ? pl : 1e-12)));
    const double zeta = sqrt(q.z * q.z + kDiskB * kDiskB), s = kDiskA + zeta;
    const double Dd2 = R2 + s * s, Dd = sqrt(Dd2), Dd3 = Dd2 * Dd;
    const double fR = -kDiskGM * R / Dd3;
    const double fz = -kDiskGM * q.z * s / (zeta > 0 ? zeta : 1e-12) / Dd3;
    if (R > 1e-12) { a.x += fR * q.x / R; a.y += fR * q.y / R; }
    a.z += fz;
    const double rr = r > 1e-12 ? r : 1e-12;
    const double r_in = rr < kHaloCut ? rr : kHaloCut, x = r_in / kHaloA;
    const double enc = kHaloGM * pow(x, kHaloGamma) / (1.0 + pow(x, kHaloGamma - 1.0));
    return add(a, mul(q, -enc / (rr * rr * rr)));
}

struct Astro { double ra, dec, plx, pmra, pmdec, rv; };

__device__ void galcen(const Astro &a, D3 &pos, D3 &vel) {
    const double ra = a.ra * kRad, dec = a.dec * kRad;
    const double d_kpc = 1.0 / a.plx, d_pc = d_kpc * 1000.0;
    const D3 e_r = d3(cos(dec) * cos(ra), cos(dec) * sin(ra), sin(dec));
    const D3 e_a = d3(-sin(ra), cos(ra), 0.0);
    const D3 e_d = d3(-sin(dec) * cos(ra), -sin(dec) * sin(ra), cos(dec));
    const D3 g = icrs_to_gal(mul(e_r, d_kpc));
    pos = d3(g.x - kR0, g.y, g.z + kZ0);
    const double va = kAuYr * 1e-3 * a.pmra * d_pc, vd = kAuYr * 1e-3 * a.pmdec * d_pc;
    const D3 v = add(add(mul(e_r, a.rv), mul(e_a, va)), mul(e_d, vd));
    const D3 gv = icrs_to_gal(d3(v.x / kKmsKpcMyr, v.y / kKmsKpcMyr, v.z / kKmsKpcMyr));
    vel = add(gv, d3(kUpec / kKmsKpcMyr, (kVc + kVpec) / kKmsKpcMyr, kWpec / kKmsKpcMyr));
}

__device__ double rv_rotation(D3 q) {
    const double R = hypot(q.x, q.y);
    if (R <= 0) return 0.0;
    const D3 a = accel_ref(d3(q.x, q.y, 0.0));
    const double ar = -(a.x * q.x + a.y * q.y) / R;
    const double vc = ar > 0 ? sqrt(R * ar) : 0.0;
    const D3 v = d3(vc * q.y / R, -vc * q.x / R, 0.0);
    const D3 los = sub(q, sun_pos());
    const double n = sqrt(dot(los, los));
    if (n <= 0) return 0.0;
    return dot(sub(v, sun_vel()), mul(los, 1.0 / n)) * kKmsKpcMyr;
}

__device__ void close_draw(Astro a, int has_rv, double rv, double e_rv, double prior, Rng *g, double *out) {
    D3 p, v;
    if (has_rv) {
        a.rv = rv + e_rv * g_or_zero(g);
    } else {
        a.rv = 0.0;
        galcen(a, p, v);
        a.rv = rv_rotation(p) + prior * g_or_zero(g);
    }
    galcen(a, p, v);
    out[0] = p.x; out[1] = p.y; out[2] = p.z; out[3] = v.x; out[4] = v.y; out[5] = v.z;
}

__device__ int sample_target(const PhTarget &t, Rng *g, double *out) {
    Astro a;
    a.ra = t.ra; a.dec = t.dec;
    for (int tries = 0; tries < 50; tries++) {
        const double plx = t.plx > 0 ? t.plx + t.e_plx * g_or_zero(g)
                                     : 1000.0 / (t.dist_pc * exp(t.e_lndist * g_or_zero(g)));
        if (!(plx > 0)) continue;
        a.plx = plx;
        a.pmra = t.pmra + t.e_pmra * g_or_zero(g);
        a.pmdec = t.pmdec + t.e_pmdec * g_or_zero(g);
        close_draw(a, t.has_rv, t.rv, t.e_rv, t.kind == 'P' ? PH_PULSAR_RV_PRIOR : PH_STAR_RV_PRIOR, g, out);
        return 0;
    }
    return -1;
}

__device__ int sample_cluster(const PhCluster &c, Rng *g, double *out) {
    Astro a;
    a.ra = c.ra; a.dec = c.dec;
    for (int tries = 0; tries < 50; tries++) {
        const double d = c.dist_pc + c.e_dist_pc * g_or_zero(g);
        if (!(d > 0)) continue;
        a.plx = 1000.0 / d;
        a.pmra = c.pmra + c.e_pmra * g_or_zero(g);
        a.pmdec = c.pmdec + c.e_pmdec * g_or_zero(g);
        close_draw(a, c.has_rv, c.rv, c.e_rv, PH_CLUSTER_RV_PRIOR, g, out);
        return 0;
    }
    return -1;
}

__device__ __forceinline__ int sample(const PhTarget &t, Rng *g, double *out) { return sample_target(t, g, out); }
__device__ __forceinline__ int sample(const PhCluster &c, Rng *g, double *out) { return sample_cluster(c, g, out); }

// nominal state and covariance of an object's draws: the covariance summed over the successful draws in draw order,
// entry by entry, then divided by their number (the host's nominal_and_cov)
template <class Obj>
__device__ void object_init(const Obj &o, int n_samp, uint64_t seed, double *ps0, double *sig) {
    double nom[6], d[6], S[36];
    sample(o, nullptr, nom);
    for (int q = 0; q < 36; q++) S[q] = 0.0;
    Rng g{seed};
    int k = 0;
    for (int i = 0; i < n_samp; i++) {
        if (sample(o, &g, d)) continue;
        const double e[6] = {d[0] - nom[0], d[1] - nom[1], d[2] - nom[2], d[3] - nom[3], d[4] - nom[4], d[5] - nom[5]};
        for (int a = 0; a < 6; a++)
            for (int b = 0; b < 6; b++) S[6 * a + b] += e[a] * e[b];
        k++;
    }
    for (int q = 0; q < 36; q++) sig[q] = S[q] / (k > 0 ? k : 1);
    for (int q = 0; q < 6; q++) ps0[q] = nom[q];
}

__global__ void k_draw_targets(int n, const PhTarget *__restrict__ t, int n_samp, const uint64_t *__restrict__ seed,
                               double *__restrict__ ps0, double *__restrict__ sig) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) object_init(t[i], n_samp, seed[i], ps0 + 6 * (size_t)i, sig + 36 * (size_t)i);
}

__global__ void k_draw_clusters(int n, const PhCluster *__restrict__ c, int n_samp, const uint64_t *__restrict__ seed,
                                double *__restrict__ ps0, double *__restrict__ sig) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        object_init(c[i], n_samp, seed[i], ps0 + 6 * (size_t)i, sig + 36 * (size_t)i);
}

// ph_pair_draw for pair q: its clones at slot[q] (room for n_clones[q]), the successful ones back to back; m[q]
__global__ void k_draw_pairs(int n_pairs, const PhTarget *__restrict__ t, const int *__restrict__ ti,
                             const PhCluster *__restrict__ c, const int *__restrict__ ci,
                             const int *__restrict__ n_clones, const uint64_t *__restrict__ seed,
                             const long long *__restrict__ slot, double *__restrict__ ps, int *__restrict__ m) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const PhTarget tq = t[ti[q]];
    const PhCluster cq = c[ci[q]];
    Rng g{seed[q]};
    double *o = ps + 12 * slot[q];
    int k = 0;
    for (int j = 0; j < n_clones[q]; j++) {
        if (sample_target(tq, &g, o + 12 * (size_t)k) || sample_cluster(cq, &g, o + 12 * (size_t)k + 6)) continue;
        k++;
    }
    m[q] = k;
}

// the successful clones of pair q (m[q] of them at slot[q]) moved to off[q], one warp per pair
__global__ void k_compact_pairs(int n_pairs, const long long *__restrict__ slot, const int *__restrict__ off,
                                const int *__restrict__ m, const double *__restrict__ src, double *__restrict__ dst) {
    const int q = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (q >= n_pairs) return;
    const double *a = src + 12 * slot[q];
    double *b = dst + 12 * (size_t)off[q];
    for (int i = lane; i < 12 * m[q]; i += 32) b[i] = a[i];
}

}  // namespace

int compact_pairs_gpu(cudaStream_t st, int n_pairs, const long long *slot, const int *off, const int *m,
                      const double *src, double *dst, std::string &err) {
    k_compact_pairs<<<(unsigned)(((size_t)n_pairs * 32 + 255) / 256), 256, 0, st>>>(n_pairs, slot, off, m, src, dst);
    return check(cudaGetLastError(), err, "k_compact_pairs");
}

int draw_targets_gpu(cudaStream_t st, int n, const PhTarget *t, int n_samp, const uint64_t *seed, double *ps0,
                     double *sig, std::string &err) {
    k_draw_targets<<<(n + 63) / 64, 64, 0, st>>>(n, t, n_samp, seed, ps0, sig);
    return check(cudaGetLastError(), err, "k_draw_targets");
}

int draw_clusters_gpu(cudaStream_t st, int n, const PhCluster *c, int n_samp, const uint64_t *seed, double *ps0,
                      double *sig, std::string &err) {
    k_draw_clusters<<<(n + 63) / 64, 64, 0, st>>>(n, c, n_samp, seed, ps0, sig);
    return check(cudaGetLastError(), err, "k_draw_clusters");
}

int draw_pairs_gpu(cudaStream_t st, int n_pairs, const PhTarget *t, const int *ti, const PhCluster *c,
                   const int *ci, const int *n_clones, const uint64_t *seed, const long long *slot, double *ps,
                   int *m, std::string &err) {
    k_draw_pairs<<<(n_pairs + 63) / 64, 64, 0, st>>>(n_pairs, t, ti, c, ci, n_clones, seed, slot, ps, m);
    return check(cudaGetLastError(), err, "k_draw_pairs");
}

}  // namespace pgx
